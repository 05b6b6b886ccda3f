// Newton-matrix factorisation and solves for a linearly implicit integrator
// step on the Jacobians of this library: M_i = I - s h_i J_i per state, LU
// with partial pivoting (the unblocked right-looking LU of LAPACK's dgetf2:
// pivot = first row of largest |a| in the column, whole-row interchange,
// column scaled by the reciprocal of the pivot when |pivot| >= DBL_MIN, else
// divided, then the rank-1 update a_rc -= l_r u_c as one FMA), and the
// forward/back substitution of dgetrs.  No reference counterpart: the
// reference lists coupling to Rosenbrock solvers as future work; this is the
// consumer of its Jacobian output.
//
// Layouts are the dense Jacobian's: order 'C' M[i][r][c] at i*nn*nn + r*nn + c,
// order 'F' at i + n*(r + nn*c); vectors as phi (C: i*nn + r, F: i + n*r);
// pivots as vectors of int32 (1-based, LAPACK's ipiv).
//
// FP64 on GB300 issues one warp instruction per 16 clocks per SM whatever the
// number of active lanes, so the factorisations keep the lanes full: each
// block holds up to four states' matrices in shared memory and spreads their
// trailing updates over all its threads.  The solves, which read each factor
// entry once, are one thread per state and bound by memory.
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>
#include <vector>

#include "../../include/pyjac_gb300.h"

int pjg_internal_fail(int code, const char* msg);
void pjg_internal_count_launch();

namespace {

constexpr int kLuMaxNN = 169;          // 169 * 169 * 8 bytes fits the 227 KB of one block
constexpr int kSolveNMax = 176;        // local vector of the solve kernel

__device__ __forceinline__ size_t mat_idx(bool F, long long i, long long n, int nn, int r, int c)
{
    return F ? (size_t)(i + n * ((long long)r + (long long)nn * c))
             : (size_t)(i * (long long)nn * nn + (long long)r * nn + c);
}
__device__ __forceinline__ size_t vec_idx(bool F, long long i, long long n, int nn, int r)
{
    return F ? (size_t)(i + n * r) : (size_t)(i * (long long)nn + r);
}

// Flattened (row, column) cursor over an m-column block, advanced by a fixed
// stride T = q m + rem (q = T / m, rem = T % m): at most one wrap per step.
struct Cursor {
    int r, c, q, rem, m;
    __device__ __forceinline__ Cursor(int start, int stride, int m_) : m(m_)
    {
        r = start / m;
        c = start - r * m;
        q = stride / m;
        rem = stride - q * m;
    }
    __device__ __forceinline__ void next()
    {
        c += rem;
        r += q;
        if (c >= m) {
            c -= m;
            ++r;
        }
    }
};

// One thread's share of loading a state's Newton matrix into shared memory:
// a[r][c] = fma(-g, J[p(r)][p(c)], delta_rc) for the elements start,
// start + stride, ... (p the permutation, or the identity when perm is null),
// B global loads in flight before their shared-memory stores (4 helps the
// permuted gathers of the sparse kernel: 97.8 -> 91.6 ms per 1M GRI states;
// the pivoting kernel is faster with 1: 149.6 against 153.6 ms).
template <bool F, int B>
__device__ __forceinline__ void load_newton(double* a, int pitch, int nn, const double* jac,
                                            long long i, long long n, double g, bool live, int start,
                                            int stride, const int* perm)
{
    const int nsq = nn * nn;
    Cursor cu(start, stride, nn);
    for (int e = start; e < nsq; e += B * stride) {
        double j[B];
        int o[B];
        bool ok[B], dg[B];
#pragma unroll
        for (int q = 0; q < B; ++q) {
            ok[q] = e + q * stride < nsq;
            o[q] = cu.r * pitch + cu.c;
            dg[q] = cu.r == cu.c;
            const int r = perm && ok[q] ? perm[cu.r] : cu.r, c = perm && ok[q] ? perm[cu.c] : cu.c;
            j[q] = (ok[q] && live) ? jac[mat_idx(F, i, n, nn, r, c)] : 0.0;
            cu.next();
        }
#pragma unroll
        for (int q = 0; q < B; ++q)
            if (ok[q]) a[o[q]] = fma(-g, j[q], dg[q] ? 1.0 : 0.0);
    }
}

constexpr long long kAbsMask = 0x7fffffffffffffffLL;
constexpr long long kDblMinBits = 0x0010000000000000LL;  // bits of DBL_MIN

// S consecutive states per block (4, or 2 or 1 where four matrices do not fit
// in shared memory) of 32 S kWarpsPerState threads, each matrix in shared
// memory with an odd row pitch (a column read by 32 lanes is free of bank
// conflicts).  Step k: warp w < S alone works on state w - the pivot (first largest |a|, compared as
// integer bit patterns, no FP64 instruction), the multiplier column scaled by
// the reciprocal (read through the interchange) and the interchange of the
// other columns of rows k and p; after a barrier every thread updates one
// trailing position in all S states (rows are interchanged in place, so the
// positions agree across states); a second barrier closes the step.  Loads
// and stores give each thread one state, so F-order accesses cover whole
// 32-byte sectors.
constexpr int kLuMaxStates = 4;
#ifndef PJG_LU_WPS
#define PJG_LU_WPS 2
#endif
constexpr int kWarpsPerState = PJG_LU_WPS;  // threads per block = 32 * S * kWarpsPerState

template <bool F, int S>
__global__ void __launch_bounds__(32 * S * kWarpsPerState) lu_factor_kernel(int nn, long long n, double s,
                                                           const double* __restrict__ h, double h0,
                                                           const double* jac, double* lu,
                                                           int32_t* __restrict__ piv,
                                                           int32_t* __restrict__ info)
{
    extern __shared__ double smem[];
    __shared__ double gst[S];
    constexpr int T = 32 * S * kWarpsPerState, TS = T / S;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int pitch = nn | 1;
    const int msz = nn * pitch;
    const int nsq = nn * nn;
    int* sp_base = reinterpret_cast<int*>(smem + (size_t)S * msz);
    const int ws = warp < S ? warp : 0;
    double* Aw = smem + (size_t)ws * msz;  // the pivot phase: warp w < S, state w
    int* spw = sp_base + ws * nn;
    const int my = tid % S, lane_s = tid / S;  // loads and stores: one state per thread
    double* Am = smem + (size_t)my * msz;
    const long long ngroups = (n + S - 1) / S;
    for (long long grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        const long long i0 = grp * S;
        const int here = (int)((n - i0) < S ? (n - i0) : S);
        if (tid < S) gst[tid] = tid < here ? s * (h ? h[i0 + tid] : h0) : 0.0;
        __syncthreads();
        load_newton<F, 1>(Am, pitch, nn, jac, i0 + my, n, gst[my], my < here, lane_s, TS, nullptr);
        __syncthreads();
        int first_zero = 0;  // lane 0 of warp w, for state w
        for (int k = 0; k < nn; ++k) {
            if (warp < S) {
                long long best = -1;
                int br = k;
                for (int r = k + lane; r < nn; r += 32) {
                    const long long v = __double_as_longlong(Aw[r * pitch + k]) & kAbsMask;
                    if (v > best) {
                        best = v;
                        br = r;
                    }
                }
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    const long long ob = __shfl_xor_sync(0xffffffffu, best, off);
                    const int orr = __shfl_xor_sync(0xffffffffu, br, off);
                    if (ob > best || (ob == best && orr < br)) {
                        best = ob;
                        br = orr;
                    }
                }
                const bool nonzero = best != 0;
                const double p = Aw[br * pitch + k];
                __syncwarp();  // every lane has read the pivot before row br's lane rewrites it
                if (lane == 0) {
                    spw[k] = br + 1;
                    if (!nonzero && !first_zero) first_zero = k + 1;
                }
                const bool recip = best >= kDblMinBits;
                const double inv = (nonzero && recip) ? __drcp_rn(p) : 0.0;
                // multipliers of rows r > k, read through the interchange; a lane
                // reads its own rows and row k, and writes only its own rows
                for (int r = k + 1 + lane; r < nn; r += 32) {
                    double v = Aw[(r == br ? k : r) * pitch + k];
                    if (nonzero) v = recip ? v * inv : v / p;
                    Aw[r * pitch + k] = v;
                }
                if (nonzero && br != k)
                    for (int c = lane; c < nn; c += 32)
                        if (c != k) {
                            const double t = Aw[k * pitch + c];
                            Aw[k * pitch + c] = Aw[br * pitch + c];
                            Aw[br * pitch + c] = t;
                        }
                __syncwarp();
                if (lane == 0 && nonzero) Aw[k * pitch + k] = p;
            }
            __syncthreads();
            const int m = nn - k - 1;
            const int mm = m * m;
            if (tid < mm) {
                const int base = (k + 1) * pitch + k + 1;
                Cursor cu(tid, T, m);
                for (int e = tid; e < mm; e += T) {
                    const int o = base + cu.r * pitch + cu.c;
                    const int ol = (k + 1 + cu.r) * pitch + k, ou = k * pitch + k + 1 + cu.c;
                    double l[S], u[S], v[S];
#pragma unroll
                    for (int q = 0; q < S; ++q) {
                        const double* B = smem + (size_t)q * msz;
                        l[q] = B[ol];
                        u[q] = B[ou];
                        v[q] = B[o];
                    }
#pragma unroll
                    for (int q = 0; q < S; ++q) smem[(size_t)q * msz + o] = fma(-l[q], u[q], v[q]);
                    cu.next();
                }
            }
            __syncthreads();
        }
        if (my < here) {
            Cursor cu(lane_s, TS, nn);
            for (int e = lane_s; e < nsq; e += TS) {
                lu[mat_idx(F, i0 + my, n, nn, cu.r, cu.c)] = Am[cu.r * pitch + cu.c];
                cu.next();
            }
            const int* spm = sp_base + my * nn;
            for (int k = lane_s; k < nn; k += TS) piv[vec_idx(F, i0 + my, n, nn, k)] = spm[k];
        }
        if (lane == 0 && warp < S && warp < here && info) info[i0 + warp] = first_zero;
        __syncthreads();
    }
}

// ---- Static-pivot sparse LU (no row interchanges), the factorisation of
// implicit chemistry solvers such as KPP: rows and columns are ordered once,
// on the host, by the Markowitz rule on the Jacobian's pattern, and step k
// updates only the structural rows R_k x columns C_k of the filled pattern.
// The matrix of a state stays dense in shared memory in the permuted order,
// so no position lookups are needed; GRI-Mech 3.0 takes 19,752 FMAs per state
// against 51,039 for the dense factorisation.
//
// Plan tables (int32, one device array): perm[nn] (permuted position ->
// variable), then the offsets roff, coff, loff, uoff [nn + 1 each] into the
// index lists ridx (R_k), cidx (C_k), lidx (columns c < r of L's row r),
// uidx (columns c > r of U's row r).
struct LuPlanView {
    int nn, nR, nC;  // nR = roff[nn], nC = coff[nn]
    const int *perm, *roff, *coff, *loff, *uoff, *ridx, *cidx, *lidx, *uidx;
};

// ints of the plan the factorisation reads: roff, coff [nn + 1], perm [nn],
// ridx [nR], cidx [nC]
inline int plan_factor_ints(const LuPlanView& v) { return 3 * v.nn + 2 + v.nR + v.nC; }

// S consecutive states per block (4, or 2 or 1 where four matrices do not fit
// in shared memory), eliminated in lockstep by 32 S kWarpsPerState threads:
// in loads, stores and scalings each thread serves one state, so F-order loads cover
// whole 32-byte sectors; in the update each thread takes one pattern position
// for all S states, so one index lookup and one barrier pair serve S states.
constexpr int kLusMaxStates = 4;

template <bool F, int S, bool TSM>
__global__ void __launch_bounds__(32 * S * kWarpsPerState) lu_sparse_kernel(long long n, double s,
                                                                            const double* __restrict__ h,
                                                                            double h0, const double* jac,
                                                                            double* lu,
                                                                            int32_t* __restrict__ info,
                                                                            LuPlanView pl)
{
    extern __shared__ double smem[];
    __shared__ double gst[S];
    __shared__ int fz[S];
    constexpr int T = 32 * S * kWarpsPerState, TS = T / S;
    const int nn = pl.nn;
    const int tid = threadIdx.x;
    const int pitch = nn | 1;
    const int msz = nn * pitch;
    const int nsq = nn * nn;
    const int my = tid % S;   // this thread's state slot in loads, stores and scalings
    const int lane_s = tid / S;
    double* A = smem + (size_t)my * msz;
    // the plan's index lists, in shared memory when they fit beside the matrices
    const int *proff = pl.roff, *pcoff = pl.coff, *pperm = pl.perm, *pridx = pl.ridx, *pcidx = pl.cidx;
    if (TSM) {
        int* tb = reinterpret_cast<int*>(smem + (size_t)S * msz);
        for (int q = tid; q <= nn; q += T) {
            tb[q] = pl.roff[q];
            tb[nn + 1 + q] = pl.coff[q];
        }
        for (int q = tid; q < nn; q += T) tb[2 * nn + 2 + q] = pl.perm[q];
        for (int q = tid; q < pl.nR; q += T) tb[3 * nn + 2 + q] = pl.ridx[q];
        for (int q = tid; q < pl.nC; q += T) tb[3 * nn + 2 + pl.nR + q] = pl.cidx[q];
        proff = tb;
        pcoff = tb + nn + 1;
        pperm = tb + 2 * nn + 2;
        pridx = tb + 3 * nn + 2;
        pcidx = pridx + pl.nR;
        __syncthreads();
    }
    const long long ngroups = (n + S - 1) / S;
    for (long long grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        const long long i0 = grp * S;
        const int here = (int)((n - i0) < S ? (n - i0) : S);
        if (tid < S) {
            gst[tid] = tid < here ? s * (h ? h[i0 + tid] : h0) : 0.0;
            fz[tid] = 0;
        }
        __syncthreads();
        load_newton<F, 4>(A, pitch, nn, jac, i0 + my, n, gst[my], my < here, lane_s, TS, pperm);
        __syncthreads();
        for (int k = 0; k < nn; ++k) {
            const int r0 = proff[k], nr = proff[k + 1] - r0;
            if (tid < S && !fz[tid]) {
                // first exactly zero pivot (k + 1), or first non-finite one, -(k + 1):
                // without interchanges a growing factor overflows, which the
                // caller learns from a negative info
                const double pv = smem[(size_t)tid * msz + k * pitch + k];
                if (pv == 0.0) fz[tid] = k + 1;
                else if (!isfinite(pv)) fz[tid] = -(k + 1);
            }
            if (nr == 0) continue;  // nothing below the pivot: no update, no barrier
            const int c0 = pcoff[k], nc = pcoff[k + 1] - c0;
            const int* R = pridx + r0;
            const int* C = pcidx + c0;
            if (lane_s < nr) {
                const double p = A[k * pitch + k];
                if (p != 0.0) {
                    const bool recip = fabs(p) >= DBL_MIN;
                    const double inv = recip ? __drcp_rn(p) : 0.0;
                    for (int q = lane_s; q < nr; q += TS) {
                        double* x = A + R[q] * pitch + k;
                        *x = recip ? *x * inv : *x / p;
                    }
                }
            }
            __syncthreads();
            const int mm = nr * nc;
            if (tid < mm) {
                Cursor cu(tid, T, nc);
                for (int e = tid; e < mm; e += T) {
                    const int r = R[cu.r], c = C[cu.c];
                    const int o = r * pitch + c, ol = r * pitch + k, ou = k * pitch + c;
                    double l[S], u[S], v[S];
#pragma unroll
                    for (int q = 0; q < S; ++q) {
                        const double* B = smem + (size_t)q * msz;
                        l[q] = B[ol];
                        u[q] = B[ou];
                        v[q] = B[o];
                    }
#pragma unroll
                    for (int q = 0; q < S; ++q) smem[(size_t)q * msz + o] = fma(-l[q], u[q], v[q]);
                    cu.next();
                }
            }
            __syncthreads();
        }
        if (my < here) {
            Cursor cu(lane_s, TS, nn);
            for (int e = lane_s; e < nsq; e += TS) {
                lu[mat_idx(F, i0 + my, n, nn, cu.r, cu.c)] = A[cu.r * pitch + cu.c];
                cu.next();
            }
        }
        if (tid < here && info) info[i0 + tid] = fz[tid];
        __syncthreads();
    }
}

// one thread per state: y = P b, L y = y and U x = y over the filled pattern
// only (row-oriented FMA dot products in increasing column order), x back to
// the variables' order
template <bool F>
__global__ void __launch_bounds__(128) lu_sparse_solve_kernel(long long n, const double* __restrict__ lu,
                                                              double* b, LuPlanView pl)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int nn = pl.nn;
    double y[kSolveNMax];
    for (int r = 0; r < nn; ++r) y[r] = b[vec_idx(F, i, n, nn, __ldg(pl.perm + r))];
    for (int r = 1; r < nn; ++r) {
        double acc = y[r];
        for (int q = __ldg(pl.loff + r); q < __ldg(pl.loff + r + 1); ++q) {
            const int c = __ldg(pl.lidx + q);
            acc = fma(-__ldg(lu + mat_idx(F, i, n, nn, r, c)), y[c], acc);
        }
        y[r] = acc;
    }
    for (int r = nn - 1; r >= 0; --r) {
        double acc = y[r];
        for (int q = __ldg(pl.uoff + r); q < __ldg(pl.uoff + r + 1); ++q) {
            const int c = __ldg(pl.uidx + q);
            acc = fma(-__ldg(lu + mat_idx(F, i, n, nn, r, c)), y[c], acc);
        }
        y[r] = acc / __ldg(lu + mat_idx(F, i, n, nn, r, r));
    }
    for (int r = 0; r < nn; ++r) b[vec_idx(F, i, n, nn, __ldg(pl.perm + r))] = y[r];
}

// one thread per state: row interchanges, unit-lower then upper substitution
// in the column order of LAPACK's dtrsv on a column-major matrix (the lower
// pass subtracts each y_c from the rows below in increasing c; the upper pass
// divides y_c by the diagonal and subtracts it from the rows above in
// decreasing c; every row accumulates by FMA)
template <bool F>
__global__ void __launch_bounds__(128) lu_solve_kernel(int nn, long long n,
                                                       const double* __restrict__ lu,
                                                       const int32_t* __restrict__ piv,
                                                       double* b)
{
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double y[kSolveNMax];
    for (int r = 0; r < nn; ++r) y[r] = b[vec_idx(F, i, n, nn, r)];
    for (int k = 0; k < nn; ++k) {
        const int p = piv[vec_idx(F, i, n, nn, k)] - 1;
        if (p > k && p < nn) {  // pjg_lu_factor's pivots satisfy k <= p < nn
            const double t = y[k];
            y[k] = y[p];
            y[p] = t;
        }
    }
    // row by row with a register accumulator: each row takes the same FMAs in
    // the same order as in the column sweeps (lower: c increasing; upper: c
    // decreasing from nn - 1)
    for (int r = 1; r < nn; ++r) {
        double acc = y[r];
        for (int c = 0; c < r; ++c) acc = fma(-__ldg(lu + mat_idx(F, i, n, nn, r, c)), y[c], acc);
        y[r] = acc;
    }
    for (int r = nn - 1; r >= 0; --r) {
        double acc = y[r];
        for (int c = nn - 1; c > r; --c) acc = fma(-__ldg(lu + mat_idx(F, i, n, nn, r, c)), y[c], acc);
        y[r] = acc / __ldg(lu + mat_idx(F, i, n, nn, r, r));
    }
    for (int r = 0; r < nn; ++r) b[vec_idx(F, i, n, nn, r)] = y[r];
}

// ---- Newton matrices too large for shared memory (nn > 169, up to 4096):
// one block of 256 threads per state, the matrix in global memory (the
// output array, factored in place), a blocked right-looking LU with panels of
// NB columns held in shared memory.  For each panel:
//   1. the panel (rows k0.., columns k0..k0+NB-1) is factored in shared
//      memory by the unblocked steps of lu_factor_kernel: pivot (first
//      largest |a|, bit-pattern comparison), whole-row interchange within the
//      panel, multipliers by the reciprocal, rank-1 update of the panel;
//   2. each thread owns whole columns outside the panel: it applies the
//      panel's interchanges to them in order, and for a column right of the
//      panel forms U's NB entries by forward substitution with the panel's
//      unit-lower block, then updates the column below by the NB multipliers.
// Every entry receives the same FMAs in the same order (k = 0, 1, ...) as in
// the unblocked algorithm, so the factors equal lu_factor_kernel's and the
// oracle's bit for bit; blocking only cuts the passes over the trailing
// matrix from nn to nn / NB.
constexpr int kBigThreads = 256;
constexpr int kBigMaxNN = 4096;

template <bool F, int NB>
__global__ void __launch_bounds__(kBigThreads, 2) lu_factor_big_kernel(int nn, long long n, double s,
                                                                    const double* __restrict__ h,
                                                                    double h0, const double* jac,
                                                                    double* lu, int32_t* __restrict__ piv,
                                                                    int32_t* __restrict__ info)
{
    extern __shared__ double P[];  // panel, column-major: P[cc * nn + rr], rr < nn - k0
    __shared__ long long wbest[kBigThreads / 32];
    __shared__ int wrow[kBigThreads / 32];
    __shared__ int spiv[NB];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int NW = kBigThreads / 32;
    for (long long i = blockIdx.x; i < n; i += gridDim.x) {
        auto A = [&](int r, int c) -> double& { return lu[mat_idx(F, i, n, nn, r, c)]; };
        const double g = s * (h ? h[i] : h0);
        const long long nsq = (long long)nn * nn;
        for (long long e = tid; e < nsq; e += kBigThreads) {
            // C order: consecutive threads along a row; F order: down a column
            const int r = F ? (int)(e % nn) : (int)(e / nn), c = F ? (int)(e / nn) : (int)(e % nn);
            const size_t o = mat_idx(F, i, n, nn, r, c);
            lu[o] = fma(-g, jac[o], r == c ? 1.0 : 0.0);  // in place when lu == jac
        }
        __syncthreads();
        int first_zero = 0;
        for (int k0 = 0; k0 < nn; k0 += NB) {
            const int w = nn - k0 < NB ? nn - k0 : NB, m = nn - k0;
            for (int e = tid; e < m * w; e += kBigThreads) {
                const int cc = e / m, rr = e - cc * m;
                P[cc * m + rr] = A(k0 + rr, k0 + cc);
            }
            __syncthreads();
            for (int kk = 0; kk < w; ++kk) {
                double* col = P + kk * m;
                long long best = -1;
                int br = kk;
                for (int rr = kk + tid; rr < m; rr += kBigThreads) {
                    const long long v = __double_as_longlong(col[rr]) & kAbsMask;
                    if (v > best) {
                        best = v;
                        br = rr;
                    }
                }
#pragma unroll
                for (int off = 16; off > 0; off >>= 1) {
                    const long long ob = __shfl_xor_sync(0xffffffffu, best, off);
                    const int orr = __shfl_xor_sync(0xffffffffu, br, off);
                    if (ob > best || (ob == best && orr < br)) {
                        best = ob;
                        br = orr;
                    }
                }
                if (lane == 0) {
                    wbest[warp] = best;
                    wrow[warp] = br;
                }
                __syncthreads();
                best = wbest[0];
                br = wrow[0];
#pragma unroll
                for (int q = 1; q < NW; ++q)
                    if (wbest[q] > best || (wbest[q] == best && wrow[q] < br)) {
                        best = wbest[q];
                        br = wrow[q];
                    }
                const bool nonzero = best > 0;
                if (tid == 0) {
                    spiv[kk] = nonzero ? br : kk;
                    piv[vec_idx(F, i, n, nn, k0 + kk)] = k0 + (nonzero ? br : kk) + 1;
                    if (!nonzero && !first_zero) first_zero = k0 + kk + 1;
                }
                if (nonzero && br != kk)  // whole rows of the panel
                    for (int cc = tid; cc < w; cc += kBigThreads) {
                        double* pc = P + cc * m;
                        const double t = pc[kk];
                        pc[kk] = pc[br];
                        pc[br] = t;
                    }
                __syncthreads();
                if (nonzero) {
                    const double p = col[kk];
                    if (best >= kDblMinBits) {
                        const double inv = __drcp_rn(p);
                        for (int rr = kk + 1 + tid; rr < m; rr += kBigThreads) col[rr] *= inv;
                    } else {
                        for (int rr = kk + 1 + tid; rr < m; rr += kBigThreads) col[rr] /= p;
                    }
                }
                __syncthreads();
                // rank-1 update of the panel's columns right of kk
                const int mr = m - kk - 1, nc = w - kk - 1;
                for (int e = tid; e < mr * nc; e += kBigThreads) {
                    const int cq = e / mr, rq = e - cq * mr;
                    const int cc = kk + 1 + cq, rr = kk + 1 + rq;
                    P[cc * m + rr] = fma(-col[rr], P[cc * m + kk], P[cc * m + rr]);
                }
                __syncthreads();
            }
            for (int e = tid; e < m * w; e += kBigThreads) {
                const int cc = e / m, rr = e - cc * m;
                A(k0 + rr, k0 + cc) = P[cc * m + rr];
            }
            // columns outside the panel, one thread each
            for (int c = tid; c < nn - w; c += kBigThreads) {
                const int cg = c < k0 ? c : c + w;
#pragma unroll 1
                for (int kk = 0; kk < w; ++kk) {
                    const int br = spiv[kk];
                    if (br != kk) {
                        double& x = A(k0 + kk, cg);
                        double& y = A(k0 + br, cg);
                        const double t = x;
                        x = y;
                        y = t;
                    }
                }
                if (cg < k0) continue;
                double u[NB];
#pragma unroll
                for (int q = 0; q < NB; ++q)
                    if (q < w) u[q] = A(k0 + q, cg);
#pragma unroll
                for (int q = 1; q < NB; ++q)
                    if (q < w)
#pragma unroll
                        for (int t = 0; t < NB; ++t)
                            if (t < q) u[q] = fma(-P[t * m + q], u[t], u[q]);
#pragma unroll
                for (int q = 1; q < NB; ++q)
                    if (q < w) A(k0 + q, cg) = u[q];
                // rows below the panel, four at a time (independent FMA chains)
                int r = w;
                for (; r + 4 <= m; r += 4) {
                    double a0 = A(k0 + r, cg), a1 = A(k0 + r + 1, cg), a2 = A(k0 + r + 2, cg),
                           a3 = A(k0 + r + 3, cg);
#pragma unroll
                    for (int q = 0; q < NB; ++q)
                        if (q < w) {
                            const double* Lq = P + q * m + r;
                            a0 = fma(-Lq[0], u[q], a0);
                            a1 = fma(-Lq[1], u[q], a1);
                            a2 = fma(-Lq[2], u[q], a2);
                            a3 = fma(-Lq[3], u[q], a3);
                        }
                    A(k0 + r, cg) = a0;
                    A(k0 + r + 1, cg) = a1;
                    A(k0 + r + 2, cg) = a2;
                    A(k0 + r + 3, cg) = a3;
                }
                for (; r < m; ++r) {
                    double a0 = A(k0 + r, cg);
#pragma unroll
                    for (int q = 0; q < NB; ++q)
                        if (q < w) a0 = fma(-P[q * m + r], u[q], a0);
                    A(k0 + r, cg) = a0;
                }
            }
            __syncthreads();
        }
        if (tid == 0 && info) info[i] = first_zero;
        __syncthreads();
    }
}

// The solve of lu_solve_kernel for nn > 176, one block of kSolveThreads per
// state (the column order lets the rows of one step proceed in parallel):
// the vector in shared memory, thread t owning rows t, t + T, ...; a barrier
// between column steps; each step's factor entries loaded one step ahead.
// Same operations in the same order as lu_solve_kernel and the oracle.
constexpr int kSolveThreads = 128;

template <bool F, int kSolveRows>  // rows per thread: kSolveRows * kSolveThreads >= nn
__global__ void __launch_bounds__(kSolveThreads) lu_solve_big_kernel(int nn, long long n,
                                                                     const double* __restrict__ lu,
                                                                     const int32_t* __restrict__ piv,
                                                                     double* b)
{
    extern __shared__ double y[];  // nn: accumulators; then nn: solved values
    double* x = y + nn;
    const int tid = threadIdx.x;
    for (long long i = blockIdx.x; i < n; i += gridDim.x) {
        for (int r = tid; r < nn; r += kSolveThreads) y[r] = b[vec_idx(F, i, n, nn, r)];
        __syncthreads();
        if (tid == 0)
            for (int k = 0; k < nn; ++k) {
                const int p = piv[vec_idx(F, i, n, nn, k)] - 1;
                if (p > k && p < nn) {
                    const double t = y[k];
                    y[k] = y[p];
                    y[p] = t;
                }
            }
        __syncthreads();
        // unit lower: step c subtracts y_c from rows r > c
        double nxt[kSolveRows];
#pragma unroll
        for (int q = 0; q < kSolveRows; ++q) {
            const int r = tid + q * kSolveThreads;
            nxt[q] = r > 0 && r < nn ? __ldg(lu + mat_idx(F, i, n, nn, r, 0)) : 0.0;
        }
        for (int c = 0; c < nn - 1; ++c) {
            double cur[kSolveRows];
#pragma unroll
            for (int q = 0; q < kSolveRows; ++q) {
                cur[q] = nxt[q];
                const int r = tid + q * kSolveThreads;
                nxt[q] = r > c + 1 && r < nn ? __ldg(lu + mat_idx(F, i, n, nn, r, c + 1)) : 0.0;
            }
            const double yc = y[c];  // final: rows <= c take no more updates
#pragma unroll
            for (int q = 0; q < kSolveRows; ++q) {
                const int r = tid + q * kSolveThreads;
                if (r > c && r < nn) y[r] = fma(-cur[q], yc, y[r]);
            }
            __syncthreads();
        }
        // upper: step c divides y_c by the diagonal, subtracts it from rows r < c
#pragma unroll
        for (int q = 0; q < kSolveRows; ++q) {
            const int r = tid + q * kSolveThreads;
            nxt[q] = r < nn - 1 ? __ldg(lu + mat_idx(F, i, n, nn, r, nn - 1)) : 0.0;
        }
        for (int c = nn - 1; c >= 0; --c) {
            double cur[kSolveRows];
#pragma unroll
            for (int q = 0; q < kSolveRows; ++q) {
                cur[q] = nxt[q];
                const int r = tid + q * kSolveThreads;
                nxt[q] = c > 0 && r < c - 1 ? __ldg(lu + mat_idx(F, i, n, nn, r, c - 1)) : 0.0;
            }
            const double yc = y[c] / __ldg(lu + mat_idx(F, i, n, nn, c, c));
            if (tid == c % kSolveThreads) x[c] = yc;
#pragma unroll
            for (int q = 0; q < kSolveRows; ++q) {
                const int r = tid + q * kSolveThreads;
                if (r < c) y[r] = fma(-cur[q], yc, y[r]);
            }
            __syncthreads();
        }
        for (int r = tid; r < nn; r += kSolveThreads) b[vec_idx(F, i, n, nn, r)] = x[r];
        __syncthreads();
    }
}

// Stage arithmetic of the two-stage Rosenbrock method ROS2, element-wise with
// a per-state step h_i:
//   op 0: out = x + h k            (the second stage's state, y + h k1)
//   op 1: out = f - 2 k            (the second stage's right-hand side)
//   op 2: out = x + h (1.5 k + 0.5 z), err = h (0.5 (k + z))
template <bool F>
__global__ void ros2_combine_kernel(int op, int nn, long long n, const double* __restrict__ h,
                                    double h0, const double* __restrict__ x,
                                    const double* __restrict__ k, const double* __restrict__ z,
                                    double* out, double* err)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n * nn) return;
    const long long i = F ? e % n : e / nn;
    const double hi = h ? h[i] : h0;
    const double kv = k[e];
    if (op == 0) {
        out[e] = fma(hi, kv, x[e]);
    } else if (op == 1) {
        out[e] = fma(-2.0, kv, x[e]);
    } else {
        const double zv = z[e];
        out[e] = fma(hi, fma(1.5, kv, 0.5 * zv), x[e]);
        if (err) err[e] = hi * (0.5 * (kv + zv));
    }
}

template <int S>
int lu_factor_launch(int nn, long long n, char order, double s, const double* h, double h0,
                     const double* jac, double* lu, int32_t* piv, int32_t* info, cudaStream_t st, int sms)
{
    const size_t smem = (size_t)S * ((size_t)nn * (nn | 1) * sizeof(double) + (size_t)nn * sizeof(int));
    const void* fn = (const void*)lu_factor_kernel<false, S>;
    const void* fnF = (const void*)lu_factor_kernel<true, S>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaFuncSetAttribute(fnF, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return pjg_internal_fail(PJG_ERR_CUDA, "cannot reserve shared memory for the LU kernel");
    int per_sm = 0;
    const int threads = 32 * S * kWarpsPerState;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem) != cudaSuccess || per_sm < 1)
        return pjg_internal_fail(PJG_ERR_CUDA, "LU kernel does not fit on the device");
    long long grid = (long long)sms * per_sm;
    const long long groups = (n + S - 1) / S;
    if (groups < grid) grid = groups;
    if (order == 'F')
        lu_factor_kernel<true, S><<<(int)grid, threads, smem, st>>>(nn, n, s, h, h0, jac, lu, piv, info);
    else
        lu_factor_kernel<false, S><<<(int)grid, threads, smem, st>>>(nn, n, s, h, h0, jac, lu, piv, info);
    return 0;
}

template <int NB>
int lu_factor_big_launch(int nn, long long n, char order, double s, const double* h, double h0,
                         const double* jac, double* lu, int32_t* piv, int32_t* info, cudaStream_t st,
                         int sms)
{
    const size_t smem = (size_t)nn * NB * sizeof(double);
    const void* fn = (const void*)lu_factor_big_kernel<false, NB>;
    const void* fnF = (const void*)lu_factor_big_kernel<true, NB>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaFuncSetAttribute(fnF, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return pjg_internal_fail(PJG_ERR_CUDA, "cannot reserve shared memory for the LU kernel");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kBigThreads, smem) != cudaSuccess ||
        per_sm < 1)
        return pjg_internal_fail(PJG_ERR_CUDA, "LU kernel does not fit on the device");
    long long grid = (long long)sms * per_sm;
    if (n < grid) grid = n;
    if (order == 'F')
        lu_factor_big_kernel<true, NB><<<(int)grid, kBigThreads, smem, st>>>(nn, n, s, h, h0, jac, lu, piv, info);
    else
        lu_factor_big_kernel<false, NB><<<(int)grid, kBigThreads, smem, st>>>(nn, n, s, h, h0, jac, lu, piv, info);
    return 0;
}

template <int R>
int lu_solve_big_launch(int nn, long long n, char order, const double* lu, const int32_t* piv,
                        double* b, cudaStream_t st)
{
    const size_t smem = 2 * (size_t)nn * sizeof(double);
    const void* fn = (const void*)lu_solve_big_kernel<false, R>;
    const void* fnF = (const void*)lu_solve_big_kernel<true, R>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaFuncSetAttribute(fnF, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return pjg_internal_fail(PJG_ERR_CUDA, "cannot reserve shared memory for the LU solve");
    const int grid = (int)(n < (1 << 30) ? n : (1 << 30));
    if (order == 'F')
        lu_solve_big_kernel<true, R><<<grid, kSolveThreads, smem, st>>>(nn, n, lu, piv, b);
    else
        lu_solve_big_kernel<false, R><<<grid, kSolveThreads, smem, st>>>(nn, n, lu, piv, b);
    return 0;
}

int sm_count(int* sms)
{
    static int cached = 0;
    if (!cached) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&cached, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return pjg_internal_fail(PJG_ERR_CUDA, "device query failed");
    }
    *sms = cached;
    return 0;
}

constexpr size_t kSmemLimit = (227u << 10) - 64;  // opt-in shared memory of one block, less the static part

// ---- host side of the static-pivot plan

// Markowitz order of a square pattern (row-major bytes, diagonal included):
// at each step the remaining diagonal entry with the least
// (row count - 1) x (column count - 1) over the remaining submatrix, the
// lowest index on ties; the pattern fills in as the step eliminates.
static void markowitz_order(int nn, std::vector<char> A, std::vector<int>& perm)
{
    std::vector<char> done(nn, 0);
    perm.clear();
    for (int step = 0; step < nn; ++step) {
        int best = -1;
        long long bscore = 0;
        for (int v = 0; v < nn; ++v) {
            if (done[v]) continue;
            long long rc = 0, cc = 0;
            for (int j = 0; j < nn; ++j)
                if (!done[j] && j != v) {
                    rc += A[(size_t)v * nn + j];
                    cc += A[(size_t)j * nn + v];
                }
            const long long sc = rc * cc;
            if (best < 0 || sc < bscore) {
                best = v;
                bscore = sc;
            }
        }
        for (int r = 0; r < nn; ++r) {
            if (done[r] || r == best || !A[(size_t)r * nn + best]) continue;
            for (int c = 0; c < nn; ++c)
                if (!done[c] && c != best && A[(size_t)best * nn + c]) A[(size_t)r * nn + c] = 1;
        }
        done[best] = 1;
        perm.push_back(best);
    }
}

struct LuPlan {
    int nn = 0;
    int* d = nullptr;  // device tables
    LuPlanView view{};
    std::vector<int> perm;
    long long fma = 0;
    int nnz_lu = 0;
};

// pattern of M = I - s h J from the Jacobian's CRS pattern (C order rows)
static int build_plan_tables(int nn, const int* row_ptr, const int* col_ind, std::vector<int>& perm,
                             std::vector<int>& tab, long long* fma, int* nnz_lu)
{
    std::vector<char> A((size_t)nn * nn, 0);
    for (int r = 0; r < nn; ++r) {
        A[(size_t)r * nn + r] = 1;
        for (int q = row_ptr[r]; q < row_ptr[r + 1]; ++q) {
            const int c = col_ind[q];
            if (c < 0 || c >= nn) return PJG_ERR_ARG;
            A[(size_t)r * nn + c] = 1;
        }
    }
    markowitz_order(nn, A, perm);
    std::vector<char> B((size_t)nn * nn);
    for (int r = 0; r < nn; ++r)
        for (int c = 0; c < nn; ++c) B[(size_t)r * nn + c] = A[(size_t)perm[r] * nn + perm[c]];
    std::vector<int> roff(1, 0), coff(1, 0), ridx, cidx;
    *fma = 0;
    for (int k = 0; k < nn; ++k) {
        const size_t r_before = ridx.size(), c_before = cidx.size();
        for (int r = k + 1; r < nn; ++r)
            if (B[(size_t)r * nn + k]) ridx.push_back(r);
        for (int c = k + 1; c < nn; ++c)
            if (B[(size_t)k * nn + c]) cidx.push_back(c);
        for (size_t a = r_before; a < ridx.size(); ++a)
            for (size_t b = c_before; b < cidx.size(); ++b) B[(size_t)ridx[a] * nn + cidx[b]] = 1;
        *fma += (long long)(ridx.size() - r_before) * (long long)(cidx.size() - c_before);
        roff.push_back((int)ridx.size());
        coff.push_back((int)cidx.size());
    }
    std::vector<int> loff(1, 0), uoff(1, 0), lidx, uidx;
    *nnz_lu = 0;
    for (int r = 0; r < nn; ++r) {
        for (int c = 0; c < nn; ++c) {
            if (!B[(size_t)r * nn + c]) continue;
            ++*nnz_lu;
            if (c < r) lidx.push_back(c);
            if (c > r) uidx.push_back(c);
        }
        loff.push_back((int)lidx.size());
        uoff.push_back((int)uidx.size());
    }
    tab.clear();
    tab.insert(tab.end(), perm.begin(), perm.end());
    for (auto* v : {&roff, &coff, &loff, &uoff}) tab.insert(tab.end(), v->begin(), v->end());
    for (auto* v : {&ridx, &cidx, &lidx, &uidx}) tab.insert(tab.end(), v->begin(), v->end());
    tab.push_back(0);  // keeps every list's end inside the array
    return 0;
}

template <int S, bool TSM>
int lu_sparse_launch(const LuPlan* pl, long long n, char order, double s, const double* h, double h0,
                     const double* jac, double* lu, int32_t* info, cudaStream_t st, int sms)
{
    const size_t smem = (size_t)S * pl->nn * (pl->nn | 1) * sizeof(double) +
                        (TSM ? (size_t)plan_factor_ints(pl->view) * sizeof(int) : 0);
    const void* fn = (const void*)lu_sparse_kernel<false, S, TSM>;
    const void* fnF = (const void*)lu_sparse_kernel<true, S, TSM>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess ||
        cudaFuncSetAttribute(fnF, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return pjg_internal_fail(PJG_ERR_CUDA, "cannot reserve shared memory for the sparse LU kernel");
    const int threads = 32 * S * kWarpsPerState;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, smem) != cudaSuccess || per_sm < 1)
        return pjg_internal_fail(PJG_ERR_CUDA, "sparse LU kernel does not fit on the device");
    long long grid = (long long)sms * per_sm;
    const long long groups = (n + S - 1) / S;
    if (groups < grid) grid = groups;
    if (order == 'F')
        lu_sparse_kernel<true, S, TSM><<<(int)grid, threads, smem, st>>>(n, s, h, h0, jac, lu, info, pl->view);
    else
        lu_sparse_kernel<false, S, TSM><<<(int)grid, threads, smem, st>>>(n, s, h, h0, jac, lu, info, pl->view);
    return 0;
}

}  // namespace

extern "C" int pjg_internal_lu_factor(int32_t nn, int64_t n, char order, double s, const double* h, double h0,
                           const double* jac, double* lu, int32_t* piv, int32_t* info,
                           cudaStream_t st)
{
    if (nn < 1 || nn > kBigMaxNN) return pjg_internal_fail(PJG_ERR_UNSUPPORTED, "LU: nn must be in [1, 4096]");
    if (n < 0) return pjg_internal_fail(PJG_ERR_ARG, "negative problem size");
    if (order != 'C' && order != 'F') return pjg_internal_fail(PJG_ERR_ARG, "order must be 'C' or 'F'");
    if (n == 0) return 0;
    if (!jac || !lu || !piv) return pjg_internal_fail(PJG_ERR_ARG, "null array");
    int sms = 0;
    if (int rc = sm_count(&sms)) return rc;
    const size_t per_state = (size_t)nn * (nn | 1) * sizeof(double) + (size_t)nn * sizeof(int);
    int rc;
    if (nn > kLuMaxNN) {
        // global-memory blocked factorisation; panel width by the shared memory it takes
        if ((size_t)nn * 16 * sizeof(double) <= kSmemLimit)
            rc = lu_factor_big_launch<16>(nn, n, order, s, h, h0, jac, lu, piv, info, st, sms);
        else if ((size_t)nn * 8 * sizeof(double) <= kSmemLimit)
            rc = lu_factor_big_launch<8>(nn, n, order, s, h, h0, jac, lu, piv, info, st, sms);
        else
            rc = lu_factor_big_launch<4>(nn, n, order, s, h, h0, jac, lu, piv, info, st, sms);
    } else if (kLuMaxStates * per_state <= kSmemLimit)
        rc = lu_factor_launch<kLuMaxStates>(nn, n, order, s, h, h0, jac, lu, piv, info, st, sms);
    else if (2 * per_state <= kSmemLimit)
        rc = lu_factor_launch<2>(nn, n, order, s, h, h0, jac, lu, piv, info, st, sms);
    else
        rc = lu_factor_launch<1>(nn, n, order, s, h, h0, jac, lu, piv, info, st, sms);
    if (rc) return rc;
    pjg_internal_count_launch();
    if (cudaGetLastError() != cudaSuccess) return pjg_internal_fail(PJG_ERR_CUDA, "LU factor launch failed");
    return 0;
}

extern "C" int pjg_internal_lu_solve(int32_t nn, int64_t n, char order, const double* lu, const int32_t* piv,
                          double* b, cudaStream_t st)
{
    if (nn < 1 || nn > kBigMaxNN) return pjg_internal_fail(PJG_ERR_UNSUPPORTED, "LU: nn must be in [1, 4096]");
    if (n < 0) return pjg_internal_fail(PJG_ERR_ARG, "negative problem size");
    if (order != 'C' && order != 'F') return pjg_internal_fail(PJG_ERR_ARG, "order must be 'C' or 'F'");
    if (n == 0) return 0;
    if (!lu || !piv || !b) return pjg_internal_fail(PJG_ERR_ARG, "null array");
    const int grid = (int)((n + 127) / 128);
    if (nn > kSolveNMax) {
        int rc;
        if (nn <= 4 * kSolveThreads) rc = lu_solve_big_launch<4>(nn, n, order, lu, piv, b, st);
        else if (nn <= 8 * kSolveThreads) rc = lu_solve_big_launch<8>(nn, n, order, lu, piv, b, st);
        else if (nn <= 16 * kSolveThreads) rc = lu_solve_big_launch<16>(nn, n, order, lu, piv, b, st);
        else rc = lu_solve_big_launch<32>(nn, n, order, lu, piv, b, st);
        if (rc) return rc;
    } else if (order == 'F')
        lu_solve_kernel<true><<<grid, 128, 0, st>>>(nn, n, lu, piv, b);
    else
        lu_solve_kernel<false><<<grid, 128, 0, st>>>(nn, n, lu, piv, b);
    pjg_internal_count_launch();
    if (cudaGetLastError() != cudaSuccess) return pjg_internal_fail(PJG_ERR_CUDA, "LU solve launch failed");
    return 0;
}

extern "C" int pjg_internal_ros2_combine(int op, int32_t nn, int64_t n, char order, const double* h, double h0,
                              const double* x, const double* k, const double* z, double* out,
                              double* err, cudaStream_t st)
{
    const long long total = (long long)n * nn;
    if (total == 0) return 0;
    const int grid = (int)((total + 255) / 256);
    if (order == 'F')
        ros2_combine_kernel<true><<<grid, 256, 0, st>>>(op, nn, n, h, h0, x, k, z, out, err);
    else
        ros2_combine_kernel<false><<<grid, 256, 0, st>>>(op, nn, n, h, h0, x, k, z, out, err);
    pjg_internal_count_launch();
    if (cudaGetLastError() != cudaSuccess) return pjg_internal_fail(PJG_ERR_CUDA, "ROS2 stage launch failed");
    return 0;
}

// static-pivot plans are owned by the mechanism (pjg_capi.cu)
extern "C" int pjg_internal_lu_plan_create(int32_t nn, const int32_t* row_ptr, const int32_t* col_ind,
                                           void** out)
{
    if (nn < 1 || nn > kLuMaxNN) return pjg_internal_fail(PJG_ERR_UNSUPPORTED, "LU: nn must be in [1, 169]");
    LuPlan* pl = new LuPlan();
    pl->nn = nn;
    std::vector<int> tab;
    if (build_plan_tables(nn, row_ptr, col_ind, pl->perm, tab, &pl->fma, &pl->nnz_lu)) {
        delete pl;
        return pjg_internal_fail(PJG_ERR_TABLES, "Jacobian pattern index out of range");
    }
    if (cudaMalloc((void**)&pl->d, tab.size() * sizeof(int)) != cudaSuccess ||
        cudaMemcpy(pl->d, tab.data(), tab.size() * sizeof(int), cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(pl->d);
        delete pl;
        return pjg_internal_fail(PJG_ERR_CUDA, "cannot upload the sparse LU plan");
    }
    const int* d = pl->d;
    LuPlanView& v = pl->view;
    v.nn = nn;
    v.perm = d;
    v.roff = d + nn;
    v.coff = v.roff + nn + 1;
    v.loff = v.coff + nn + 1;
    v.uoff = v.loff + nn + 1;
    v.ridx = v.uoff + nn + 1;
    v.nR = tab[2 * nn];
    v.nC = tab[3 * nn + 1];
    v.cidx = v.ridx + tab[2 * nn];      // + roff[nn]
    v.lidx = v.cidx + tab[3 * nn + 1];  // + coff[nn]
    v.uidx = v.lidx + tab[4 * nn + 2];  // + loff[nn]
    *out = pl;
    return 0;
}

extern "C" void pjg_internal_lu_plan_destroy(void* p)
{
    LuPlan* pl = static_cast<LuPlan*>(p);
    if (!pl) return;
    cudaFree(pl->d);
    delete pl;
}

extern "C" void pjg_internal_lu_plan_info(const void* p, int32_t* perm, int32_t* nnz_lu, int64_t* fma)
{
    const LuPlan* pl = static_cast<const LuPlan*>(p);
    if (perm)
        for (int k = 0; k < pl->nn; ++k) perm[k] = pl->perm[k];
    if (nnz_lu) *nnz_lu = pl->nnz_lu;
    if (fma) *fma = pl->fma;
}

extern "C" int pjg_internal_lu_factor_sparse(const void* p, int64_t n, char order, double s, const double* h,
                                             double h0, const double* jac, double* lu, int32_t* info,
                                             cudaStream_t st)
{
    const LuPlan* pl = static_cast<const LuPlan*>(p);
    if (n < 0) return pjg_internal_fail(PJG_ERR_ARG, "negative problem size");
    if (order != 'C' && order != 'F') return pjg_internal_fail(PJG_ERR_ARG, "order must be 'C' or 'F'");
    if (n == 0) return 0;
    if (!jac || !lu) return pjg_internal_fail(PJG_ERR_ARG, "null array");
    int sms = 0;
    if (int rc = sm_count(&sms)) return rc;
    // states per block: the most (4, 2, 1) whose matrices fit, with the
    // plan's index lists beside them when those fit too
    const size_t per_state = (size_t)pl->nn * (pl->nn | 1) * sizeof(double);
    const size_t tabs = (size_t)plan_factor_ints(pl->view) * sizeof(int);
    const size_t limit = kSmemLimit;
    int rc;
    if (kLusMaxStates * per_state + tabs <= limit)
        rc = lu_sparse_launch<kLusMaxStates, true>(pl, n, order, s, h, h0, jac, lu, info, st, sms);
    else if (kLusMaxStates * per_state <= limit)
        rc = lu_sparse_launch<kLusMaxStates, false>(pl, n, order, s, h, h0, jac, lu, info, st, sms);
    else if (2 * per_state + tabs <= limit)
        rc = lu_sparse_launch<2, true>(pl, n, order, s, h, h0, jac, lu, info, st, sms);
    else if (2 * per_state <= limit)
        rc = lu_sparse_launch<2, false>(pl, n, order, s, h, h0, jac, lu, info, st, sms);
    else if (per_state + tabs <= limit)
        rc = lu_sparse_launch<1, true>(pl, n, order, s, h, h0, jac, lu, info, st, sms);
    else
        rc = lu_sparse_launch<1, false>(pl, n, order, s, h, h0, jac, lu, info, st, sms);
    if (rc) return rc;
    pjg_internal_count_launch();
    if (cudaGetLastError() != cudaSuccess) return pjg_internal_fail(PJG_ERR_CUDA, "sparse LU launch failed");
    return 0;
}

extern "C" int pjg_internal_lu_solve_sparse(const void* p, int64_t n, char order, const double* lu, double* b,
                                            cudaStream_t st)
{
    const LuPlan* pl = static_cast<const LuPlan*>(p);
    if (n < 0) return pjg_internal_fail(PJG_ERR_ARG, "negative problem size");
    if (order != 'C' && order != 'F') return pjg_internal_fail(PJG_ERR_ARG, "order must be 'C' or 'F'");
    if (n == 0) return 0;
    if (!lu || !b) return pjg_internal_fail(PJG_ERR_ARG, "null array");
    const int grid = (int)((n + 127) / 128);
    if (order == 'F')
        lu_sparse_solve_kernel<true><<<grid, 128, 0, st>>>(n, lu, b, pl->view);
    else
        lu_sparse_solve_kernel<false><<<grid, 128, 0, st>>>(n, lu, b, pl->view);
    pjg_internal_count_launch();
    if (cudaGetLastError() != cudaSuccess) return pjg_internal_fail(PJG_ERR_CUDA, "sparse LU solve launch failed");
    return 0;
}

// host only: the Markowitz order and the counts of a pattern (no device work;
// any nn up to 4,096, beyond what the factorisation kernels take)
extern "C" int pjg_lu_symbolic(int32_t nn, const int32_t* row_ptr, const int32_t* col_ind, int32_t* perm,
                               int32_t* nnz_lu, int64_t* fma)
{
    if (nn < 1 || nn > 4096) return pjg_internal_fail(PJG_ERR_UNSUPPORTED, "LU symbolic: nn must be in [1, 4096]");
    if (!row_ptr || !col_ind) return pjg_internal_fail(PJG_ERR_ARG, "null array");
    std::vector<int> pv, tab;
    long long f = 0;
    int z = 0;
    if (build_plan_tables(nn, row_ptr, col_ind, pv, tab, &f, &z))
        return pjg_internal_fail(PJG_ERR_ARG, "pattern index out of range");
    if (perm)
        for (int k = 0; k < nn; ++k) perm[k] = pv[k];
    if (nnz_lu) *nnz_lu = z;
    if (fma) *fma = f;
    return 0;
}

extern "C" int pjg_lu_factor(int32_t nn, int64_t n, char order, double s, const double* h, double h0,
                             const double* jac, double* lu, int32_t* piv, int32_t* info, void* stream)
{
    return pjg_internal_lu_factor(nn, n, order, s, h, h0, jac, lu, piv, info, (cudaStream_t)stream);
}

extern "C" int pjg_lu_solve(int32_t nn, int64_t n, char order, const double* lu, const int32_t* piv,
                            double* b, void* stream)
{
    return pjg_internal_lu_solve(nn, n, order, lu, piv, b, (cudaStream_t)stream);
}
