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
// number of active lanes, so the factorisation spreads each state's flattened
// trailing block over the threads of a block (one state per block, its matrix
// in shared memory) to keep the lanes full; the solve, which reads each
// factor entry once, is one thread per state and bound by HBM.
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>

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

constexpr long long kAbsMask = 0x7fffffffffffffffLL;
constexpr long long kDblMinBits = 0x0010000000000000LL;  // bits of DBL_MIN

// One state per block of LU_WARPS warps, its matrix in shared memory (odd
// row pitch: a column read by 32 lanes is free of bank conflicts).  Step k:
// every warp finds the pivot (integer comparison of |a| bit patterns, no
// FP64 instruction); warp 0 forms the interchanged multiplier column scaled
// by the reciprocal into lvec while all threads interchange the other
// columns of rows k and p; after a barrier the trailing block gets the rank-1
// update (elements spread flat over the block's threads, LU_BATCH per thread at
// a time) and column k takes lvec; a second barrier closes the step.
#ifndef LU_WARPS
#define LU_WARPS 2  // 193 ms per 1M GRI states; 1, 3 and 4 warps: 201, 211, 205 ms
#endif
#ifndef LU_MINB
#define LU_MINB 9
#endif
#ifndef LU_BATCH
#define LU_BATCH 4  // trailing elements a thread loads before it stores
#endif
#define LU_THREADS (32 * LU_WARPS)

template <bool F>
__global__ void __launch_bounds__(LU_THREADS, LU_MINB) lu_factor_kernel(int nn, long long n, double s,
                                                                  const double* __restrict__ h,
                                                                  double h0, const double* jac,
                                                                  double* lu,
                                                                  int32_t* __restrict__ piv,
                                                                  int32_t* __restrict__ info)
{
    extern __shared__ double smem[];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int pitch = nn | 1;
    double* a = smem;
    double* lvec = a + (size_t)nn * pitch;
    int* sp = reinterpret_cast<int*>(lvec + nn);
    const int nsq = nn * nn;
    for (long long i = blockIdx.x; i < n; i += gridDim.x) {
        const double g = s * (h ? h[i] : h0);
        {
            Cursor cu(tid, LU_THREADS, nn);
            for (int e = tid; e < nsq; e += LU_THREADS) {
                const double j = jac[mat_idx(F, i, n, nn, cu.r, cu.c)];
                a[cu.r * pitch + cu.c] = fma(-g, j, cu.r == cu.c ? 1.0 : 0.0);
                cu.next();
            }
        }
        __syncthreads();
        int first_zero = 0;  // thread 0's
        for (int k = 0; k < nn; ++k) {
            long long best = -1;
            int br = k;
            for (int r = k + lane; r < nn; r += 32) {
                const long long v = __double_as_longlong(a[r * pitch + k]) & kAbsMask;
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
            const int m = nn - k - 1;
            double p = 0.0;
            if (warp == 0) {
                p = a[br * pitch + k];
                if (lane == 0) {
                    sp[k] = br + 1;
                    if (!nonzero && !first_zero) first_zero = k + 1;
                }
                const bool recip = best >= kDblMinBits;
                const double inv = (nonzero && recip) ? __drcp_rn(p) : 0.0;
                for (int r = k + 1 + lane; r < nn; r += 32) {
                    double v = a[(r == br ? k : r) * pitch + k];
                    if (nonzero) v = recip ? v * inv : v / p;
                    lvec[r] = v;
                }
            }
            if (nonzero && br != k)
                for (int c = tid; c < nn; c += LU_THREADS)
                    if (c != k) {
                        const double t = a[k * pitch + c];
                        a[k * pitch + c] = a[br * pitch + c];
                        a[br * pitch + c] = t;
                    }
            __syncthreads();
            if (tid == 0 && nonzero) a[k * pitch + k] = p;
            for (int r = k + 1 + tid; r < nn; r += LU_THREADS) a[r * pitch + k] = lvec[r];
            const int mm = m * m;
            if (tid < mm) {
                const double* urow = a + k * pitch + k + 1;
                const double* lv = lvec + k + 1;
                double* t = a + (k + 1) * pitch + k + 1;
                Cursor cu(tid, LU_THREADS, m);
                for (int e = tid; e < mm; e += LU_BATCH * LU_THREADS) {
                    int o[LU_BATCH];
                    double l[LU_BATCH], u[LU_BATCH], v[LU_BATCH];
                    bool ok[LU_BATCH];
#pragma unroll
                    for (int q = 0; q < LU_BATCH; ++q) {
                        ok[q] = e + q * LU_THREADS < mm;
                        o[q] = cu.r * pitch + cu.c;
                        if (ok[q]) {
                            l[q] = lv[cu.r];
                            u[q] = urow[cu.c];
                            v[q] = t[o[q]];
                        }
                        cu.next();
                    }
#pragma unroll
                    for (int q = 0; q < LU_BATCH; ++q)
                        if (ok[q]) t[o[q]] = fma(-l[q], u[q], v[q]);
                }
            }
            __syncthreads();
        }
        {
            Cursor cu(tid, LU_THREADS, nn);
            for (int e = tid; e < nsq; e += LU_THREADS) {
                lu[mat_idx(F, i, n, nn, cu.r, cu.c)] = a[cu.r * pitch + cu.c];
                cu.next();
            }
        }
        for (int k = tid; k < nn; k += LU_THREADS) piv[vec_idx(F, i, n, nn, k)] = sp[k];
        if (tid == 0 && info) info[i] = first_zero;
        __syncthreads();
    }
}

// one thread per state: row interchanges, unit-lower then upper substitution
// (row-oriented: each y_r accumulates its dot product in increasing column
// order by FMA, and the upper rows divide by the diagonal)
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
    for (int r = 1; r < nn; ++r) {
        double acc = y[r];
        for (int c = 0; c < r; ++c) acc = fma(-__ldg(lu + mat_idx(F, i, n, nn, r, c)), y[c], acc);
        y[r] = acc;
    }
    for (int r = nn - 1; r >= 0; --r) {
        double acc = y[r];
        for (int c = r + 1; c < nn; ++c) acc = fma(-__ldg(lu + mat_idx(F, i, n, nn, r, c)), y[c], acc);
        y[r] = acc / __ldg(lu + mat_idx(F, i, n, nn, r, r));
    }
    for (int r = 0; r < nn; ++r) b[vec_idx(F, i, n, nn, r)] = y[r];
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

int lu_factor_config(int nn, size_t* smem, int* grid)
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return pjg_internal_fail(PJG_ERR_CUDA, "device query failed");
    }
    *smem = (size_t)nn * (nn | 1) * sizeof(double) + (size_t)nn * (sizeof(double) + sizeof(int));
    const void* fn = (const void*)lu_factor_kernel<false>;
    const void* fnF = (const void*)lu_factor_kernel<true>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem) != cudaSuccess ||
        cudaFuncSetAttribute(fnF, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem) != cudaSuccess)
        return pjg_internal_fail(PJG_ERR_CUDA, "cannot reserve shared memory for the LU kernel");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, LU_THREADS, *smem) != cudaSuccess ||
        per_sm < 1)
        return pjg_internal_fail(PJG_ERR_CUDA, "LU kernel does not fit on the device");
    *grid = sms * per_sm;
    return 0;
}

}  // namespace

extern "C" int pjg_internal_lu_factor(int32_t nn, int64_t n, char order, double s, const double* h, double h0,
                           const double* jac, double* lu, int32_t* piv, int32_t* info,
                           cudaStream_t st)
{
    if (nn < 1 || nn > kLuMaxNN) return pjg_internal_fail(PJG_ERR_UNSUPPORTED, "LU: nn must be in [1, 169]");
    if (n < 0) return pjg_internal_fail(PJG_ERR_ARG, "negative problem size");
    if (order != 'C' && order != 'F') return pjg_internal_fail(PJG_ERR_ARG, "order must be 'C' or 'F'");
    if (n == 0) return 0;
    if (!jac || !lu || !piv) return pjg_internal_fail(PJG_ERR_ARG, "null array");
    int grid = 1;
    size_t smem = 0;
    if (int rc = lu_factor_config(nn, &smem, &grid)) return rc;
    if (n < grid) grid = (int)n;
    if (order == 'F')
        lu_factor_kernel<true><<<grid, LU_THREADS, smem, st>>>(nn, n, s, h, h0, jac, lu, piv, info);
    else
        lu_factor_kernel<false><<<grid, LU_THREADS, smem, st>>>(nn, n, s, h, h0, jac, lu, piv, info);
    pjg_internal_count_launch();
    if (cudaGetLastError() != cudaSuccess) return pjg_internal_fail(PJG_ERR_CUDA, "LU factor launch failed");
    return 0;
}

extern "C" int pjg_internal_lu_solve(int32_t nn, int64_t n, char order, const double* lu, const int32_t* piv,
                          double* b, cudaStream_t st)
{
    if (nn < 1 || nn > kLuMaxNN) return pjg_internal_fail(PJG_ERR_UNSUPPORTED, "LU: nn must be in [1, 169]");
    if (n < 0) return pjg_internal_fail(PJG_ERR_ARG, "negative problem size");
    if (order != 'C' && order != 'F') return pjg_internal_fail(PJG_ERR_ARG, "order must be 'C' or 'F'");
    if (n == 0) return 0;
    if (!lu || !piv || !b) return pjg_internal_fail(PJG_ERR_ARG, "null array");
    const int grid = (int)((n + 127) / 128);
    if (order == 'F')
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
