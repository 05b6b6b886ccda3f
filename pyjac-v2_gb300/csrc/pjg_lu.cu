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
// number of active lanes, so the factorisation gives each state a whole warp
// and spreads the flattened trailing block over the lanes (one state per
// warp, its matrix in shared memory); the solve, which reads each factor
// entry once, is one thread per state and bound by HBM.
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

// advance a flattened (row, column) cursor of an m-column block by 32 elements
__device__ __forceinline__ void adv32(int& r, int& c, int m)
{
    c += 32;
    while (c >= m) {
        c -= m;
        ++r;
    }
}

template <bool F>
__global__ void __launch_bounds__(256) lu_factor_kernel(int nn, long long n, double s,
                                                        const double* __restrict__ h, double h0,
                                                        const double* jac, double* lu,
                                                        int32_t* __restrict__ piv,
                                                        int32_t* __restrict__ info, int wpb)
{
    extern __shared__ double smem[];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int pitch = nn | 1;  // odd pitch: a column read by 32 lanes is free of bank conflicts
    double* a = smem + (size_t)w * nn * pitch;
    int* sp = reinterpret_cast<int*>(smem + (size_t)wpb * nn * pitch) + w * nn;
    const long long stride = (long long)gridDim.x * wpb;
    const int nsq = nn * nn;
    for (long long i = (long long)blockIdx.x * wpb + w; i < n; i += stride) {
        const double g = s * (h ? h[i] : h0);
        for (int e = lane; e < nsq; e += 32) {
            const int r = e / nn, c = e - r * nn;
            const double j = jac[mat_idx(F, i, n, nn, r, c)];
            a[r * pitch + c] = fma(-g, j, r == c ? 1.0 : 0.0);
        }
        __syncwarp();
        int first_zero = 0;
        for (int k = 0; k < nn; ++k) {
            // pivot: first row of largest |a_rk|, r >= k (|x| compared as bit patterns)
            long long best = -1;
            int br = k;
            for (int r = k + lane; r < nn; r += 32) {
                const long long v = __double_as_longlong(a[r * pitch + k]) & 0x7fffffffffffffffLL;
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
            if (lane == 0) sp[k] = br + 1;
            const double p = a[br * pitch + k];
            const int m = nn - k - 1;
            if (p != 0.0) {
                if (br != k)
                    for (int c = lane; c < nn; c += 32) {
                        const double t = a[k * pitch + c];
                        a[k * pitch + c] = a[br * pitch + c];
                        a[br * pitch + c] = t;
                    }
                __syncwarp();
                if (fabs(p) >= DBL_MIN) {
                    const double inv = 1.0 / p;
                    for (int r = k + 1 + lane; r < nn; r += 32) a[r * pitch + k] *= inv;
                } else {
                    for (int r = k + 1 + lane; r < nn; r += 32) a[r * pitch + k] /= p;
                }
            } else if (!first_zero) {
                first_zero = k + 1;
            }
            __syncwarp();
            // rank-1 update of the m x m trailing block, four elements per lane at a time
            const int mm = m * m;
            if (mm > 0) {
                const double* urow = a + k * pitch + k + 1;
                const double* lcol = a + (k + 1) * pitch + k;
                double* t = a + (k + 1) * pitch + k + 1;
                int r = lane / m, c = lane - (lane / m) * m;
                for (int e = lane; e < mm; e += 128) {
                    int o[4];
                    double l[4], u[4], v[4];
                    bool ok[4];
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        ok[q] = e + 32 * q < mm;
                        o[q] = r * pitch + c;
                        if (ok[q]) {
                            l[q] = lcol[r * pitch];
                            u[q] = urow[c];
                            v[q] = t[o[q]];
                        }
                        adv32(r, c, m);
                    }
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (ok[q]) t[o[q]] = fma(-l[q], u[q], v[q]);
                }
            }
            __syncwarp();
        }
        for (int e = lane; e < nsq; e += 32) {
            const int r = e / nn, c = e - r * nn;
            lu[mat_idx(F, i, n, nn, r, c)] = a[r * pitch + c];
        }
        for (int k = lane; k < nn; k += 32) piv[vec_idx(F, i, n, nn, k)] = sp[k];
        if (lane == 0 && info) info[i] = first_zero;
        __syncwarp();
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

int lu_factor_config(int nn, int* wpb, size_t* smem, int* grid)
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
            return pjg_internal_fail(PJG_ERR_CUDA, "device query failed");
    }
    const size_t per_warp = (size_t)nn * (nn | 1) * sizeof(double) + (size_t)nn * sizeof(int);
    int w = (int)((48u << 10) / per_warp);
    *wpb = w < 1 ? 1 : (w > 8 ? 8 : w);
    *smem = per_warp * *wpb;
    const void* fn = (const void*)lu_factor_kernel<false>;
    const void* fnF = (const void*)lu_factor_kernel<true>;
    if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem) != cudaSuccess ||
        cudaFuncSetAttribute(fnF, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem) != cudaSuccess)
        return pjg_internal_fail(PJG_ERR_CUDA, "cannot reserve shared memory for the LU kernel");
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32 * *wpb, *smem) != cudaSuccess ||
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
    int wpb = 1, grid = 1;
    size_t smem = 0;
    if (int rc = lu_factor_config(nn, &wpb, &smem, &grid)) return rc;
    const long long need = (n + wpb - 1) / wpb;
    if (need < grid) grid = (int)need;
    if (order == 'F')
        lu_factor_kernel<true><<<grid, 32 * wpb, smem, st>>>(nn, n, s, h, h0, jac, lu, piv, info, wpb);
    else
        lu_factor_kernel<false><<<grid, 32 * wpb, smem, st>>>(nn, n, s, h, h0, jac, lu, piv, info, wpb);
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
