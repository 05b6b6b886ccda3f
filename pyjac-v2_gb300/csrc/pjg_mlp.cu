// BF16 tensor-core (tcgen05) GEMM kernels for the learned species-rate
// surrogate: an MLP whose layers are Y = act(X W^T + b) with BF16 weights and
// activations and FP32 accumulation in tensor memory.
//
// Two kernels cover forward, input-gradient (dgrad) and weight-gradient
// (wgrad) passes; both multiply K-major operands staged in shared memory in the
// no-swizzle core-matrix layout (8 rows x 16 bytes per core matrix), with one
// elected thread issuing tcgen05.mma and completion signalled through an
// mbarrier:
//
// * umma_rows_kernel: C[M x N] = A[M x K] . B[N x K]^T for a tall A (M = states)
//   and a small resident B (weights, N, K <= 256).  Persistent over 128-row tiles
//   of A; the epilogue reads the accumulator with tcgen05.ld and fuses bias,
//   SiLU, SiLU' (for dgrad), BF16 conversion, a transposed copy (the K-major
//   operand of the next wgrad) and column sums (bias gradients).
// * umma_wgrad_kernel: C[Mo x No] += A[Mo x Kb] . B[No x Kb]^T with the long
//   reduction over states split across CTAs; FP32 partial results are added to
//   the output with atomics.
//
// Waits on mbarriers are bounded; on timeout the kernel records an error
// (pjg_mlp_status) and finishes without hanging.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "pjg_umma.cuh"

namespace {

__device__ int g_umma_err = 0;

using bf16 = __nv_bfloat16;

struct RowsArgs {
    const bf16* A;
    int64_t lda;
    const bf16* B;
    int64_t ldb;
    int64_t M;
    int N, K;
    const float* bias;
    int act;           // 1: SiLU
    const bf16* zp;    // dgrad: multiply by SiLU'(zp)
    int64_t ldzp;
    bf16* Y;
    int64_t ldy;
    bf16* YT;          // transposed copy YT[n * ldyt + m]
    int64_t ldyt;
    bf16* Z;           // pre-activation copy
    int64_t ldz;
    float* Y32;        // FP32 output
    int64_t ldy32;
    float* colsum;     // += column sums of the output
};

// logistic sigmoid with the fast division intrinsic (2 ulp in FP32; results are
// rounded to BF16), shared by every kernel so that training and inference
// evaluate SiLU identically
// sigmoid(x) = (1 + tanh(x / 2)) / 2 with the hardware tanh (tanh.approx.f32,
// relative error about 2^-11, below the BF16 rounding the activations take):
// one special-function operation instead of an exponential and a reciprocal,
// which bound the epilogues (16 special-function results per clock per SM)
__device__ __forceinline__ float tanh_approx(float x)
{
    float y;
    asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float sigmoidf_(float x) { return fmaf(0.5f, tanh_approx(0.5f * x), 0.5f); }

__global__ void __launch_bounds__(128, 1) umma_rows_kernel(const RowsArgs g)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_s;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int kc = g.K >> 3;  // 16-byte chunks per row
    uint8_t* sB = smem;
    uint8_t* sA = smem + (size_t)g.N * g.K * 2;
    const uint32_t ncols = g.N <= 32 ? 32u : (g.N <= 64 ? 64u : (g.N <= 128 ? 128u : 256u));
    if (warp == 0) {
        umma::tmem_alloc(&tmem_s, ncols);
        umma::tmem_relinquish();
    }
    if (tid == 0) umma::mbar_init(&mbar, 1);
    for (int idx = tid; idx < g.N * kc; idx += 128) {
        const int n = idx / kc, c = idx - n * kc;
        umma::cp_async16(sB + ((size_t)(n >> 3) * kc + c) * 128 + (n & 7) * 16, g.B + (int64_t)n * g.ldb + c * 8, 16);
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tmem_s;
    const uint32_t idesc = umma::idesc_bf16(128, g.N);
    const uint32_t sAu = umma::smem_u32(sA), sBu = umma::smem_u32(sB);
    const uint32_t sbo = (uint32_t)kc * 128;
    uint32_t phase = 0;
    const int64_t ntiles = (g.M + 127) / 128;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t row0 = t * 128;
        for (int idx = tid; idx < 128 * kc; idx += 128) {
            const int r = idx / kc, c = idx - r * kc;
            const int64_t grow = row0 + r;
            const bool ok = grow < g.M;
            umma::cp_async16(sA + ((size_t)(r >> 3) * kc + c) * 128 + (r & 7) * 16,
                             g.A + (ok ? grow : 0) * g.lda + c * 8, ok ? 16u : 0u);
        }
        umma::cp_async_wait_all();
        umma::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            umma::fence_after();
            for (int ks = 0; ks < (g.K >> 4); ++ks) {
                const uint64_t ad = umma::sdesc(sAu + ks * 256, 128, sbo);
                const uint64_t bd = umma::sdesc(sBu + ks * 256, 128, sbo);
                umma::mma_bf16(tmem, ad, bd, idesc, ks > 0 ? 1u : 0u);
            }
            umma::mma_commit(&mbar);
        }
        if (!umma::mbar_wait(&mbar, phase) && lane == 0) atomicExch(&g_umma_err, 1);
        phase ^= 1;
        umma::fence_after();
        const int m = warp * 32 + lane;
        const int64_t grow = row0 + m;
        const bool ok = grow < g.M;
        for (int c0 = 0; c0 < g.N; c0 += 32) {
            float v[32];
            umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            alignas(16) bf16 yb[32];
            alignas(16) bf16 zb[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int n = c0 + j;
                float x = v[j];
                if (g.bias) x += __ldg(g.bias + n);
                zb[j] = __float2bfloat16(x);
                if (g.zp) {
                    const float z = ok ? __bfloat162float(g.zp[grow * g.ldzp + n]) : 0.0f;
                    const float sg = sigmoidf_(z);
                    x *= sg * (1.0f + z * (1.0f - sg));
                }
                const float y = g.act ? x * sigmoidf_(x) : x;
                v[j] = y;
                yb[j] = __float2bfloat16(y);
            }
            if (ok) {
                if (g.Y) {
                    uint4* d = reinterpret_cast<uint4*>(g.Y + grow * g.ldy + c0);
                    const uint4* s = reinterpret_cast<const uint4*>(yb);
#pragma unroll
                    for (int q = 0; q < 4; ++q) d[q] = s[q];
                }
                if (g.Z) {
                    uint4* d = reinterpret_cast<uint4*>(g.Z + grow * g.ldz + c0);
                    const uint4* s = reinterpret_cast<const uint4*>(zb);
#pragma unroll
                    for (int q = 0; q < 4; ++q) d[q] = s[q];
                }
                if (g.YT) {
#pragma unroll
                    for (int j = 0; j < 32; ++j) g.YT[(int64_t)(c0 + j) * g.ldyt + grow] = yb[j];
                }
                if (g.Y32) {
                    float4* d = reinterpret_cast<float4*>(g.Y32 + grow * g.ldy32 + c0);
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        d[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
                }
            }
            if (g.colsum) {
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    float sv = ok ? v[j] : 0.0f;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) sv += __shfl_xor_sync(0xffffffffu, sv, o);
                    if (lane == 0) atomicAdd(g.colsum + c0 + j, sv);
                }
            }
        }
        umma::fence_before();
        __syncthreads();
    }
    umma::fence_after();
    __syncthreads();
    if (warp == 0) umma::tmem_dealloc(tmem, ncols);
}

struct WgradArgs {
    const bf16* A;   // [Mo x Kb], Kb contiguous
    int64_t lda;
    const bf16* B;   // [No x Kb]
    int64_t ldb;
    int Mo, No;
    int64_t Kb, kchunk;
    float* C;        // [Mo x No] += A B^T
    int64_t ldc;
};

constexpr int WK = 64;  // reduction block staged per step

__global__ void __launch_bounds__(128, 1) umma_wgrad_kernel(const WgradArgs g)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t mbar;
    __shared__ uint32_t tmem_s;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    constexpr int kc = WK / 8;
    uint8_t* sA = smem;                       // 128 x WK
    uint8_t* sB = smem + 128 * WK * 2;        // No x WK
    const uint32_t ncols = g.No <= 32 ? 32u : (g.No <= 64 ? 64u : (g.No <= 128 ? 128u : 256u));
    if (warp == 0) {
        umma::tmem_alloc(&tmem_s, ncols);
        umma::tmem_relinquish();
    }
    if (tid == 0) umma::mbar_init(&mbar, 1);
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tmem_s;
    const uint32_t idesc = umma::idesc_bf16(128, g.No);
    const uint32_t sAu = umma::smem_u32(sA), sBu = umma::smem_u32(sB);
    const int mrow0 = blockIdx.x * 128;
    const int64_t k0 = (int64_t)blockIdx.y * g.kchunk;
    const int64_t k1 = k0 + g.kchunk < g.Kb ? k0 + g.kchunk : g.Kb;
    uint32_t phase = 0;
    bool first = true;
    for (int64_t kb = k0; kb < k1; kb += WK) {
        for (int idx = tid; idx < 128 * kc; idx += 128) {
            const int r = idx / kc, c = idx - r * kc;
            const bool ok = mrow0 + r < g.Mo;
            umma::cp_async16(sA + ((size_t)(r >> 3) * kc + c) * 128 + (r & 7) * 16,
                             g.A + (int64_t)(ok ? mrow0 + r : 0) * g.lda + kb + c * 8, ok ? 16u : 0u);
        }
        for (int idx = tid; idx < g.No * kc; idx += 128) {
            const int n = idx / kc, c = idx - n * kc;
            umma::cp_async16(sB + ((size_t)(n >> 3) * kc + c) * 128 + (n & 7) * 16,
                             g.B + (int64_t)n * g.ldb + kb + c * 8, 16u);
        }
        umma::cp_async_wait_all();
        umma::fence_proxy_async();
        __syncthreads();
        if (tid == 0) {
            umma::fence_after();
#pragma unroll
            for (int ks = 0; ks < WK / 16; ++ks) {
                const uint64_t ad = umma::sdesc(sAu + ks * 256, 128, kc * 128);
                const uint64_t bd = umma::sdesc(sBu + ks * 256, 128, kc * 128);
                umma::mma_bf16(tmem, ad, bd, idesc, (first && ks == 0) ? 0u : 1u);
            }
            umma::mma_commit(&mbar);
        }
        first = false;
        if (!umma::mbar_wait(&mbar, phase) && lane == 0) atomicExch(&g_umma_err, 1);
        phase ^= 1;
        umma::fence_after();
        __syncthreads();
    }
    if (k1 > k0) {
        const int m = mrow0 + warp * 32 + lane;
        for (int c0 = 0; c0 < g.No; c0 += 32) {
            float v[32];
            umma::tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            if (m < g.Mo)
                for (int j = 0; j < 32; ++j) atomicAdd(g.C + (int64_t)m * g.ldc + c0 + j, v[j]);
        }
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    if (warp == 0) umma::tmem_dealloc(tmem, ncols);
}


// ---------------------------------------------------------------------------
// Fused forward pass of the whole network, 64 -> 256 -> 256 -> 256 -> 256 -> 64
// (SiLU on the hidden layers), for inference.  A persistent CTA takes 128-row
// tiles; a tile's activations stay in shared memory from layer to layer (the
// epilogue of layer l writes the BF16 A operand of layer l + 1), so only the
// features are read from and the FP32 outputs written to global memory.  The
// weights stream from L2 through a two-slot ring of 64 KB: each chunk (W0,
// each 128-row half of W1..W3, W4) is pre-packed in the no-swizzle core-matrix
// layout, so one 1-D bulk copy moves it, completing on the slot's mbarrier.
// Thread 0 issues the copies and the MMAs; the copies of the next layer's
// weights run while 16 warps (four per TMEM lane quarter, each a quarter of
// the columns) read the accumulator from TMEM and apply bias and SiLU.
struct FusedArgs {
    const bf16* X;       // [M x 64] features
    int64_t ldx, M;
    const uint8_t* W[5]; // packed weights: 256x64, 256x256 (x3), 64x256
    const float* b[5];
    float* Y;            // [M x 64] outputs
    int64_t ldy;
};

constexpr uint32_t FUSED_SLOT = 64 * 1024;
constexpr size_t FUSED_SMEM = 3 * (size_t)FUSED_SLOT;  // activation tile + two weight slots

__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b)
{
    const uint32_t lo = __bfloat16_as_ushort(__float2bfloat16(a));
    const uint32_t hi = __bfloat16_as_ushort(__float2bfloat16(b));
    return lo | (hi << 16);
}

// SiLU of the fused inference epilogue, the same expression as the layer kernels'
__device__ __forceinline__ float silu_fast(float x) { return x * sigmoidf_(x); }

constexpr int FUSED_THREADS = 512;  // 16 warps: four per TMEM lane quarter, each a quarter of the columns

__global__ void __launch_bounds__(FUSED_THREADS, 1) mlp_fused_kernel(const FusedArgs g)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ uint64_t full[2];
    __shared__ uint64_t mmab;
    __shared__ uint32_t tmem_s;
    __shared__ int s_abort;
    __shared__ float sbias[4 * 256 + 64];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int quarter = warp & 3, part = warp >> 2;  // TMEM lanes 32 * quarter.., column quarter
    uint8_t* sA = smem;
    uint8_t* sW[2] = {smem + FUSED_SLOT, smem + 2 * FUSED_SLOT};
    if (warp == 0) {
        umma::tmem_alloc(&tmem_s, 256);
        umma::tmem_relinquish();
    }
    if (tid == 0) {
        umma::mbar_init(&full[0], 1);
        umma::mbar_init(&full[1], 1);
        umma::mbar_init(&mmab, 1);
        s_abort = 0;
    }
    for (int i = tid; i < 4 * 256 + 64; i += FUSED_THREADS)
        sbias[i] = i < 1024 ? __ldg(g.b[i >> 8] + (i & 255)) : __ldg(g.b[4] + (i - 1024));
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    const uint32_t tmem = tmem_s;
    const uint32_t sAu = umma::smem_u32(sA);
    const uint32_t sWu[2] = {umma::smem_u32(sW[0]), umma::smem_u32(sW[1])};
    // thread 0's copy bookkeeping: expected parity and copies in flight per slot
    uint32_t fphase[2] = {0u, 0u}, mphase = 0u;
    bool pending[2] = {false, false};
    bool mma_late = false;  // an MMA whose completion wait ran out
    auto issue = [&](int slot, const uint8_t* src, uint32_t bytes) {
        umma::mbar_expect_tx(&full[slot], bytes);
        umma::bulk_g2s(sW[slot], src, bytes, &full[slot]);
        pending[slot] = true;
    };
    auto take = [&](int slot) -> bool {
        const bool ok = umma::mbar_wait(&full[slot], fphase[slot]);
        fphase[slot] ^= 1u;
        pending[slot] = false;
        return ok;
    };
    const int64_t ntiles = (g.M + 127) / 128;
    if (tid == 0 && blockIdx.x < ntiles) {
        issue(0, g.W[0], 32 * 1024);
        issue(1, g.W[1], FUSED_SLOT);
    }
    bool aborted = false;
    for (int64_t t = blockIdx.x; t < ntiles && !aborted; t += gridDim.x) {
        const int64_t row0 = t * 128;
        const bool more = t + gridDim.x < ntiles;
        // features -> A operand of layer 0 (K = 64: 8 chunks of 16 bytes per row)
        for (int idx = tid; idx < 128 * 8; idx += FUSED_THREADS) {
            const int r = idx >> 3, c = idx & 7;
            const int64_t grow = row0 + r;
            const bool ok = grow < g.M;
            umma::cp_async16(sA + ((size_t)(r >> 3) * 8 + c) * 128 + (r & 7) * 16,
                             g.X + (ok ? grow : 0) * g.ldx + c * 8, ok ? 16u : 0u);
        }
        umma::cp_async_wait_all();
        umma::fence_proxy_async();
        __syncthreads();
        for (int l = 0; l < 5; ++l) {
            if (tid == 0) {
                umma::fence_after();
                bool ok = true;
                if (l == 0) {
                    ok = take(0);
                    const uint32_t id = umma::idesc_bf16(128, 256);
                    for (int ks = 0; ks < 4; ++ks)
                        umma::mma_bf16(tmem, umma::sdesc(sAu + ks * 256, 128, 8 * 128),
                                       umma::sdesc(sWu[0] + ks * 256, 128, 8 * 128), id, ks ? 1u : 0u);
                } else if (l < 4) {
                    ok = take(1) & take(0);
                    const uint32_t id = umma::idesc_bf16(128, 128);
                    for (int h = 0; h < 2; ++h)  // half 0 (rows 0..127 of W) in slot 1, half 1 in slot 0
                        for (int ks = 0; ks < 16; ++ks)
                            umma::mma_bf16(tmem + 128u * h, umma::sdesc(sAu + ks * 256, 128, 32 * 128),
                                           umma::sdesc(sWu[1 - h] + ks * 256, 128, 32 * 128), id,
                                           ks ? 1u : 0u);
                } else {
                    ok = take(1);
                    const uint32_t id = umma::idesc_bf16(128, 64);
                    for (int ks = 0; ks < 16; ++ks)
                        umma::mma_bf16(tmem, umma::sdesc(sAu + ks * 256, 128, 32 * 128),
                                       umma::sdesc(sWu[1] + ks * 256, 128, 32 * 128), id, ks ? 1u : 0u);
                }
                umma::mma_commit(&mmab);
                if (!ok) s_abort = 1;
            }
            const bool mok = umma::mbar_wait(&mmab, mphase);
            if (!mok) {
                if (lane == 0) s_abort = 1;
                if (tid == 0) mma_late = true;
            } else {
                mphase ^= 1u;
            }
            umma::fence_after();
            if (tid == 0) {
                // the weights of the next layer (or the next tile's first layers)
                if (l == 0) {
                    issue(0, g.W[1] + FUSED_SLOT, FUSED_SLOT);
                } else if (l < 3) {
                    issue(1, g.W[l + 1], FUSED_SLOT);
                    issue(0, g.W[l + 1] + FUSED_SLOT, FUSED_SLOT);
                } else if (l == 3) {
                    issue(1, g.W[4], 32 * 1024);
                    if (more) issue(0, g.W[0], 32 * 1024);
                } else if (more) {
                    issue(1, g.W[1], FUSED_SLOT);
                }
            }
            const int m = quarter * 32 + lane;
            const int64_t grow = row0 + m;
            const uint32_t trow = tmem + ((uint32_t)(quarter * 32) << 16);
            if (l < 4) {
                const float* bias = sbias + 256 * l;
                for (int c0 = 64 * part; c0 < 64 * part + 64; c0 += 32) {
                    float v[32];
                    umma::tmem_ld32(trow + (uint32_t)c0, v);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        uint32_t w[4];
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            w[e] = pack_bf16x2(silu_fast(v[8 * q + 2 * e] + bias[c0 + 8 * q + 2 * e]),
                                               silu_fast(v[8 * q + 2 * e + 1] + bias[c0 + 8 * q + 2 * e + 1]));
                        const int c = (c0 >> 3) + q;
                        *reinterpret_cast<uint4*>(sA + ((size_t)(m >> 3) * 32 + c) * 128 + (m & 7) * 16) =
                            make_uint4(w[0], w[1], w[2], w[3]);
                    }
                }
            } else if (part < 2) {
                const float* bias = sbias + 1024;
                const int c0 = 32 * part;
                float v[32];
                umma::tmem_ld32(trow + (uint32_t)c0, v);
                if (grow < g.M) {
                    float4* d = reinterpret_cast<float4*>(g.Y + grow * g.ldy + c0);
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        d[q] = make_float4(v[4 * q] + bias[c0 + 4 * q], v[4 * q + 1] + bias[c0 + 4 * q + 1],
                                           v[4 * q + 2] + bias[c0 + 4 * q + 2],
                                           v[4 * q + 3] + bias[c0 + 4 * q + 3]);
                }
            }
            umma::fence_before();
            umma::fence_proxy_async();
            __syncthreads();
            if (s_abort) {
                aborted = true;
                break;
            }
        }
    }
    if (tid == 0) {
        if (aborted) atomicExch(&g_umma_err, 1);
        // no copy or MMA may still be writing this CTA's memory when it exits
        for (int slot = 0; slot < 2; ++slot)
            if (pending[slot]) take(slot);
        if (mma_late) umma::mbar_wait(&mmab, mphase);
    }
    umma::fence_before();
    __syncthreads();
    umma::fence_after();
    if (warp == 0) umma::tmem_dealloc(tmem, 256);
}

// ---------------------------------------------------------------------------
// Surrogate input and output stages (thread per state, C-order states).
//
// Features: X[s] = BF16 of ((T - 1500) / 400, (ln P - mu_P) / sd_P,
// (log10 max(c_k, floor) - mu_k) / sd_k for the ns - 1 species, 0 ...) with
// c_k = max(n_k, 0) / V; logarithms in FP32 (the features are BF16).
__global__ void surr_features_kernel(int64_t n, int nn, const double* __restrict__ phi,
                                     const double* __restrict__ param, const double* __restrict__ st,
                                     bf16* X, float floor_c)
{
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const double* p = phi + s * nn;
    const float inv_v = (float)(1.0 / p[1]);  // one FP64 division per state; the rest is FP32
    // st: lnP_mu, lnP_sd, lc_mu[nn - 2], lc_sd[nn - 2]
    alignas(16) bf16 f[64];
    f[0] = __float2bfloat16((float)(p[0] - 1500.0) * 0.0025f);
    f[1] = __float2bfloat16((float)((log(param[s]) - st[0]) / st[1]));
    const int nsp = nn - 2;
    for (int k = 0; k < nsp; ++k) {
        const float c = fmaxf((float)p[2 + k], 0.0f) * inv_v;
        const float lc = log10f(fmaxf(c, floor_c));
        f[2 + k] = __float2bfloat16(__fdividef(lc - (float)st[2 + k], (float)st[2 + nsp + k]));
    }
    for (int k = nn; k < 64; ++k) f[k] = __float2bfloat16(0.0f);
    uint4* d = reinterpret_cast<uint4*>(X + s * 64);
    const uint4* src = reinterpret_cast<const uint4*>(f);
#pragma unroll
    for (int q = 0; q < 8; ++q) d[q] = src[q];
}

// Outputs: y_j = sinh(Y[s][j] z_sd_j + z_mu_j) s_j (FP32 transcendental, FP64
// result) for the 53 rates {dT/dt, dn_k/dt}; dphi = (Tdot, extra-variable rate
// recomputed as the FP64 path does, the ndot_k); lerr[s] = Y[s][err_col].
__global__ void surr_outputs_kernel(int64_t n, int nn, const float* __restrict__ Y,
                                    const double* __restrict__ phi,
                                    const double* __restrict__ param,
                                    const double* __restrict__ st, int err_col,
                                    double* __restrict__ dphi, float* __restrict__ lerr)
{
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const int nout = nn - 1;                       // Tdot + (nn - 2) species rates
    const double* zmu = st;
    const double* zsd = st + nout;
    const double* sc = st + 2 * nout;
    const double* omw = st + 3 * nout;             // 1 - W_k / W_ns, nn - 2 values
    const float* y = Y + s * 64;
    const double* p = phi + s * nn;
    double* o = dphi + s * nn;
    const double T = fmin(10000.0, fmax(100.0, p[0]));
    const double V = fmax(p[1], 1e-30);
    const double P = param[s];
    double dE = 0.0;  // sum_k (1 - W_k / W_ns) ndot_k; divided by V once below
    for (int j = 0; j < nout; ++j) {
        const float z = fmaf(y[j], (float)zsd[j], (float)zmu[j]);
        const double v = (double)sinhf(z) * sc[j];
        if (j == 0) {
            o[0] = v;
        } else {
            o[1 + j] = v;
            dE = fma(v, omw[j - 1], dE);
        }
    }
    o[1] = V * o[0] / T + dE * T * 8314.4621 / P;
    lerr[s] = y[err_col];
}

int sm_count()
{
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        if (n <= 0) n = 1;
    }
    return n;
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15) == 0; }

}  // namespace

// launchers (declared in pjg_mlp.cuh-free form: used only by pjg_capi.cu)
int mlp_launch_rows(const void* A, int64_t lda, const void* B, int64_t ldb, int64_t M, int N, int K,
                 const float* bias, int act, const void* zp, int64_t ldzp, void* Y, int64_t ldy,
                 void* YT, int64_t ldyt, void* Z, int64_t ldz, float* Y32, int64_t ldy32,
                 float* colsum, void* stream)
{
    if (M <= 0) return 0;
    if (N < 32 || N > 256 || N % 32 || K < 16 || K > 256 || K % 16 || !A || !B) return -1;
    if (lda % 8 || ldb % 8 || !aligned16(A) || !aligned16(B)) return -1;
    if ((Y && (ldy % 8 || !aligned16(Y))) || (Z && (ldz % 8 || !aligned16(Z))) ||
        (Y32 && (ldy32 % 4 || !aligned16(Y32))))
        return -1;
    RowsArgs g;
    g.A = (const bf16*)A; g.lda = lda; g.B = (const bf16*)B; g.ldb = ldb;
    g.M = M; g.N = N; g.K = K; g.bias = bias; g.act = act;
    g.zp = (const bf16*)zp; g.ldzp = ldzp;
    g.Y = (bf16*)Y; g.ldy = ldy; g.YT = (bf16*)YT; g.ldyt = ldyt; g.Z = (bf16*)Z; g.ldz = ldz;
    g.Y32 = Y32; g.ldy32 = ldy32; g.colsum = colsum;
    const size_t smem = (size_t)(N + 128) * K * 2;
    cudaFuncSetAttribute(umma_rows_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    const int64_t ntiles = (M + 127) / 128;
    const int grid = (int)(ntiles < sm_count() ? ntiles : sm_count());
    umma_rows_kernel<<<grid, 128, smem, (cudaStream_t)stream>>>(g);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int mlp_launch_wgrad(const void* A, int64_t lda, const void* B, int64_t ldb, int Mo, int No, int64_t Kb,
                  float* C, int64_t ldc, void* stream)
{
    if (Kb <= 0) return 0;
    if (No < 32 || No > 256 || No % 32 || Mo <= 0 || Kb % WK || !A || !B || !C) return -1;
    if (lda % 8 || ldb % 8 || !aligned16(A) || !aligned16(B)) return -1;
    WgradArgs g;
    g.A = (const bf16*)A; g.lda = lda; g.B = (const bf16*)B; g.ldb = ldb;
    g.Mo = Mo; g.No = No; g.Kb = Kb; g.C = C; g.ldc = ldc;
    const int mt = (Mo + 127) / 128;
    int splits = (sm_count() + mt - 1) / mt;
    int64_t chunk = (Kb + splits - 1) / splits;
    chunk = (chunk + WK - 1) / WK * WK;
    splits = (int)((Kb + chunk - 1) / chunk);
    g.kchunk = chunk;
    const size_t smem = (size_t)(128 + No) * WK * 2;
    cudaFuncSetAttribute(umma_wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    umma_wgrad_kernel<<<dim3(mt, splits), 128, smem, (cudaStream_t)stream>>>(g);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int mlp_launch_fused(const void* X, int64_t ldx, int64_t M, const void* const* W,
                     const float* const* b, float* Y, int64_t ldy, void* stream)
{
    if (M <= 0) return 0;
    if (!X || !Y || ldx % 8 || ldy % 4 || ldx < 64 || ldy < 64 || !aligned16(X) || !aligned16(Y))
        return -1;
    FusedArgs g;
    g.X = (const bf16*)X;
    g.ldx = ldx;
    g.M = M;
    for (int l = 0; l < 5; ++l) {
        if (!W[l] || !b[l] || !aligned16(W[l])) return -1;
        g.W[l] = (const uint8_t*)W[l];
        g.b[l] = b[l];
    }
    g.Y = Y;
    g.ldy = ldy;
    cudaFuncSetAttribute(mlp_fused_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FUSED_SMEM);
    const int64_t ntiles = (M + 127) / 128;
    const int grid = (int)(ntiles < sm_count() ? ntiles : sm_count());
    mlp_fused_kernel<<<grid, FUSED_THREADS, FUSED_SMEM, (cudaStream_t)stream>>>(g);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int surr_launch_features(int64_t n, int nn, const double* phi, const double* param,
                         const double* st, void* X, float floor_c, void* stream)
{
    if (n <= 0) return 0;
    if (nn > 64 || nn < 3 || !aligned16(X)) return -1;
    surr_features_kernel<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
        n, nn, phi, param, st, (bf16*)X, floor_c);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int surr_launch_outputs(int64_t n, int nn, const float* Y, const double* phi, const double* param,
                        const double* st, int err_col, double* dphi, float* lerr, void* stream)
{
    if (n <= 0) return 0;
    if (nn > 65 || nn < 3 || err_col < 0 || err_col >= 64) return -1;
    surr_outputs_kernel<<<(unsigned)((n + 127) / 128), 128, 0, (cudaStream_t)stream>>>(
        n, nn, Y, phi, param, st, err_col, dphi, lerr);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int mlp_error_flag(int clear)
{
    int h = 0;
    cudaMemcpyFromSymbol(&h, g_umma_err, sizeof(int));
    if (clear) {
        const int z = 0;
        cudaMemcpyToSymbol(g_umma_err, &z, sizeof(int));
    }
    return h;
}
