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

__device__ __forceinline__ float sigmoidf_(float x) { return 1.0f / (1.0f + __expf(-x)); }

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
