// pjg_vjp_noalloc: the J^T v evaluation without any device allocation.
//
// Some callers cannot let a library allocate device memory at call time:
// CFD and reacting-flow solvers that call the chemistry once per cell
// batch and time step from a hot loop (cudaMalloc and cudaFree can
// synchronise the whole device and stall every other stream), codes that
// must not fail for out-of-memory half-way through a simulation, and hosts
// that hand every byte of the GPU to their own pool allocator.  pjg_vjp may
// grow the mechanism's working buffer with cudaMalloc; this entry point
// instead uses a fixed scratch array that lives in this file for the life of
// the process, and calls no cudaMalloc, cudaFree or allocating library
// routine.
//
// The scratch array is kScratchDoubles doubles (16 MiB) on every device that
// loads the library, held until the process exits.  It holds the kernel's
// per-state working arrays (10 * Ns doubles per state, 4,240 bytes for
// GRI-Mech 3.0), so one launch covers up to floor(16 MiB / (80 Ns bytes))
// states rounded down to a multiple of 128 (3,840 for GRI-Mech 3.0); larger
// problems run as several launches in order on the caller's stream.  A
// mechanism whose 128-state block does not fit (more than 1,638 species) is
// rejected with PJG_ERR_ARG.
//
// Set-up: the first call on each device, with that device current, takes the
// array's device address with cudaGetSymbolAddress (a host-side name of a
// __device__ array is not a device address).  That first call should come
// before any stream capture on the device.
//
// Every call shares the one array, which keeps the contents the last call
// left there.  The kernel writes every scratch element before it reads it, so
// nothing needs clearing between calls, but calls that overlap on the GPU
// (for example on two streams) race on the array and must be serialised by
// the caller.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <mutex>

#include "../../include/pyjac_gb300.h"
#include "pjg_eval.cuh"

int pjg_internal_fail(int code, const char* msg);
void pjg_internal_fill_args(const pjg_mech* m, EvalArgs* a);
int pjg_internal_mech_ns(const pjg_mech* m);
int pjg_internal_check_device(const pjg_mech* m);
void pjg_internal_count_launch();

namespace {

constexpr size_t kScratchDoubles = size_t(2) << 20;  // 16 MiB
static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

constexpr int kMaxDevices = 64;
double* g_scratch_addr[kMaxDevices] = {};
std::mutex g_setup_mu;

int scratch_for_current_device(double** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return pjg_internal_fail(PJG_ERR_CUDA, "cudaGetDevice failed");
    if (dev < 0 || dev >= kMaxDevices) return pjg_internal_fail(PJG_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> g(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        double* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress((void**)&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            char msg[256];
            snprintf(msg, sizeof(msg), "cudaGetSymbolAddress of the no-alloc scratch failed: %s",
                     cudaGetErrorString(e));
            return pjg_internal_fail(PJG_ERR_CUDA, msg);
        }
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return 0;
}

}  // namespace

extern "C" int pjg_vjp_noalloc(pjg_mech* mech, int64_t n, char order, int conp, const double* param,
                               const double* phi, const double* v, double* out, void* stream)
{
    if (!mech) return pjg_internal_fail(PJG_ERR_ARG, "null mechanism");
    if (n < 0) return pjg_internal_fail(PJG_ERR_ARG, "negative problem size");
    if (order != 'C' && order != 'F') return pjg_internal_fail(PJG_ERR_ARG, "order must be 'C' or 'F'");
    if (n == 0) return 0;
    if (!param || !phi || !v || !out) return pjg_internal_fail(PJG_ERR_ARG, "null array");
    const int ns = pjg_internal_mech_ns(mech);
    const size_t per_state = (size_t)ARR_N_JAC * ns;  // doubles
    int64_t chunk = (int64_t)(kScratchDoubles / per_state) / PJG_BLOCK * PJG_BLOCK;
    if (chunk < PJG_BLOCK) {
        char msg[256];
        snprintf(msg, sizeof(msg),
                 "pjg_vjp_noalloc: %d species need %zu bytes of scratch per 128 states, more than "
                 "the fixed %zu-byte array", ns, per_state * 8 * PJG_BLOCK, kScratchDoubles * 8);
        return pjg_internal_fail(PJG_ERR_ARG, msg);
    }
    // the scratch address below is the current device's: the mechanism's
    // tables must live there too
    int rc = pjg_internal_check_device(mech);
    if (rc) return rc;
    double* scratch = nullptr;
    rc = scratch_for_current_device(&scratch);
    if (rc) return rc;
    if (chunk > n) chunk = n;
    const bool F = order == 'F';
    const int NN = ns + 1;
    for (int64_t off = 0; off < n; off += chunk) {
        const int64_t cnt = n - off < chunk ? n - off : chunk;
        EvalArgs a;
        pjg_internal_fill_args(mech, &a);
        a.n = cnt;
        a.conp = conp;
        a.param = param + off;
        if (F) {
            a.phi = phi + off;
            a.phi_ss = 1;
            a.phi_sj = n;
            a.v = v + off;
            a.vjp = out + off;
        } else {
            a.phi = phi + off * NN;
            a.phi_ss = NN;
            a.phi_sj = 1;
            a.v = v + off * NN;
            a.vjp = out + off * NN;
        }
        a.scratch = scratch;
        a.sc_ld = chunk;
        rc = pjg_launch_eval(a, 2, stream);
        if (rc) {
            char msg[256];
            snprintf(msg, sizeof(msg), "pjg_vjp_noalloc: kernel launch failed: %s",
                     pjg_launch_error_string());
            return pjg_internal_fail(PJG_ERR_CUDA, msg);
        }
        pjg_internal_count_launch();
    }
    return 0;
}
