/*
 * Host driver around the reference's shipped generated kernels
 * (pyJac-v2 examples/opencl/<mech>/{chem_utils,species_rates,jacobian}.ocl).
 *
 * Test infrastructure only (the numeric oracle and the timed CPU baseline):
 * nothing in the product links this file.  It is compiled by oracle/build_ref.sh
 * with -I pointing at the reference example directory; no reference source is
 * copied.
 *
 * Chunking mirrors the reference's lockstep OpenMP driver
 * (pyjac/core/driver_kernels.py:321-350): each OpenMP thread owns one working
 * buffer `rwk` and evaluates chunks of 128 states through the generated
 * `species_rates` / `jacobian` functions, one work item (lane) at a time.
 * Inputs/outputs use the reference's F ("state innermost") order:
 * phi[i + n * j], dphi[i + n * j], jac[i + n * p] where p is the flattened
 * Jacobian index of the shipped build (dense F order for H2/O2, CCS for GRI).
 */
#include "cl_shim.h"
#include <omp.h>
#include <vector>

namespace clshim {
thread_local int lid = 0;
thread_local int gid = 0;
thread_local int ngroups = 1;
}

#include "chem_utils.ocl"
#include "species_rates.ocl"
#include "jacobian.ocl"

#ifndef REF_RWK
#error "REF_RWK (doubles per work group of the shipped working buffer) must be defined"
#endif
#ifndef REF_JAC_SIZE
#error "REF_JAC_SIZE (Jacobian entries per state of the shipped build) must be defined"
#endif

extern "C" {

int ref_info(int* ns, int* nn, int* jac_size)
{
    *ns = NS;
    *nn = NN;
    *jac_size = REF_JAC_SIZE;
    return 0;
}

/* which: 0 = species rates (output NN per state), 1 = Jacobian (REF_JAC_SIZE) */
static int run(int which, long n, const double* P, const double* phi, double* out,
               int nthreads)
{
    if (n <= 0) return 0;
    const long nchunks = (n + 127) / 128;
    const int out_len = which == 0 ? NN : REF_JAC_SIZE;
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
    {
        std::vector<double> rwk((size_t)REF_RWK, 0.0);
        std::vector<double> P_l(128), phi_l(128 * (size_t)NN), out_l(128 * (size_t)out_len);
        clshim::gid = 0;
        clshim::ngroups = 1;
#pragma omp for schedule(dynamic, 4)
        for (long c = 0; c < nchunks; ++c) {
            const long off = c * 128;
            const int cnt = (int)((n - off) < 128 ? (n - off) : 128);
            for (int l = 0; l < 128; ++l) {
                const long s = off + (l < cnt ? l : 0);
                P_l[l] = P[s];
                for (int j = 0; j < NN; ++j) phi_l[l + 128 * j] = phi[s + n * j];
            }
            for (int l = 0; l < 128; ++l) {
                clshim::lid = l;
                if (which == 0)
                    species_rates(nullptr, P_l.data(), phi_l.data(), out_l.data(), rwk.data());
                else
                    jacobian(nullptr, P_l.data(), phi_l.data(), out_l.data(), rwk.data());
            }
            for (int l = 0; l < cnt; ++l)
                for (int p = 0; p < out_len; ++p) out[off + l + n * p] = out_l[l + 128 * p];
        }
    }
    return 0;
}

int ref_species_rates(long n, const double* P, const double* phi, double* dphi, int nthreads)
{
    return run(0, n, P, phi, dphi, nthreads);
}

int ref_jacobian(long n, const double* P, const double* phi, double* jac, int nthreads)
{
    return run(1, n, P, phi, jac, nthreads);
}

/* the shipped chem_utils kernel (eval_cp, eval_h, eval_b): cp, h and the
 * Gibbs function b of every species at T = phi[i] (guarded), F order
 * out[i + n * k] for k < NS */
int ref_chem_utils(long n, const double* phi, double* cp, double* h, double* b, int nthreads)
{
    if (n <= 0) return 0;
    const long nchunks = (n + 127) / 128;
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
    {
        std::vector<double> rwk((size_t)REF_RWK, 0.0);
        std::vector<double> phi_l(128 * (size_t)NN), cp_l(128 * (size_t)NS), h_l(128 * (size_t)NS),
            b_l(128 * (size_t)NS);
        clshim::gid = 0;
        clshim::ngroups = 1;
#pragma omp for schedule(dynamic, 4)
        for (long c = 0; c < nchunks; ++c) {
            const long off = c * 128;
            const int cnt = (int)((n - off) < 128 ? (n - off) : 128);
            for (int l = 0; l < 128; ++l) {
                const long s = off + (l < cnt ? l : 0);
                for (int j = 0; j < NN; ++j) phi_l[l + 128 * j] = phi[s + n * j];
            }
            for (int l = 0; l < 128; ++l) {
                clshim::lid = l;
                chem_utils(nullptr, b_l.data(), phi_l.data(), h_l.data(), cp_l.data(), rwk.data());
            }
            for (int l = 0; l < cnt; ++l)
                for (int k = 0; k < NS; ++k) {
                    cp[off + l + n * k] = cp_l[l + 128 * k];
                    h[off + l + n * k] = h_l[l + 128 * k];
                    b[off + l + n * k] = b_l[l + 128 * k];
                }
        }
    }
    return 0;
}

}  // extern "C"
