/*
 * pyjac-v2_gb300 C ABI: batched species rates and analytical Jacobians of a
 * chemical-kinetic mechanism on one GB300 (sm_103a), FP64 throughout.
 *
 * This ABI replaces the runtime boundary of pyJac-v2's generated code:
 *   - the generated C++ kernel class (pyjac/kernel_utils/common/kernel.hpp.in:86-335,
 *     kernel.cpp.in:539-633): Kernel(problem_size, work_size, do_not_compile),
 *     resize(), operator()(double* param, double* phi, double* out),
 *     requiredMemorySize(), numSpecies(), numReactions(), order();
 *   - the generated device entry points species_rates(t, P_arr, phi, dphi, rwk)
 *     and jacobian(t, P_arr, phi, jac, rwk)
 *     (examples/opencl/ch4/species_rates.ocl:354, jacobian.ocl:1130) and their
 *     lockstep drivers (pyjac/core/driver_kernels.py:321-367);
 *   - the Cython wrapper's arrays, passed as &arr[0]
 *     (pyjac/pywrap/pyjacob_wrapper.pyx.in:19-92).
 *
 * Data conventions are pyJac's (pyjac/core/array_creator.py:1938-2110):
 *   phi  = (T, V or P, n_0 .. n_{Ns-2}) per state, NN = Ns + 1 entries;
 *   param = P (constant pressure, conp) or V (constant volume);
 *   dphi = d phi / dt;
 *   order 'C': phi[i*NN + j], dense jac[i*NN*NN + row*NN + col],
 *              sparse jac[i*nnz + p] in CRS order;
 *   order 'F': phi[i + N*j],  dense jac[i + N*row + N*NN*col],
 *              sparse jac[i + N*p] in CCS order.
 *
 * Every function returns 0 on success and a negative pjg_status on error; none
 * aborts.  pjg_last_error() returns a thread-local description of the last
 * error.  Functions taking a `stream` are asynchronous on that CUDA stream
 * (cudaStream_t passed as void*; NULL = legacy default stream) and take
 * device pointers; pjg_kernel_call takes host pointers and is synchronous,
 * as the reference's operator() is.
 */
#ifndef PYJAC_GB300_H
#define PYJAC_GB300_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum pjg_status {
    PJG_OK = 0,
    PJG_ERR_ARG = -1,        /* invalid argument (null pointer, bad size, bad enum) */
    PJG_ERR_CUDA = -2,       /* a CUDA runtime call failed */
    PJG_ERR_TABLES = -3,     /* inconsistent or unsupported mechanism tables */
    PJG_ERR_UNSUPPORTED = -4 /* option combination not supported */
};

enum pjg_kind { PJG_SPECIES_RATES = 0, PJG_JACOBIAN = 1 };
enum pjg_jac_format { PJG_JAC_FULL = 0, PJG_JAC_SPARSE = 1 };

/* Host-side mechanism tables produced by the Python front end
 * (pyjac-v2_gb300/pack.py).  All arrays are read during pjg_mech_create and
 * may be freed afterwards.  Byte layouts are documented in
 * pyjac-v2_gb300/csrc/pjg_tables.cuh. */
typedef struct pjg_tables {
    int32_t ns;              /* species, bath gas last */
    int32_t nr;              /* reactions */
    int32_t flags;           /* bit 0: mechanism has PLOG/Chebyshev (needs ln P);
                              * bit 1: the 'approximate' Jacobian type, which omits
                              * the bath-gas terms d n_Ns / d n_j of the species
                              * columns (create_jacobian.py:186-190, :3578-3582,
                              * :4187-4191); the pattern arrays must be the
                              * approximate type's */
    const void* rxn;         /* nr reaction records, 192 bytes each */
    const double* species;   /* ns species records, 48 doubles each (PJG_SP_DOUBLES) */
    const int32_t* thd_spec; /* third-body species lists */
    const double* thd_coef;  /* efficiency minus flag, aligned with thd_spec */
    int32_t n_thd;           /* length of thd_spec / thd_coef */
    const double* aux;       /* PLOG / Chebyshev parameter blocks */
    int32_t n_aux;           /* length of aux in doubles */
    /* Jacobian non-zero pattern (create_jacobian.py:235-282) */
    int32_t nnz;
    const int32_t* crs_row_ptr;  /* NN + 1 */
    const int32_t* crs_col_ind;  /* nnz */
    const int32_t* ccs_col_ptr;  /* NN + 1 */
    const int32_t* ccs_row_ind;  /* nnz */
} pjg_tables;

typedef struct pjg_mech pjg_mech;
typedef struct pjg_kernel pjg_kernel;

/* Upload tables to the current CUDA device. */
int pjg_mech_create(const pjg_tables* tables, pjg_mech** out);
int pjg_mech_destroy(pjg_mech* mech);
/* numSpecies() / numReactions() of kernel.hpp.in */
int pjg_mech_info(const pjg_mech* mech, int32_t* ns, int32_t* nr, int32_t* nnz);

/* Jacobian index arrays of kernel order: CRS (row_ptr, col_ind) for 'C',
 * CCS (col_ptr, row_ind) for 'F' (create_jacobian.py:235-282).  ptr has NN+1
 * entries, ind has nnz; either may be NULL to query only *nnz. */
int pjg_jacobian_indices(const pjg_mech* mech, char order, int32_t* ptr, int32_t* ind,
                         int32_t* nnz);

/* Device-pointer entry points (asynchronous on `stream`).
 * Replace the generated species_rates / jacobian drivers.  Calls on one
 * mechanism share its device working buffer (grown on demand): calls that
 * can overlap on the GPU, on different streams, must be serialised by the
 * caller or use separate pjg_mech objects. */
int pjg_species_rates(pjg_mech* mech, int64_t n, char order, int conp, const double* param,
                      const double* phi, double* dphi, void* stream);
int pjg_jacobian(pjg_mech* mech, int64_t n, char order, int conp, int jac_format,
                 const double* param, const double* phi, double* jac, void* stream);
/* The Jacobian and the species rates of the same states in one pass (an
 * implicit solver needs both at every step): jac as pjg_jacobian writes it,
 * dphi (laid out like phi) bit for bit as pjg_species_rates writes it.  No
 * reference counterpart (the reference evaluates them in separate kernels). */
int pjg_jacobian_rates(pjg_mech* mech, int64_t n, char order, int conp, int jac_format,
                       const double* param, const double* phi, double* jac, double* dphi,
                       void* stream);
/* Species thermo, the chem_utils kernel type (pyjac/core/rate_subs.py
 * write_chem_utils :3391-3444; examples/opencl/ch4/chem_utils.ocl:49): at
 * the guarded temperature T = min(max(phi_T, 100 K), 10,000 K) of each state,
 * cp, h and the Gibbs function b of every species (cv, u and b when conp is
 * 0).  Each output holds Ns values per state: [i*Ns + k] for order 'C',
 * [i + n*k] for 'F'.  phi as above (only T is read). */
int pjg_chem_utils(pjg_mech* mech, int64_t n, char order, int conp, const double* phi, double* cp,
                   double* h, double* b, void* stream);
/* Vector-Jacobian product out = J^T v (dense J of kernel order; v, out have NN
 * entries per state in `order`).  No reference counterpart: the adjoint used
 * by the torch wdot autograd.Function. */
int pjg_vjp(pjg_mech* mech, int64_t n, char order, int conp, const double* param,
            const double* phi, const double* v, double* out, void* stream);
/* pjg_vjp without any device allocation, for callers that cannot allocate
 * at call time (solvers calling from a hot loop where cudaMalloc/cudaFree
 * would synchronise the device, hosts whose pool owns all device memory).
 * No counterpart in the reference.  Scratch is a fixed 16 MiB array inside
 * the library on each device, held until the process exits; larger problems
 * run as several launches on `stream`; mechanisms needing more than 16 MiB
 * per 128 states (more than 1,638 species) are rejected with PJG_ERR_ARG.  The
 * first call on a device takes the array's address (call it before any
 * stream capture).  All calls share the array: calls that overlap on the GPU
 * race. */
int pjg_vjp_noalloc(pjg_mech* mech, int64_t n, char order, int conp, const double* param,
                    const double* phi, const double* v, double* out, void* stream);

/* Kernel objects: the reference's Kernel class (kernel.hpp.in:86-335).
 * problem_size = states per call; work_size is accepted for API
 * compatibility (the reference's OpenMP thread / OpenCL group count) and
 * ignored: the GPU kernels size their own grids.  Host pointers (pinned host
 * memory lets the copies overlap the evaluation); each call streams the
 * states through a ring of three device buffers of two waves of resident
 * blocks each (155,648 states on a 152-SM GB300), copying one chunk in and
 * another out while a third is evaluated, and returns when the outputs are
 * in `out`.  A kernel object owns its device buffers, so kernel objects may
 * be used from different threads at once. */
int pjg_kernel_create(pjg_mech* mech, int kind, size_t problem_size, size_t work_size,
                      char order, int conp, int jac_format, pjg_kernel** out);
int pjg_kernel_resize(pjg_kernel* k, size_t problem_size, size_t work_size);
int pjg_kernel_call(pjg_kernel* k, const double* param, const double* phi, double* out);
/* requiredMemorySize(): device bytes held by the kernel object */
int pjg_kernel_required_memory(const pjg_kernel* k, size_t* bytes);
int pjg_kernel_destroy(pjg_kernel* k);

/* Surrogate network building blocks (no reference counterpart: the learned
 * wdot surrogate beside the FP64 path).  Operands are BF16 (raw 16-bit
 * storage, row-major, leading dimensions in elements, multiples of 8, 16-byte
 * aligned); products accumulate in FP32 on the tcgen05 tensor cores.
 *
 * pjg_mlp_linear: Y = act(X W^T + b) for X [M x K] and W [N x K]
 * (32 <= N <= 256, N % 32 == 0; 16 <= K <= 256, K % 16 == 0).  act 1 = SiLU.
 * When zprev is given (input-gradient pass) the product is multiplied by
 * SiLU'(zprev) before act.  Optional outputs: Y (BF16), YT (BF16, transposed,
 * YT[n * ldyt + m]), Z (BF16 pre-activation), Y32 (FP32), colsum (FP32,
 * += column sums of the result; bias gradients).
 * pjg_mlp_wgrad: C [Mo x No] += A [Mo x Kb] B [No x Kb]^T (FP32 C; Kb % 64 == 0),
 * the weight gradient reduced over states.
 * pjg_mlp_status: 1 if a tensor-core kernel timed out waiting for its
 * accumulator since the last clear. */
int pjg_mlp_linear(const void* X, int64_t ldx, const void* W, int64_t ldw, int64_t M, int N, int K,
                   const float* bias, int act, const void* zprev, int64_t ldzp, void* Y, int64_t ldy,
                   void* YT, int64_t ldyt, void* Z, int64_t ldz, float* Y32, int64_t ldy32,
                   float* colsum, void* stream);
int pjg_mlp_wgrad(const void* A, int64_t lda, const void* B, int64_t ldb, int Mo, int No,
                  int64_t Kb, float* C, int64_t ldc, void* stream);
int pjg_mlp_status(int clear);
/* The whole surrogate forward pass in one launch: Y [M x 64] (FP32) =
 * L4(SiLU(L3(SiLU(L2(SiLU(L1(SiLU(L0(X)))))))) for X [M x 64] BF16, where
 * Ll(a) = a Wl^T + bl with W0 [256 x 64], W1..W3 [256 x 256], W4 [64 x 256].
 * W[l] points at Wl in BF16, packed in 8-row x 16-byte core matrices, row
 * group major: byte ((n / 8) * (K / 8) + k / 8) * 128 + (n % 8) * 16 + (k % 8) * 2
 * holds W[n][k].  b[l] are FP32 biases.  Activations stay on chip between the
 * layers.  No reference counterpart (the learned wdot surrogate). */
int pjg_mlp_forward(const void* X, int64_t ldx, int64_t M, const void* const* W,
                    const float* const* b, float* Y, int64_t ldy, void* stream);
/* Surrogate input and output stages on device arrays (states in order 'C',
 * constant pressure).  Features: X [n x 64] BF16 = ((T - 1500) / 400,
 * (ln P - mu_P) / sd_P, (log10 max(c_k, floor) - mu_k) / sd_k ..., 0 ...),
 * c_k = max(n_k, 0) / V; stats = (mu_P, sd_P, mu[nn - 2], sd[nn - 2]).
 * Outputs: from the network outputs Y [n x 64] FP32, the rates
 * y_j = sinh(Y_j z_sd_j + z_mu_j) s_j of (dT/dt, dn_k/dt) and the
 * extra-variable rate recomputed from them as the FP64 path does, written to
 * dphi [n x nn]; lerr[n] = Y[s][err_col] (the predicted log10 error);
 * stats = (z_mu[nn - 1], z_sd[nn - 1], s[nn - 1], 1 - W_k / W_ns [nn - 2]).
 * No reference counterpart (the learned wdot surrogate). */
int pjg_surrogate_features(int64_t n, int32_t nn, const double* phi, const double* param,
                           const double* stats, void* X, double floor_c, void* stream);
int pjg_surrogate_outputs(int64_t n, int32_t nn, const float* Y, const double* phi,
                          const double* param, const double* stats, int32_t err_col, double* dphi,
                          float* lerr, void* stream);

/* Binary initial-condition files: the reference's read_initial_conditions
 * (pyjac/kernel_utils/common/read_initial_conditions.cpp.in:30-116).  One
 * record of NN + 1 doubles per state, C order on disk:
 * [T, param, phi_1 (extra variable), n_0 .. n_{Ns-2}], param = P (conp) or V
 * (conv).  Read fills param[n] and phi in `order`; a file that is missing or
 * holds fewer than n records returns PJG_ERR_ARG with a message (the reference
 * exits the process).  Write is the inverse.  Host memory, host code. */
int pjg_read_initial_conditions(const char* filename, int64_t n, int32_t nn, char order,
                                double* param, double* phi);
int pjg_write_initial_conditions(const char* filename, int64_t n, int32_t nn, char order,
                                 const double* param, const double* phi);

/* Linearly implicit integrator step on device arrays (asynchronous on
 * `stream`).  No reference counterpart: the reference names coupling its
 * Jacobians to Rosenbrock solvers as future work; these are that consumer.
 *
 * pjg_lu_factor: per state i, M_i = I - s h_i J_i (h_i = h[i], or h0 when h
 * is NULL; s h_i rounded once, then each entry fma(-s h_i, J, delta)),
 * factorised as P M = L U by LAPACK dgetf2's algorithm (partial pivoting on the
 * first largest |a|, whole-row interchanges, column scaled by 1/pivot when
 * |pivot| >= DBL_MIN, rank-1 update by FMA).  jac and lu are dense nn x nn
 * per state in the layout pjg_jacobian writes (order 'C': [n][nn][nn]
 * row-major; 'F': i + n*(row + nn*col)); lu may equal jac.  L (unit
 * diagonal, not stored) below and U on and above the diagonal.  piv: nn
 * 1-based row interchanges per state, laid out like phi; info[n] (optional):
 * 0, or k for the first exactly zero pivot U(k,k) (1-based; LAPACK's info).
 * 1 <= nn <= 4096: up to 169 a state's matrix lives in shared memory; above,
 * it is factored in place in lu (global memory) in panels of up to 16
 * columns, with the same operations in the same order, so the factors are
 * the same; larger sizes return PJG_ERR_UNSUPPORTED.
 * pjg_lu_solve: b (laid out like phi) <- M^-1 b from pjg_lu_factor's output.
 *
 * Static-pivot sparse LU (the factorisation of implicit chemistry solvers
 * such as KPP: no row interchanges).  The mechanism's Jacobian pattern plus
 * the diagonal is ordered once by the Markowitz rule (the remaining diagonal
 * entry with the least (row count - 1)(column count - 1), lowest index on
 * ties; symmetric permutation perm[position] = variable) and factored
 * symbolically; step k then updates only the filled pattern's rows x
 * columns.  pjg_lu_symbolic: that order and the counts (FMAs per state,
 * entries of L + U) for a CRS pattern, host only, any nn up to 4,096 (to
 * size larger mechanisms' factorisations; the sparse kernels take nn <= 169).  pjg_lu_plan_info: the same
 * for a mechanism (the plan is built on first use and kept with it).
 * pjg_lu_factor_sparse: M_i = I - s h_i J_i as for pjg_lu_factor, factored
 * without interchanges in the permuted order: lu[i][r][c] (dense layout of
 * jac) holds the factors of M_i[perm[r]][perm[c]] (zeros outside the filled
 * pattern); info[i] = k for the first exactly zero pivot (1-based step),
 * -k when the first pivot that is not finite comes first (without
 * interchanges a growing factor can overflow: the caller should then fall
 * back to pjg_lu_factor), 0 otherwise.
 * pjg_lu_solve_sparse: b (laid out like phi, variables' order) <- M^-1 b.
 *
 * pjg_ros2_step: one step of the L-stable Rosenbrock method ROS2
 * (gamma = 1 + 1/sqrt 2) from phi with step h_i: dense Jacobian and rates
 * at phi in one pass (pjg_jacobian_rates), one factorisation (lu_kind 0:
 * partial pivoting; 1: the static-pivot sparse plan), two solves, one more
 * rates evaluation;
 * phi_new = phi + 1.5 h k1 + 0.5 h k2 and, if err is not NULL, the embedded
 * first-order error estimate err = 0.5 h (k1 + k2).  Work arrays: jac_work
 * n*nn*nn doubles (holds the factors on return), piv_work n*nn int32
 * (lu_kind 0 only), vec_work 2*n*nn doubles (k1, k2 on return).  phi_new
 * must not alias phi. */
int pjg_lu_factor(int32_t nn, int64_t n, char order, double s, const double* h, double h0,
                  const double* jac, double* lu, int32_t* piv, int32_t* info, void* stream);
int pjg_lu_solve(int32_t nn, int64_t n, char order, const double* lu, const int32_t* piv,
                 double* b, void* stream);
int pjg_lu_symbolic(int32_t nn, const int32_t* row_ptr, const int32_t* col_ind, int32_t* perm,
                    int32_t* nnz_lu, int64_t* fma_per_state);
int pjg_lu_plan_info(pjg_mech* mech, int32_t* perm, int32_t* nnz_lu, int64_t* fma_per_state);
int pjg_lu_factor_sparse(pjg_mech* mech, int64_t n, char order, double s, const double* h,
                         double h0, const double* jac, double* lu, int32_t* info, void* stream);
int pjg_lu_solve_sparse(pjg_mech* mech, int64_t n, char order, const double* lu, double* b,
                        void* stream);
int pjg_ros2_step(pjg_mech* mech, int64_t n, char order, int conp, const double* param,
                  const double* phi, const double* h, double h0, int lu_kind, double* phi_new,
                  double* err, double* jac_work, int32_t* piv_work, double* vec_work,
                  int32_t* info, void* stream);

/* Page-lock (pin) a caller's host range in place for the kernel objects'
 * copies (cudaHostRegister), and release it.  Measured on GB300 after other
 * processes had churned host memory: dense GRI Jacobian calls into buffers
 * the CPU had first touched and then registered took 145-210 ms per 1M
 * states, against 146-334 ms (alternating) into cudaHostAlloc buffers. */
int pjg_host_register(void* ptr, size_t bytes);
int pjg_host_unregister(void* ptr);

/* Copy the last error message of this thread into buf (always NUL-terminated). */
int pjg_last_error(char* buf, size_t len);

#ifdef __cplusplus
}
#endif
#endif
