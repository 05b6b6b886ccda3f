/*
 * CPU oracle for pyJac-v2's species-rate and analytical-Jacobian path.
 *
 * TEST INFRASTRUCTURE ONLY.  Used by tests/ (as the checker), by
 * __graft_entry__.smoke() and by bench.py's CPU-baseline leg; never linked or
 * called by the product library.
 *
 * The mechanism is described with the reference's own table layout, i.e. the
 * dictionary returned by pyjac/core/rate_subs.py:assign_rates (:74-537),
 * flattened to plain arrays.  All arrays are owned by the caller.
 */
#ifndef PYJAC_ORACLE_H
#define PYJAC_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_mech {
    int ns, nr;                 /* species (incl. bath gas, last) and reactions */
    /* net stoichiometry, rate_subs.py:129-182 */
    const int* net_off;         /* nr + 1 */
    const int* net_spec;        /* species per entry */
    const int* net_nu;          /* 2 per entry: (product nu, reactant nu) */
    const int* nu_sum;          /* nr */
    const int* rev_mask;        /* nr: index among reversible reactions, or -1 */
    /* reaction -> index in each sub-table, or -1 */
    const int* rxn_simple;
    const int* rxn_plog;
    const int* rxn_cheb;
    const int* rxn_thd;
    const int* rxn_fall;
    /* simple Arrhenius, rate_subs.py:219-270 */
    const int* simple_type;     /* 0: A, 1: A T^b (integer b), 2..4: exp(lnA + b lnT - Ta/T) */
    const double *simple_A, *simple_b, *simple_Ta;
    /* PLOG, rate_subs.py:436-453: params[4][n_plog][maxP] = (lnP, lnA, b, Ta) */
    int plog_maxP;
    const int* plog_numP;
    const double* plog_params;
    int n_plog;
    /* Chebyshev, rate_subs.py:419-434 */
    int cheb_maxT, cheb_maxP, n_cheb;
    const int *cheb_nT, *cheb_nP;
    const double* cheb_params;  /* [n_cheb][maxT][maxP] */
    const double* cheb_Plim;    /* [n_cheb][2], ln P */
    const double* cheb_Tlim;    /* [n_cheb][2], 1 / T */
    /* third bodies, rate_subs.py:366-404 */
    const int* thd_type;        /* 1 mix, 2 species, 3 unity */
    const int* thd_off;         /* n_thd + 1 */
    const int* thd_spec;
    const double* thd_eff;
    /* fall-off, rate_subs.py:297-365 */
    const int* fall_ftype;      /* 0 fall-off, 1 chemically activated */
    const int* fall_blend;      /* 1 Lindemann, 2 Troe, 3 SRI */
    const int* fall_type;       /* rate type of the "other" Arrhenius rate */
    const double *fall_A, *fall_b, *fall_Ta;
    const int* fall_troe;       /* fall index -> Troe index or -1 */
    const int* fall_sri;        /* fall index -> SRI index or -1 */
    const double *troe_a, *troe_T1, *troe_T2, *troe_T3;   /* T1, T3 inverted */
    const double *sri_a, *sri_b, *sri_c, *sri_d, *sri_e;
    /* thermo, rate_subs.py:406-418, :458 */
    const double *a_lo, *a_hi;  /* [ns][7] */
    const double* T_mid;
    const double* mw_post;      /* ns - 1 */
    /* 1: the 'approximate' Jacobian type, without the bath-gas ("_ns")
     * terms in the species columns (create_jacobian.py:186-190, :3578-3582,
     * :4187-4191) */
    int jac_approx;
} orc_mech;

/* phi: [n][ns+1] = (T, V or P, n_0 .. n_{ns-2}); param: P (conp) or V (conv).
 * dphi: [n][ns+1].  jac: dense [n][ns+1][ns+1], jac[i][row][col] = d dphi_row / d phi_col.
 * Returns 0 on success, negative on bad arguments. */
int orc_species_rates(const orc_mech* m, long n, int conp, const double* param,
                      const double* phi, double* dphi, int nthreads);
int orc_jacobian(const orc_mech* m, long n, int conp, const double* param,
                 const double* phi, double* jac, int nthreads);
/* Cancellation scale of every dphi entry: the rate sums evaluated with
 * absolute values (sum |nu| (|rop_f| + |rop_r|) |ci| per species, propagated
 * through the T and extra-variable rates).  A parity metric, not a reference
 * quantity. */
/* One state's intermediates of the species-rate evaluation: forward and
 * reverse rate constants (nr each), reduced pressures and blending factors
 * (one per fall-off reaction), net molar production rates (ns), dphi
 * (ns + 1) and concentrations (ns).  Any output may be NULL. */
int orc_rates_detail(const orc_mech* m, int conp, double param, const double* phi, double* kf,
                     double* kr, double* Pr, double* Fi, double* wdot, double* dphi, double* conc);
int orc_rates_scale(const orc_mech* m, long n, int conp, const double* param,
                    const double* phi, double* scale, int nthreads);
/* Species thermo of the chem_utils kernel type (rate_subs.py write_chem_utils
 * :3391-3444, polyfit_kernel_gen :3281-3388): at the guarded T = phi[i][0],
 * cp (cv for conv), h (u) and the Gibbs function b of every species,
 * out[i][k] for k < ns. */
int orc_chem_utils(const orc_mech* m, long n, int conp, const double* phi, double* cp,
                   double* h, double* b);
/* Newton matrix of an implicit step, M_i = I - s h_i J_i (h NULL: h0), LU with
 * partial pivoting (LAPACK dgetf2's algorithm), C order only: jac, lu
 * [n][nn][nn], piv [n][nn] 1-based, info [n] (may be NULL).  lu may equal jac. */
int orc_lu_factor(int nn, long n, double s, const double* h, double h0, const double* jac,
                  double* lu, int* piv, int* info);
/* b [n][nn] <- M^-1 b from orc_lu_factor's factors */
int orc_lu_solve(int nn, long n, const double* lu, const int* piv, double* b);
/* static-pivot sparse LU on a plan (permutation, per-step row and column
 * lists R_k, C_k, and the filled pattern's L and U rows), C order */
int orc_lu_sparse_factor(int nn, long n, double s, const double* h, double h0, const double* jac,
                         const int* perm, const int* roff, const int* ridx, const int* coff,
                         const int* cidx, double* lu, int* info);
int orc_lu_sparse_solve(int nn, long n, const double* lu, const int* perm, const int* loff,
                        const int* lidx, const int* uoff, const int* uidx, double* b);
/* stage arithmetic of the ROS2 Rosenbrock step, C order */
int orc_ros2_combine(int op, int nn, long n, const double* h, double h0, const double* x,
                     const double* k, const double* z, double* out, double* err);

#ifdef __cplusplus
}
#endif
#endif
