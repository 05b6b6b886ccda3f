// Kernel argument block and per-state array layout shared by the evaluation
// kernels (pjg_eval.cu) and their host launcher (pjg_capi.cu).
#pragma once
#include <cstdint>
#include "pjg_tables.cuh"

#define PJG_BLOCK 128
// columns of the species block whose row-T and row-E sums the dense assembly
// keeps in registers at a time
#define PJG_DENSE_COLS 4

// per-state arrays (each ns doubles)
enum {
    ARR_CONC = 0,  // concentrations c_k
    ARR_EP,        // exp(b_k), the reactant factor of 1 / Kc, where the state's
                   // |b| allow (StateVars::split); else the Gibbs function b_k
    ARR_EM,        // exp(-b_k), the product factor of 1 / Kc (split states)
    ARR_WDOT,      // net molar production rates
    ARR_N_RATES,
    ARR_DB = ARR_N_RATES,  // d b_k / dT
    ARR_NSROW,     // per-row sum of bath-gas terms, subtracted from every species column
    ARR_HW,        // h_k - h_ns W_k / W_ns (row-0 weights)
    ARR_CP,        // specific heats
    ARR_DCP,       // d cp_k / dT
    ARR_H,         // specific enthalpies (energies at constant volume)
    ARR_N_JAC
};

struct EvalArgs {
    // mechanism
    const PjgRxn* rxn;
    const double* sp;
    const int* thd_spec;
    const double* thd_coef;
    const double* aux;
    int ns, nr;
    int nr_e22;      // reactions [0, nr_e22) are of the class A + B <=> C + D (see pjg_rxn.cuh)
    int ma_off[11];  // then [ma_off[q], ma_off[q + 1]) of mass-action pattern q (MaP0..MaP9),
                     // ma_off[0] = nr_e22
    int tp_off[4];   // then [tp_off[q], tp_off[q + 1]) of third-body pattern q (TpP0..TpP2),
                     // tp_off[0] = ma_off[10]; the others from tp_off[3]
    // 690 / (largest sum |nu| of a reversible reaction), at most 138: the bound
    // on every |b_k| of a state for the per-species factors of 1 / Kc
    double kc_split_max;
    int need_logP;
    int jac_approx;  // 'approximate' Jacobian type: no bath-gas terms in the species columns
    // states
    int64_t n;  // states in this launch
    int conp;
    const double* param;
    const double* phi;
    int64_t phi_ss, phi_sj;  // element (s, j) at phi[s * phi_ss + j * phi_sj]
    double* dphi;            // optional
    int64_t dphi_ss, dphi_sj;
    // per-state arrays in global scratch: array a, species k, state s at
    // scratch[(a * ns + k) * sc_ld + s]
    double* scratch;
    int64_t sc_ld;
    // Jacobian accumulator: acc[slot * acc_ld + s]
    double* acc;
    int64_t acc_ld;
    int nslot;
    const int* rxn_slot_off;  // nr + 1
    const int* rxn_slots;
    const int* row_off;       // ns (rows of species 0..ns-2)
    const int2* row_list;     // (species column j, slot)
    const int* col_off;       // ns
    const int2* col_list;     // (species row k, slot)
    const int* sp_slots;      // 2 per species row: slot(k, T), slot(k, E)
    const int* cj_slots;      // 2 per species column: slot(T, j), slot(E, j)
    int s00, s01, s10, s11;
    // dense output: slot of (row r, column c) = r * dense_rs + c * dense_cs
    // (0, 0 for a sparse output, whose slots come from the tables)
    int dense_rs, dense_cs;
    // for species columns [PJG_DENSE_COLS c, PJG_DENSE_COLS (c + 1)), entries
    // dchunk_list[dchunk_off[c] .. dchunk_off[c + 1]) = k << 4 | mask, the species
    // rows k (increasing) with a structurally nonzero entry there, bit q of mask
    // for column PJG_DENSE_COLS c + q; for a sparse output dchunk_slots holds
    // the four slots of each listed row (-1 outside the pattern)
    const int* dchunk_off;
    const int* dchunk_list;
    const int4* dchunk_slots;
    // vector-Jacobian product
    const double* v;          // v[s * phi_ss + j * phi_sj]
    double* vjp;              // same layout
};

// host launchers (pjg_eval.cu)
int pjg_launch_eval(const EvalArgs& a, int kind, void* stream);
// CUDA's description of the error of this thread's last pjg_launch_eval
const char* pjg_launch_error_string();
// resident blocks per SM of the evaluation kernel of `kind`
int pjg_eval_blocks_per_sm(int kind);
int pjg_launch_zero(double* acc, int64_t ld, int64_t n, int nslot, void* stream);
int pjg_fp64_probe(int blocks, int threads, int iters, double* out, void* stream);
int pjg_launch_fexp(const double* x, double* y, int64_t n, void* stream);
int pjg_launch_chem_utils(const double* sp, int ns, int64_t n, int conp, const double* phi,
                          int64_t phi_ss, double* cp, double* h, double* b, int64_t out_ss,
                          int64_t out_sk, void* stream);
int pjg_launch_transpose(const double* src, int64_t ld, int64_t n, int nslot, double* dst,
                         void* stream);
