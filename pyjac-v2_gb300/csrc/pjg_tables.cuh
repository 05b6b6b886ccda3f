// Device-side mechanism tables of pyjac-v2_gb300.
//
// The mechanism is read by every thread with warp-uniform addresses (one
// thread per thermochemical state, all threads walk the same reaction list),
// so each record is a fixed-size, 16-byte-aligned block that a warp fetches
// as broadcast vector loads.
//
// Reaction record (192 bytes):
//   int   flags      bit layout RX_* below
//   int   nspec      distinct species in the reaction (<= PJG_MAXSP)
//   int   thd_off    first entry of this reaction's third-body list
//   int   thd_cnt    entries in that list (listed species other than the bath gas,
//                    and the bath gas itself when listed)
//   int   aux        offset of the PLOG / Chebyshev block in `aux`
//   int   nu_sum     sum of net stoichiometric coefficients (for Kc)
//   int   bint       integer temperature exponent of rate form 1
//   int   fbint      same for the fall-off "other" rate
//   uint  ent[8]     species entries sorted by species index:
//                    bits 0-15 species, 16-23 reactant nu, 24-31 product nu
//   double p[16]     parameters, indices P_* below
// The field semantics follow pyJac's assign_rates (pyjac/core/rate_subs.py:74-537):
// A is ln A for the full Arrhenius form and A itself for forms 0/1, Troe T1 and T3
// are stored inverted, SRI defaults d = 1, e = 0.
//
// Species record: see SP_* below.
//
// Third-body list entries: species index and (efficiency - flag), where flag is 1
// for mixture / unity third bodies and 0 for a single-species third body, so that
// [M] = flag * P / (R T) + sum coef * c (rate_subs.py get_thd_body_concs :1788-1901).
//
// PLOG block: numP, then (ln P, ln A, b, Ta) per pressure.
// Chebyshev block: nT, nP, Tmin, Tmax (as 1/T), Pmin, Pmax (as ln P), then nT x nP
// coefficients, row-major in (T, P).
#pragma once
#include <cstdint>

#define PJG_MAXSP 8
#define PJG_RXN_BYTES 192

// flags
#define RX_FORM_MASK 0x7      // 0: A, 1: A T^b (integer b), 2: Arrhenius, 3: PLOG, 4: Chebyshev
#define RX_REV (1 << 3)
#define RX_THD_SHIFT 4        // 0 none, 1 mixture, 2 single species, 3 unity
#define RX_BLEND_SHIFT 6      // 0 none, 1 Lindemann, 2 Troe, 3 SRI
#define RX_CHEM (1 << 8)      // chemically activated (else fall-off)
#define RX_FFORM_SHIFT 9      // rate form of the fall-off "other" rate (0..2)
#define RX_HASNS (1 << 11)    // the bath gas is a reactant or product
#define RX_NSLIST (1 << 12)   // the bath gas appears in the third-body list
#define RX_T2 (1 << 13)       // Troe T** present (non-zero)
#define RX_SRID (1 << 14)     // SRI d != 1
#define RX_SRIE (1 << 15)     // SRI e != 0
#define RX_SRIEINT (1 << 16)  // SRI e is integral
// set by the library's packing (pjg_capi.cu), clear in the tables it is given:
#define RX_SAMEM (1 << 20)    // [M] equals the previous packed reaction's (same group)
#define RX_SAMELNM (1 << 21)  // and ln [M] was formed by an earlier reaction of that run

#define RX_FORM(f) ((f) & RX_FORM_MASK)
#define RX_THD(f) (((f) >> RX_THD_SHIFT) & 3)
#define RX_BLEND(f) (((f) >> RX_BLEND_SHIFT) & 3)
#define RX_FFORM(f) (((f) >> RX_FFORM_SHIFT) & 3)

enum { THD_NONE = 0, THD_MIX = 1, THD_SPEC = 2, THD_UNITY = 3 };
enum { BL_NONE = 0, BL_LIND = 1, BL_TROE = 2, BL_SRI = 3 };
enum { FORM_A = 0, FORM_AT = 1, FORM_ARR = 2, FORM_PLOG = 3, FORM_CHEB = 4 };

// parameter indices in PjgRxn::p
#define P_A 0
#define P_B 1
#define P_TA 2
#define P_FA 3
#define P_FB 4
#define P_FTA 5
#define P_F0 6     // Troe a      | SRI a
#define P_F1 7     // Troe 1/T*** | SRI b
#define P_F2 8     // Troe T**    | SRI c
#define P_F3 9     // Troe 1/T*   | SRI d
#define P_F4 10    //             | SRI e
#define P_PSUM 11  // (P_atm / R)^nu_sum, evaluated on the host like the reference
#define P_FLAG 12  // 1 for mixture/unity third bodies, 0 for a single species
#define P_CNS 13   // (efficiency of the bath gas - flag) when listed, else 0
#define P_MOD 14   // flag + P_CNS: d[M]/dT = -P * mod / (R T^2)

struct __align__(16) PjgRxn {
    int flags, nspec, thd_off, thd_cnt;
    int aux, nu_sum, bint, fbint;
    unsigned ent[PJG_MAXSP];
    double p[16];
};
static_assert(sizeof(PjgRxn) == PJG_RXN_BYTES, "reaction record size");

// Species record (48 doubles): T_mid, W_k / W_ns, 1 - W_k / W_ns, padding, then
// one 20-double block per temperature range (low at SP_LO, high at SP_HI):
//   a0..a6, the NASA-7 coefficients;
//   a1/2, a2/3, a3/4, a4/5   (enthalpy and d b / dT polynomials);
//   a1/2, a2/6, a3/12, a4/20 (Gibbs polynomial);
//   2 a2, 3 a3, 4 a4         (d cp / dT);
//   a0 - 1, a6 - a0.
// The quotients are formed once on the host so that the kernels evaluate the
// polynomials of pyjac/core/rate_subs.py:3335-3356 without FP64 divisions.
#define SP_TMID 0
#define SP_MW 1
#define SP_OMW 2
#define SP_LO 8
#define SP_HI 28
#define PJG_SP_DOUBLES 48
#define TH_A 0
#define TH_Q 7
#define TH_R 11
#define TH_S 15
#define TH_A0M1 18
#define TH_A6MA0 19

__host__ __device__ inline int ent_spec(unsigned e) { return (int)(e & 0xffffu); }
__host__ __device__ inline int ent_nuf(unsigned e) { return (int)((e >> 16) & 0xffu); }
__host__ __device__ inline int ent_nur(unsigned e) { return (int)(e >> 24); }
