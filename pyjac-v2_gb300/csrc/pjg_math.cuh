// Device math shared by the evaluation kernels.
//
// GB300 executes FP64 at 2 FMA/clock/SM, so the kernels are bound by the
// number of FP64 instructions: helpers here avoid FP64 divisions and reuse
// logarithms where the algebra allows it.
#pragma once
#include <cstdint>
#include "pjg_tables.cuh"

#define RU 8314.4621
#define EXP_MAX 690.775527898
#define SMALL 1e-300
#define LN10 2.302585092994046
#define INV_LN10 0.4342944819032518

namespace pjg {

__device__ __forceinline__ double ldg(const double* p) { return __ldg(p); }

// Integer power by repeated multiplication (the reference's fast_powi,
// examples/opencl/ch4/species_rates.oclh:11-40); p is warp-uniform and >= 0.
__device__ __forceinline__ double powi(double v, int p)
{
    switch (p) {
    case 0: return 1.0;
    case 1: return v;
    case 2: return v * v;
    case 3: return v * v * v;
    case 4: return v * v * v * v;
    case 5: return v * v * v * v * v;
    }
    double r = v * v * v * v * v * v;
    for (int i = 6; i < p; ++i) r *= v;
    return r;
}

// multiply acc by v^p for a small non-negative warp-uniform p (skips p == 0)
__device__ __forceinline__ double mulpow(double acc, double v, int p)
{
    if (p == 0) return acc;
    if (p == 1) return acc * v;
    if (p == 2) return acc * (v * v);
    return acc * powi(v, p);
}

// Table of 2^(j/2^B), j = 0 .. 2^B - 1, in shared memory (B = PJG_EXP_BITS):
// every kernel that calls fexp fills one per block with fill_exp_table before
// its first use, copied from the generated pjg_exp2_table (B = 8, 10, 11).
// B = 10 (1,024 entries, 8 KB) is the default: its degree-3 minimax
// polynomial has one FMA fewer than B = 8's degree-4 Taylor polynomial.  The
// random lookups meet bank conflicts, which B = 4 (16 entries, one bank pair
// each) avoids and B = 0 (no table) does without, both at the price of a
// longer polynomial.  Measured on GB300 (1,048,576 GRI-Mech 3.0 states, F
// order): B = 4 and B = 0 against B = 6, the Jacobian kernel 2.6 % and 8.3 %
// slower, the species-rate kernel 13 % and 30 % slower; B = 8 against B = 6,
// the Jacobian 73.5 against 74.3 ms and the species rates 29.0 against 30.1
// ms; later B = 10 against B = 8, the Jacobian 70.4 against 70.9 ms and the
// species rates 23.3 against 24.2 ms.  B = 11 (16 KB per block) equals B = 10
// on GRI and slows the 500-species mechanism's Jacobian by 13 %.  The FP64
// instruction count, not the shared-memory lookups, sets the time.
#ifndef PJG_EXP_BITS
#define PJG_EXP_BITS 10
#endif
#define PJG_EXP_TAB (1 << PJG_EXP_BITS)
}  // namespace pjg
#include "pjg_exp_table.h"  // pjg_exp2_table for B = 8, 10, 11 (gen_exp_table.py)
namespace pjg {

__device__ __forceinline__ void fill_exp_table(double* tab)
{
    for (int j = threadIdx.x; j < PJG_EXP_TAB; j += blockDim.x)
#ifdef PJG_EXP_HAVE_TABLE
        tab[j] = pjg_exp2_table[j];
#else
        tab[j] = exp2((double)j * (1.0 / PJG_EXP_TAB));
#endif
}

// exp(x) by the table-driven method of P. T. P. Tang ("Table-driven
// implementation of the exponential function in IEEE floating-point
// arithmetic", ACM TOMS 15(2), 1989): x = (2^B m + j) ln2 / 2^B + r with
// |r| <= ln2 / 2^(B+1), so exp(x) = 2^m 2^(j/2^B) exp(r).  exp(r) is a
// polynomial: of degree 3 for B = 10 and 11 with minimax coefficients
// (gen_exp_table.py; |r| <= 3.4e-4, largest relative error 9.4e-17 for
// B = 10), else the Taylor polynomial, of degree 4 for B = 8 (|r| <= 0.00136,
// truncation below 4e-17 relative), 5 for B = 6 (|r| <= 0.0055, below
// 4e-17), 7 for B = 4 (|r| <= 0.022, below 2e-18) and 13 for B = 0
// (|r| <= 0.35, below 5e-18).  The reduction is Cody and Waite's with
// ln2 split in two (the leading part is the double nearest ln 2, the trailing
// part the rest), each product taken by one FMA.  The scale 2^m goes into the
// exponent field with an integer add.  |x| >= 708, infinities and NaN take
// the library exp.  Tested against the CUDA library exp: within 3 ulp.
__device__ __forceinline__ double fexp(double x, const double* tab)
{
    if ((__double_as_longlong(x) & 0x7fffffffffffffffLL) >= 0x4086200000000000LL)  // |x| >= 708
        return exp(x);
    const double inv = 1.4426950408889634 * PJG_EXP_TAB;             // 2^B / ln 2
    const double l1 = 0.6931471805599453 * (1.0 / PJG_EXP_TAB);       // ln 2 / 2^B, leading part
    const double l2 = 2.3190468138462996e-17 * (1.0 / PJG_EXP_TAB);   // ln 2 / 2^B - l1
    const double shift = 6755399441055744.0;       // 1.5 * 2^52: rounds to an integer
    const double t = fma(x, inv, shift);
    const double nd = t - shift;                   // nearest integer to 2^B x / ln 2
    const int n = __double2loint(t);               // the same integer
    double r = fma(-nd, l1, x);
    r = fma(-nd, l2, r);
    // q = (exp(r) - 1) / r by Horner's rule on the Taylor coefficients 1/k!
    // (B >= 10: on the minimax coefficients of gen_exp_table.py)
#if PJG_EXP_BITS >= 10
    double q = fma(r, PJG_EXP_C3, PJG_EXP_C2);
    q = fma(q, r, 1.0);
#elif PJG_EXP_BITS >= 8
    double q = 1.0 / 24;
#elif PJG_EXP_BITS >= 6
    double q = fma(r, 1.0 / 120, 1.0 / 24);
#elif PJG_EXP_BITS >= 4
    double q = fma(r, 1.0 / 40320, 1.0 / 5040);
    q = fma(q, r, 1.0 / 720);
    q = fma(q, r, 1.0 / 120);
    q = fma(q, r, 1.0 / 24);
#else
    double q = fma(r, 1.0 / 87178291200.0, 1.0 / 6227020800.0);
    q = fma(q, r, 1.0 / 479001600.0);
    q = fma(q, r, 1.0 / 39916800.0);
    q = fma(q, r, 1.0 / 3628800.0);
    q = fma(q, r, 1.0 / 362880.0);
    q = fma(q, r, 1.0 / 40320);
    q = fma(q, r, 1.0 / 5040);
    q = fma(q, r, 1.0 / 720);
    q = fma(q, r, 1.0 / 120);
    q = fma(q, r, 1.0 / 24);
#endif
#if PJG_EXP_BITS < 10
    q = fma(q, r, 1.0 / 6);
    q = fma(q, r, 0.5);
    q = fma(q, r, 1.0);
#endif
#if PJG_EXP_BITS > 0
    const double tj = tab[n & (PJG_EXP_TAB - 1)];
    const double y = fma(tj, r * q, tj);
#else
    const double y = fma(r, q, 1.0);
#endif
    return __longlong_as_double(__double_as_longlong(y) + ((long long)(n >> PJG_EXP_BITS) << 52));
}

// min(c, x) for a positive constant c on the integer pipe (GB300's FP64 pipe
// is the kernels' bound): as signed 64-bit integers, doubles order like
// their values against a positive c, negative values having the sign bit set.
// Equal to fmin(c, x) for every x but a NaN with the sign bit set, which it
// returns where fmin returns c.
__device__ __forceinline__ double min_pos(double c, double x)
{
    return __double_as_longlong(x) < __double_as_longlong(c) ? x : c;
}

// |x| <= c for a positive constant c on the integer pipe (false for NaN)
__device__ __forceinline__ bool abs_le(double x, double c)
{
    return (__double_as_longlong(x) & 0x7fffffffffffffffLL) <= __double_as_longlong(c);
}

// x != 0.0 on the integer pipe (either zero compares equal, NaN unequal)
__device__ __forceinline__ bool nonzero(double x) { return (__double_as_longlong(x) << 1) != 0; }

// exp(min(x, 690.775527898)), the reference's guarded exponential
// (pyjac/core/instruction_creator.py GuardedExp :436-448)
__device__ __forceinline__ double gexp(double x, const double* tab) { return fexp(min_pos(EXP_MAX, x), tab); }

// positive-argument max(1e-300, x) guard without an FP64 instruction: for
// x >= 0 the IEEE order equals the integer order of the bit patterns, and a
// negative x (sign bit set) compares below.
__device__ __forceinline__ double gsmall(double x)
{
    const long long b = __double_as_longlong(x);
    const long long s = 0x01a56e1fc2f8f359LL;  // bits of 1e-300
    return __longlong_as_double(b > s ? b : s);
}

// Arrhenius forms of rate_subs.py get_simple_arrhenius_rates (:2642-3023)
__device__ __forceinline__ double arrhenius(int form, double A, double b, double Ta, int bint,
                                            double Tc, double logT, double Tinv, const double* tab)
{
    if (form == FORM_A) return A;
    // fast_powi of a negative exponent inverts its base first
    if (form == FORM_AT) return A * (bint < 0 ? powi(Tinv, -bint) : powi(Tc, bint));
    return gexp(A + logT * b + -1.0 * Ta * Tinv, tab);
}

// the same, also giving ln k (the clamped exponent) for the exponential form
// (has_ln false for the forms A and A T^b)
__device__ __forceinline__ double arrhenius_ln(int form, double A, double b, double Ta, int bint,
                                               double Tc, double logT, double Tinv,
                                               const double* tab, double& lnk, bool& has_ln)
{
    has_ln = form > FORM_AT;
    if (form == FORM_A) return A;
    if (form == FORM_AT) return A * (bint < 0 ? powi(Tinv, -bint) : powi(Tc, bint));
    lnk = min_pos(EXP_MAX, A + logT * b + -1.0 * Ta * Tinv);
    return fexp(lnk, tab);
}

// PLOG: ln kf interpolated linearly in ln P between bracketing pressures,
// clamped outside the table (rate_subs.py :2187-2224).  Returns ln kf, and
// d ln kf / dT (explicit factor Tjinv = 1/T) and d ln kf / d ln P.
__device__ inline double plog_logk(const double* blk, double logT, double Tinv, double logP,
                                   double Tjinv, double* dT, double* dlnP)
{
    const int np = (int)ldg(blk);
    const double* q = blk + 1;
    const int last = np - 1;
    int lo = 0, hi = 0;
    const bool lower = logP <= ldg(q);
    const bool upper = logP > ldg(q + 4 * last);
    if (upper) {
        lo = last;
        hi = last;
    }
    for (int k = 0; k < last; ++k)
        if (logP > ldg(q + 4 * k) && logP <= ldg(q + 4 * (k + 1))) {
            lo = k;
            hi = k + 1;
        }
    const double* a = q + 4 * lo;
    const double* b = q + 4 * hi;
    const double k1 = ldg(a + 1) + logT * ldg(a + 2) - ldg(a + 3) * Tinv;
    const double k2 = ldg(b + 1) + logT * ldg(b + 2) - ldg(b + 3) * Tinv;
    const double d1 = (ldg(a + 2) + ldg(a + 3) * Tjinv) * Tjinv;
    const double d2 = (ldg(b + 2) + ldg(b + 3) * Tjinv) * Tjinv;
    double kf = k1;
    *dT = d1;
    *dlnP = 0.0;
    if (!(lower || upper)) {
        const double w = (logP - ldg(a)) / (ldg(b) - ldg(a));
        kf = (-k1 + k2) * w + kf;
        *dT = d1 + (d2 - d1) * w;
        *dlnP = (k2 - k1) / (ldg(b) - ldg(a));
    }
    return kf;
}

// Chebyshev: log10 kf = sum_t sum_p a_tp T_t(Tred) T_p(Pred) (rate_subs.py :2028-2067),
// with d log10 kf / dT and d log10 kf / d ln P.
__device__ inline double cheb_log10k(const double* blk, double Tinv, double logP, double Tjinv,
                                     double* dT, double* dlnP)
{
    const int nT = (int)ldg(blk), nP = (int)ldg(blk + 1);
    const double Tmin = ldg(blk + 2), Tmax = ldg(blk + 3);
    const double Pmin = ldg(blk + 4), Pmax = ldg(blk + 5);
    const double* a = blk + 6;
    const double Tred = (-Tmax - Tmin + 2 * Tinv) / (Tmax - Tmin);
    const double Pred = (-Pmax - Pmin + 2 * logP) / (Pmax - Pmin);
    double kf = 0.0, dkT = 0.0, dkP = 0.0;
    double tm2 = 1.0, tm1 = Tred, dtm2 = 0.0, dtm1 = 1.0;
    for (int t = 0; t < nT; ++t) {
        double tp, dtp;
        if (t == 0) {
            tp = 1.0;
            dtp = 0.0;
        } else if (t == 1) {
            tp = Tred;
            dtp = 1.0;
        } else {
            tp = 2 * Tred * tm1 - tm2;
            dtp = 2 * tm1 + 2 * Tred * dtm1 - dtm2;
            tm2 = tm1;
            tm1 = tp;
            dtm2 = dtm1;
            dtm1 = dtp;
        }
        double temp = 0.0, dtemp = 0.0;
        double pm2 = 1.0, pm1 = Pred, dpm2 = 0.0, dpm1 = 1.0;
        for (int p = 0; p < nP; ++p) {
            double pp, dpp;
            if (p == 0) {
                pp = 1.0;
                dpp = 0.0;
            } else if (p == 1) {
                pp = Pred;
                dpp = 1.0;
            } else {
                pp = 2 * Pred * pm1 - pm2;
                dpp = 2 * pm1 + 2 * Pred * dpm1 - dpm2;
                pm2 = pm1;
                pm1 = pp;
                dpm2 = dpm1;
                dpm1 = dpp;
            }
            const double c = ldg(a + t * nP + p);
            temp = temp + pp * c;
            dtemp = dtemp + dpp * c;
        }
        kf = kf + tp * temp;
        dkT += dtp * temp;
        dkP += tp * dtemp;
    }
    *dT = dkT * (-2.0 * Tjinv * Tjinv / (Tmax - Tmin));
    *dlnP = dkP * (2.0 / (Pmax - Pmin));
    return kf;
}

// NASA-7 properties of one species at T (rate_subs.py polyfit_kernel_gen :3335-3356)
struct Thermo {
    double cp, h, b, db, dcp;
};

template <bool DERIV>
__device__ __forceinline__ Thermo thermo(const double* rec, double Tc, double logT, double Tinv,
                                         bool conp)
{
    const double* c = rec + (Tc < ldg(rec + SP_TMID) ? SP_LO : SP_HI);
    const double a0 = ldg(c + 0), a1 = ldg(c + 1), a2 = ldg(c + 2), a3 = ldg(c + 3),
                 a4 = ldg(c + 4), a5 = ldg(c + 5);
    Thermo t;
    // cp (cv) and h (u)
    const double cpoly = Tc * (Tc * (Tc * (Tc * a4 + a3) + a2) + a1);
    const double hpoly = Tc * (Tc * (Tc * (Tc * (Tc * ldg(c + TH_Q + 3) + ldg(c + TH_Q + 2)) +
                                           ldg(c + TH_Q + 1)) + ldg(c + TH_Q)) + a0);
    if (conp) {
        t.cp = RU * (cpoly + a0);
        t.h = RU * (hpoly + a5);
    } else {
        t.cp = RU * (cpoly + ldg(c + TH_A0M1));
        t.h = RU * (hpoly - Tc + a5);
    }
    // Gibbs function b = S/R - H/RT (with the -ln T of Kc folded in)
    t.b = Tc * (Tc * (Tc * (Tc * ldg(c + TH_R + 3) + ldg(c + TH_R + 2)) + ldg(c + TH_R + 1)) +
                ldg(c + TH_R)) + ldg(c + TH_A0M1) * logT + ldg(c + TH_A6MA0) + -1.0 * a5 * Tinv;
    if (DERIV) {
        t.db = Tc * (Tc * (Tc * ldg(c + TH_Q + 3) + ldg(c + TH_Q + 2)) + ldg(c + TH_Q + 1)) +
               ldg(c + TH_Q) + Tinv * (ldg(c + TH_A0M1) + a5 * Tinv);
        t.dcp = RU * (Tc * (Tc * (Tc * ldg(c + TH_S + 2) + ldg(c + TH_S + 1)) + ldg(c + TH_S)) + a1);
    } else {
        t.db = 0.0;
        t.dcp = 0.0;
    }
    return t;
}

}  // namespace pjg
