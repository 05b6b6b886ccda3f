/*
 * CPU oracle: a plain-C restatement of pyJac-v2's species-rate and
 * analytical-Jacobian evaluation, one state at a time, following the
 * reference's sub-kernel order.
 *
 * TEST INFRASTRUCTURE ONLY (checker for tests/, smoke() and the CPU-baseline
 * leg of bench.py).  The product never links this file.
 *
 * Species rates follow pyjac/core/rate_subs.py get_specrates_kernel (:3026)
 * and its sub-kernels; the Jacobian follows create_jacobian.py
 * get_jacobian_kernel (:4899) and its blocks.  Each function below names the
 * reference generator it restates.  Numeric guards follow
 * pyjac/core/instruction_creator.py:370-478 and pyjac/utils.py:280-292:
 * T clamped to [100, 10000] K, V >= 1e-30, moles/concentrations >= 1e-300 where
 * the reference guards them, exp(min(x, 690.775527898)), log(max(x, 1e-300)).
 * As in the reference, explicit T, V and P factors of the Jacobian blocks use
 * the unclamped state values.
 */
#include "pyjac_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define RU 8314.4621
#define PATM 101325.0
#define EXP_MAX 690.775527898
#define SMALL 1e-300
#define LN10 2.302585092994046

/* Integer power by repeated multiplication (fast_powi,
 * examples/opencl/ch4/species_rates.oclh:11-40). */
static double powi(double v, int p)
{
    if (p < 0) {
        v = 1.0 / v;
        p = -p;
    }
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

static double gexp(double x) { return exp(fmin(EXP_MAX, x)); }

typedef struct ws {
    int n_fall, n_thd;
    double *conc, *kf, *kr, *kf_fall, *thd_conc, *Pr, *Fi, *Fcent, *Atroe, *Btroe;
    double *Xsri, *b, *pres_mod, *ropf, *ropr, *wdot, *h, *cp, *dcp, *db, *dphi;
    double *gross, *scale; /* cancellation scale of wdot and of dphi (test metric only) */
} ws;

/* Arrhenius forms of rate_subs.py get_simple_arrhenius_rates (:2642-3023). */
static double arrhenius(int type, double A, double b, double Ta, double Tc, double logT,
                        double Tinv)
{
    if (type == 0) return A;
    if (type == 1) return A * powi(Tc, (int)b);
    return gexp(A + logT * b + -1.0 * Ta * Tinv);
}

/* PLOG bracket (rate_subs.py get_plog_arrhenius_rates :2084-2250). */
static void plog_bracket(const orc_mech* m, int pi, double logP, int* lo, int* hi, int* oor)
{
    const int np = m->n_plog, mp = m->plog_maxP;
    const double* lp = m->plog_params + (size_t)0 * np * mp + (size_t)pi * mp;
    const int numP = m->plog_numP[pi] - 1;
    int l = 0, h = 0;
    int lower = logP <= lp[0];
    int upper = logP > lp[numP];
    if (upper) {
        l = numP;
        h = numP;
    }
    for (int k = 0; k < numP; ++k)
        if (logP > lp[k] && logP <= lp[k + 1]) {
            l = k;
            h = k + 1;
        }
    *lo = l;
    *hi = h;
    *oor = lower || upper;
}

static double plog_par(const orc_mech* m, int which, int pi, int j)
{
    return m->plog_params[(size_t)which * m->n_plog * m->plog_maxP + (size_t)pi * m->plog_maxP + j];
}

/* ln kf and d ln kf / dT (at fixed P) and d ln kf / d ln P of a PLOG reaction. */
static double plog_logk(const orc_mech* m, int pi, double logT, double Tinv, double logP,
                        double Tj_inv, double* dlnk_dT, double* dlnk_dlnP)
{
    int lo, hi, oor;
    plog_bracket(m, pi, logP, &lo, &hi, &oor);
    double k1 = plog_par(m, 1, pi, lo) + logT * plog_par(m, 2, pi, lo) - plog_par(m, 3, pi, lo) * Tinv;
    double k2 = plog_par(m, 1, pi, hi) + logT * plog_par(m, 2, pi, hi) - plog_par(m, 3, pi, hi) * Tinv;
    double d1 = (plog_par(m, 2, pi, lo) + plog_par(m, 3, pi, lo) * Tj_inv) * Tj_inv;
    double d2 = (plog_par(m, 2, pi, hi) + plog_par(m, 3, pi, hi) * Tj_inv) * Tj_inv;
    double kf = k1;
    *dlnk_dT = d1;
    *dlnk_dlnP = 0.0;
    if (!oor) {
        double w = (logP - plog_par(m, 0, pi, lo)) / (plog_par(m, 0, pi, hi) - plog_par(m, 0, pi, lo));
        kf = (-k1 + k2) * w + kf;
        *dlnk_dT = d1 + (d2 - d1) * w;
        *dlnk_dlnP = (k2 - k1) / (plog_par(m, 0, pi, hi) - plog_par(m, 0, pi, lo));
    }
    return kf;
}

/* log10 kf of a Chebyshev reaction (rate_subs.py get_cheb_arrhenius_rates
 * :1904-2083) and its derivatives d log10 kf / dT and d log10 kf / d ln P. */
static double cheb_log10k(const orc_mech* m, int ci, double Tinv, double logP, double Tj_inv,
                          double* dT, double* dlnP)
{
    const int nT = m->cheb_nT[ci], nP = m->cheb_nP[ci];
    const double Tmin = m->cheb_Tlim[2 * ci], Tmax = m->cheb_Tlim[2 * ci + 1];
    const double Pmin = m->cheb_Plim[2 * ci], Pmax = m->cheb_Plim[2 * ci + 1];
    const double Tred = (-Tmax - Tmin + 2 * Tinv) / (Tmax - Tmin);
    const double Pred = (-Pmax - Pmin + 2 * logP) / (Pmax - Pmin);
    double tp[64], pp[64], dtp[64], dpp[64];
    int nmax = nT > nP ? nT : nP;
    if (nmax < 2) nmax = 2;
    tp[0] = 1.0; tp[1] = Tred; pp[0] = 1.0; pp[1] = Pred;
    dtp[0] = 0.0; dtp[1] = 1.0; dpp[0] = 0.0; dpp[1] = 1.0;
    for (int p = 2; p < nmax; ++p) {
        tp[p] = 2 * Tred * tp[p - 1] - tp[p - 2];
        pp[p] = 2 * Pred * pp[p - 1] - pp[p - 2];
        dtp[p] = 2 * tp[p - 1] + 2 * Tred * dtp[p - 1] - dtp[p - 2];
        dpp[p] = 2 * pp[p - 1] + 2 * Pred * dpp[p - 1] - dpp[p - 2];
    }
    const double* a = m->cheb_params + (size_t)ci * m->cheb_maxT * m->cheb_maxP;
    double kf = 0.0, dkT = 0.0, dkP = 0.0;
    for (int t = 0; t < nT; ++t) {
        double temp = 0.0, dtemp = 0.0;
        for (int p = 0; p < nP; ++p) {
            temp = temp + pp[p] * a[t * m->cheb_maxP + p];
            dtemp = dtemp + dpp[p] * a[t * m->cheb_maxP + p];
        }
        kf = kf + tp[t] * temp;
        dkT += dtp[t] * temp;
        dkP += tp[t] * dtemp;
    }
    /* dTred/dT = -2 / (T^2 (Tmax - Tmin)); dPred/dlnP = 2 / (Pmax - Pmin) */
    *dT = dkT * (-2.0 * Tj_inv * Tj_inv / (Tmax - Tmin));
    *dlnP = dkP * (2.0 / (Pmax - Pmin));
    return kf;
}

static void thermo_coeffs(const orc_mech* m, int k, double T, const double** a)
{
    *a = (T < m->T_mid[k]) ? m->a_lo + 7 * k : m->a_hi + 7 * k;
}

/* Species rates for one state: rate_subs.py get_specrates_kernel (:3026-3278). */
static void eval_rates(const orc_mech* m, int conp, double param, const double* phi, ws* w)
{
    const int ns = m->ns, nr = m->nr, last = ns - 1;
    const double T = phi[0];
    const double Tc = fmin(10000.0, fmax(100.0, T));
    const double logT = log(Tc), Tinv = 1.0 / Tc;
    const double V = conp ? phi[1] : param;
    const double P = conp ? param : phi[1];
    const double Vinv = 1.0 / fmax(1e-30, V);
    const double logP = log(P);

    /* get_concentrations, rate_subs.py:597-706 */
    double nsum = 0.0;
    w->conc[last] = P / (RU * Tc);
    for (int k = 0; k < last; ++k) {
        double nk = fmax(SMALL, phi[2 + k]);
        nsum = nsum + nk;
        w->conc[k] = nk * Vinv;
    }
    w->conc[last] = w->conc[last] + -1.0 * fmax(SMALL, nsum) * Vinv;

    /* forward rate constants: simple / PLOG / Chebyshev */
    for (int i = 0; i < nr; ++i) {
        int si = m->rxn_simple[i];
        if (si >= 0) {
            w->kf[i] = arrhenius(m->simple_type[si], m->simple_A[si], m->simple_b[si],
                                 m->simple_Ta[si], Tc, logT, Tinv);
        } else if (m->rxn_plog[i] >= 0) {
            double d1, d2;
            w->kf[i] = gexp(plog_logk(m, m->rxn_plog[i], logT, Tinv, logP, Tinv, &d1, &d2));
        } else {
            double d1, d2;
            double l10 = cheb_log10k(m, m->rxn_cheb[i], Tinv, logP, Tinv, &d1, &d2);
            w->kf[i] = exp(LN10 * fmin(EXP_MAX, l10));
        }
    }
    /* fall-off "other" rate (rateconst_fullfall) */
    for (int f = 0; f < w->n_fall; ++f)
        w->kf_fall[f] = arrhenius(m->fall_type[f], m->fall_A[f], m->fall_b[f], m->fall_Ta[f], Tc,
                                  logT, Tinv);
    /* third-body concentrations, rate_subs.py get_thd_body_concs :1788-1901 */
    for (int t = 0; t < w->n_thd; ++t) {
        int not_spec = m->thd_type[t] != 2;
        double tc = P * not_spec / (RU * T);
        for (int e = m->thd_off[t]; e < m->thd_off[t + 1]; ++e)
            tc = tc + (m->thd_eff[e] + -1.0 * not_spec) * w->conc[m->thd_spec[e]];
        w->thd_conc[t] = tc;
    }
    /* reduced pressure and blending (rate_subs.py :2251-2641) */
    for (int i = 0; i < nr; ++i) {
        int f = m->rxn_fall[i];
        if (f < 0) continue;
        int t = m->rxn_thd[i];
        double kinf, k0;
        if (!m->fall_ftype[f]) {
            kinf = w->kf[i];
            k0 = w->kf_fall[f];
        } else {
            kinf = w->kf_fall[f];
            k0 = w->kf[i];
        }
        double Pr = w->thd_conc[t] * k0 / kinf;
        w->Pr[f] = Pr;
        double Fi = 1.0;
        if (m->fall_troe[f] >= 0) {
            int q = m->fall_troe[f];
            double logPr = log10(fmax(SMALL, Pr));
            double Fc = m->troe_a[q] * gexp(-1.0 * Tc * m->troe_T1[q]) +
                        (1.0 + -1.0 * m->troe_a[q]) * gexp(-1.0 * Tc * m->troe_T3[q]);
            if (m->troe_T2[q] != 0.0) Fc = Fc + gexp(-1.0 * m->troe_T2[q] / Tc);
            double logFc = log10(fmax(SMALL, Fc));
            double B = -1.1762 * logFc + -1.0 * 0.14 * logPr + 0.806;
            double A = -0.67 * logFc + logPr + -0.4;
            w->Fcent[f] = Fc;
            w->Atroe[f] = A;
            w->Btroe[f] = B;
            Fi = pow(fmax(SMALL, Fc), 1.0 / (A * A / (B * B) + 1.0));
        } else if (m->fall_sri[f] >= 0) {
            int q = m->fall_sri[f];
            double logPr = log10(fmax(SMALL, Pr));
            double X = 1.0 / (logPr * logPr + 1.0);
            Fi = pow(m->sri_a[q] * gexp(-m->sri_b[q] * Tinv) + gexp(-Tc / m->sri_c[q]), X);
            if (m->sri_d[q] != 1.0) Fi = Fi * m->sri_d[q];
            if (m->sri_e[q] != 0.0) {
                double e = m->sri_e[q];
                Fi = Fi * (e == (double)(int)e ? powi(Tc, (int)e) : pow(Tc, e));
            }
            w->Xsri[f] = X;
        }
        w->Fi[f] = Fi;
    }
    /* Gibbs function b_k (polyfit_kernel_gen 'b', rate_subs.py:3349) */
    for (int k = 0; k < ns; ++k) {
        const double* a;
        thermo_coeffs(m, k, Tc, &a);
        w->b[k] = Tc * (Tc * (Tc * (Tc * a[4] / 20.0 + a[3] / 12.0) + a[2] / 6.0) + a[1] / 2.0) +
                  (a[0] + -1.0) * logT + -1.0 * a[0] + a[6] + -1.0 * a[5] * Tinv;
    }
    /* equilibrium constants and reverse rates (get_rev_rates :1627-1787) */
    for (int i = 0; i < nr; ++i) {
        if (m->rev_mask[i] < 0) {
            w->kr[i] = 0.0;
            continue;
        }
        double Pval = m->nu_sum[i] > 0 ? PATM / RU : RU / PATM;
        double Psum = powi(Pval, abs(m->nu_sum[i]));
        double Bsum = 0.0;
        for (int e = m->net_off[i]; e < m->net_off[i + 1]; ++e) {
            int nu = m->net_nu[2 * e] - m->net_nu[2 * e + 1];
            if (nu != 0) Bsum = Bsum + nu * w->b[m->net_spec[e]];
        }
        double Kc = Psum * gexp(Bsum);
        w->kr[i] = w->kf[i] / Kc;
    }
    /* pressure modification (get_rxn_pres_mod :1510-1626) */
    for (int i = 0; i < nr; ++i) {
        int t = m->rxn_thd[i];
        if (t < 0) continue;
        int f = m->rxn_fall[i];
        if (f < 0) {
            w->pres_mod[t] = w->thd_conc[t];
        } else {
            double ci = w->Fi[f] / (1.0 + w->Pr[f]);
            if (!m->fall_ftype[f]) ci = ci * w->Pr[f];
            w->pres_mod[t] = ci;
        }
    }
    /* rates of progress (get_rop :1371-1509, get_rop_net :1170-1370) and
     * net production (get_spec_rates :1079-1167) */
    for (int k = 0; k < ns; ++k) w->wdot[k] = 0.0, w->gross[k] = 0.0;
    for (int i = 0; i < nr; ++i) {
        double rf = w->kf[i], rr = w->kr[i];
        for (int e = m->net_off[i]; e < m->net_off[i + 1]; ++e) {
            double c = w->conc[m->net_spec[e]];
            rf = rf * powi(c, m->net_nu[2 * e + 1]);
            if (m->rev_mask[i] >= 0) rr = rr * powi(c, m->net_nu[2 * e]);
        }
        if (m->rev_mask[i] < 0) rr = 0.0;
        w->ropf[i] = rf;
        w->ropr[i] = rr;
        double net = rf;
        if (m->rev_mask[i] >= 0) net = net + -1.0 * rr;
        if (m->rxn_thd[i] >= 0) net = net * w->pres_mod[m->rxn_thd[i]];
        for (int e = m->net_off[i]; e < m->net_off[i + 1]; ++e) {
            int nu = m->net_nu[2 * e] - m->net_nu[2 * e + 1];
            w->wdot[m->net_spec[e]] = w->wdot[m->net_spec[e]] + nu * net;
#ifndef ORC_COUNTING /* test metric, not part of the reference's arithmetic */
            double ci_ = m->rxn_thd[i] >= 0 ? fabs(w->pres_mod[m->rxn_thd[i]]) : 1.0;
            w->gross[m->net_spec[e]] += fabs((double)nu) * (fabs(rf) + fabs(rr)) * ci_;
#endif
        }
    }
    /* molar rates, temperature and extra-variable rates (:709-1076) */
    const double Vval = fmax(1e-30, V);
    for (int k = 0; k < last; ++k) w->dphi[2 + k] = Vval * w->wdot[k];
    double upper = 0.0, lower = 0.0;
    for (int k = 0; k < ns; ++k) {
        const double* a;
        thermo_coeffs(m, k, Tc, &a);
        double cpk, hk;
        if (conp) {
            hk = RU * (Tc * (Tc * (Tc * (Tc * (Tc * a[4] / 5.0 + a[3] / 4.0) + a[2] / 3.0) + a[1] / 2.0) + a[0]) + a[5]);
            cpk = RU * (Tc * (Tc * (Tc * (Tc * a[4] + a[3]) + a[2]) + a[1]) + a[0]);
        } else {
            hk = RU * (Tc * (Tc * (Tc * (Tc * (Tc * a[4] / 5.0 + a[3] / 4.0) + a[2] / 3.0) + a[1] / 2.0) + a[0]) - Tc + a[5]);
            cpk = RU * (Tc * (Tc * (Tc * (Tc * a[4] + a[3]) + a[2]) + a[1]) + a[0] - 1.0);
        }
        w->h[k] = hk;
        w->cp[k] = cpk;
        w->dcp[k] = RU * (Tc * (Tc * (4.0 * Tc * a[4] + 3.0 * a[3]) + 2.0 * a[2]) + a[1]);
        w->db[k] = Tc * (Tc * (Tc * a[4] / 5.0 + a[3] / 4.0) + a[2] / 3.0) + a[1] / 2.0 +
                   Tinv * (a[0] + -1.0 + a[5] * Tinv);
        lower = lower + w->conc[k] * cpk;
        upper = upper + hk * w->wdot[k];
    }
    w->dphi[0] = 0.0 + -1.0 * upper / lower;
    double dE = 0.0;
    for (int k = 0; k < last; ++k) dE = dE + (1.0 + -1.0 * m->mw_post[k]) * w->wdot[k];
    if (conp) {
        w->dphi[1] = Vval * w->dphi[0] / Tc;
        w->dphi[1] = w->dphi[1] + Vval * dE * Tc * RU / P;
    } else {
        w->dphi[1] = P * w->dphi[0] / Tc;
        w->dphi[1] = w->dphi[1] + Tc * RU * dE;
    }
#ifndef ORC_COUNTING
    /* cancellation scale of each output: the same sums with absolute values
     * (a test metric, left out of the operation count) */
    double su = 0.0, sE = 0.0;
    for (int k = 0; k < ns; ++k) su += fabs(w->h[k]) * w->gross[k];
    for (int k = 0; k < last; ++k) sE += fabs(1.0 - m->mw_post[k]) * w->gross[k];
    double sT = su / fabs(lower);
    w->scale[0] = sT;
    w->scale[1] = conp ? Vval * sT / Tc + Vval * sE * Tc * RU / P : P * sT / Tc + Tc * RU * sE;
    for (int k = 0; k < last; ++k) w->scale[2 + k] = Vval * w->gross[k];
#endif
}

/* d ci / d x for a fall-off / chemically-activated reaction, given
 * d Pr / dx = Pr * theta + theta_n and the direct part of d ln Fi / dx
 * (create_jacobian.py dci_*_dT :2117-2588, dci_*_dE :362-880, dci_*_dnj
 * :3558-4168 all reduce to this form). */
static double dci_fall(const orc_mech* m, const ws* w, int f, double theta, double theta_n,
                       double dlnFi_direct)
{
    const double Pr = w->Pr[f], Fi = w->Fi[f];
    /* pres_mod of this reaction */
    double pmod = Fi / (1.0 + Pr);
    if (!m->fall_ftype[f]) pmod = pmod * Pr;
    double dPr = Pr * theta + theta_n;
    double dlnFi_dPr = 0.0;
    if (m->fall_troe[f] >= 0) {
        double A = w->Atroe[f], B = w->Btroe[f];
        double absq = A * A + B * B;
        dlnFi_dPr = -2.0 * A * B * log(fmax(SMALL, w->Fcent[f])) * (0.14 * A + B) /
                    (fmax(SMALL, Pr) * absq * absq * LN10);
    } else if (m->fall_sri[f] >= 0) {
        /* ln Fi = X ln Q + ln d + e ln T with dX/dPr = -2 X^2 log10(Pr) / (Pr ln 10);
         * eval_jacobian keeps ln Q of SRI reactions in Fcent */
        double X = w->Xsri[f];
        double logPr = log10(fmax(SMALL, Pr));
        dlnFi_dPr = -2.0 * X * X * logPr / (fmax(SMALL, Pr) * LN10) * w->Fcent[f];
    }
    double d = pmod * (dlnFi_dPr * dPr + dlnFi_direct - dPr / (Pr + 1.0));
    if (!m->fall_ftype[f]) d = d + theta * pmod + Fi * theta_n / (Pr + 1.0);
    return d;
}

/* Analytical Jacobian for one state: create_jacobian.py get_jacobian_kernel
 * (:4899-5128).  J is dense NN x NN, J[row * NN + col]. */
static void eval_jacobian(const orc_mech* m, int conp, double param, const double* phi, ws* w,
                          double* J)
{
    const int ns = m->ns, nr = m->nr, last = ns - 1, NN = ns + 1;
    eval_rates(m, conp, param, phi, w);
    memset(J, 0, sizeof(double) * NN * NN);
    const double Tj = phi[0], Tjinv = 1.0 / phi[0];
    const double Tc = fmin(10000.0, fmax(100.0, Tj));
    const double Vj = conp ? phi[1] : param;
    const double P = conp ? param : phi[1];
    const double logP = log(P);
    const double Tdot = w->dphi[0];
#define JAC(r, c) J[(size_t)(r) * NN + (c)]

    /* SRI needs ln Q at every use; keep it in Fcent (unused by SRI). */
    for (int f = 0; f < w->n_fall; ++f)
        if (m->fall_sri[f] >= 0) {
            int q = m->fall_sri[f];
            w->Fcent[f] = log(m->sri_a[q] * gexp(-m->sri_b[q] / Tc) + gexp(-Tc / m->sri_c[q]));
        }

    /* dRopidnj and dRopidnj_ns (create_jacobian.py:4169-4522) */
    for (int i = 0; i < nr; ++i) {
        const int o0 = m->net_off[i], o1 = m->net_off[i + 1];
        const double kf = w->kf[i];
        const double kr = m->rev_mask[i] >= 0 ? w->kr[i] : 0.0;
        const double ci = m->rxn_thd[i] >= 0 ? w->pres_mod[m->rxn_thd[i]] : 1.0;
        int has_ns = 0;
        for (int e = o0; e < o1; ++e) has_ns |= m->net_spec[e] == last;
        for (int ek = o0; ek < o1; ++ek) {
            const int sk = m->net_spec[ek];
            if (sk == last) continue;
            const int nuk = m->net_nu[2 * ek] - m->net_nu[2 * ek + 1];
            for (int ej = o0; ej < o1; ++ej) {
                const int sj = m->net_spec[ej];
                if (sj == last) continue;
                double Sr = m->net_nu[2 * ej], Sf = m->net_nu[2 * ej + 1];
                for (int e = o0; e < o1; ++e) {
                    int nr_ = m->net_nu[2 * e], nf_ = m->net_nu[2 * e + 1];
                    if (m->net_spec[e] == sj) {
                        nr_ -= 1;
                        nf_ -= 1;
                    }
                    double c = fmax(SMALL, w->conc[m->net_spec[e]]);
                    Sr = Sr * powi(c, nr_);
                    Sf = Sf * powi(c, nf_);
                }
                JAC(sk + 2, sj + 2) += (kf * Sf + -1.0 * kr * Sr) * ci * nuk;
            }
        }
        if (has_ns && !m->jac_approx) {
            for (int ek = o0; ek < o1; ++ek) {
                const int sk = m->net_spec[ek];
                if (sk == last) continue;
                const int nuk = m->net_nu[2 * ek] - m->net_nu[2 * ek + 1];
                double Sr = 1.0, Sf = 1.0;
                for (int e = o0; e < o1; ++e) {
                    int nr_ = m->net_nu[2 * e], nf_ = m->net_nu[2 * e + 1];
                    double c = fmax(SMALL, w->conc[m->net_spec[e]]);
                    if (m->net_spec[e] == last) {
                        Sr = Sr * nr_;
                        nr_ -= 1;
                    }
                    Sr = Sr * powi(c, nr_);
                    if (m->net_spec[e] == last) {
                        Sf = Sf * nf_;
                        nf_ -= 1;
                    }
                    Sf = Sf * powi(c, nf_);
                }
                double upd = (kr * Sr + -1.0 * kf * Sf) * ci * nuk;
                for (int j = 0; j < last; ++j) JAC(sk + 2, j + 2) += upd;
            }
        }
    }

    /* third-body and fall-off contributions to the species block
     * (dci_thd_dnj :3558, dci_{lind,troe,sri}_dnj :3600-4168) */
    for (int i = 0; i < nr; ++i) {
        const int t = m->rxn_thd[i];
        if (t < 0) continue;
        const int f = m->rxn_fall[i];
        const int o0 = m->net_off[i], o1 = m->net_off[i + 1];
        const double R = w->ropf[i] - (m->rev_mask[i] >= 0 ? w->ropr[i] : 0.0);
        const int ttype = m->thd_type[t];
        double fac = 1.0;
        if (f >= 0) {
            double k0 = m->fall_ftype[f] ? w->kf[i] : w->kf_fall[f];
            double kinf = m->fall_ftype[f] ? w->kf_fall[f] : w->kf[i];
            /* d ci / d[M] = dci(theta = 0, theta_n = k0 / kinf) */
            fac = dci_fall(m, w, f, 0.0, k0 / kinf, 0.0);
        }
        int ns_listed = 0;
        double ns_eff = 1.0;
        for (int e = m->thd_off[t]; e < m->thd_off[t + 1]; ++e)
            if (m->thd_spec[e] == last) {
                ns_listed = 1;
                ns_eff = m->thd_eff[e];
            }
        for (int e = m->thd_off[t]; e < m->thd_off[t + 1]; ++e) {
            const int sj = m->thd_spec[e];
            if (sj == last) continue;
            double dci = ttype == 2 ? 1.0 : (ttype == 1 ? m->thd_eff[e] + -1.0 : 0.0);
            for (int ek = o0; ek < o1; ++ek) {
                const int sk = m->net_spec[ek];
                if (sk == last) continue;
                const int nuk = m->net_nu[2 * ek] - m->net_nu[2 * ek + 1];
                JAC(sk + 2, sj + 2) += nuk * dci * R * fac;
            }
        }
        if (ns_listed && !m->jac_approx) {
            double dci = ttype == 2 ? -1.0 : (ttype == 1 ? 1.0 + -1.0 * ns_eff : 0.0);
            for (int ek = o0; ek < o1; ++ek) {
                const int sk = m->net_spec[ek];
                if (sk == last) continue;
                const int nuk = m->net_nu[2 * ek] - m->net_nu[2 * ek + 1];
                for (int j = 0; j < last; ++j) JAC(sk + 2, j + 2) += nuk * dci * R * fac;
            }
        }
    }

    /* thermo sums (cp_total, eval_dcp, eval_db) */
    double cp_tot = 0.0;
    for (int k = 0; k < ns; ++k) cp_tot = cp_tot + w->cp[k] * w->conc[k];

    /* dTdot_dnj (:3382) and dEdot_dnj (:3266) */
    const double fixed = conp ? P : Vj, extra = conp ? Vj : P;
    for (int j = 0; j < last; ++j) {
        double sum = 0.0, sumE = 0.0;
        for (int k = 0; k < last; ++k) {
            sum = sum + (w->h[k] + -1.0 * w->h[last] * m->mw_post[k]) * JAC(k + 2, j + 2);
            sumE = sumE + (1.0 - m->mw_post[k]) * JAC(k + 2, j + 2);
        }
        JAC(0, j + 2) = -1.0 * (sum + Tdot * (w->cp[j] + -1.0 * w->cp[last])) / (Vj * cp_tot);
        JAC(1, j + 2) += Tj * RU * sumE / fixed + extra * JAC(0, j + 2) * Tjinv;
    }

    /* temperature column: dRopi_dT (+ PLOG/Cheb) :2589-3108, dRopi_dT_ns,
     * dci_*_dT :2117-2588 */
    for (int i = 0; i < nr; ++i) {
        const int o0 = m->net_off[i], o1 = m->net_off[i + 1];
        const int t = m->rxn_thd[i], f = m->rxn_fall[i];
        const double ci = t >= 0 ? w->pres_mod[t] : 1.0;
        double dkf;
        int si = m->rxn_simple[i];
        if (si >= 0) {
            dkf = (m->simple_b[si] + m->simple_Ta[si] * Tjinv) * Tjinv;
        } else if (m->rxn_plog[i] >= 0) {
            double dP;
            plog_logk(m, m->rxn_plog[i], log(Tc), 1.0 / Tc, logP, Tjinv, &dkf, &dP);
        } else {
            double dP;
            cheb_log10k(m, m->rxn_cheb[i], 1.0 / Tc, logP, Tjinv, &dkf, &dP);
            dkf *= LN10;
        }
        double d = w->ropf[i] * dkf;
        if (m->rev_mask[i] >= 0) {
            double dB = 0.0;
            for (int e = o0; e < o1; ++e)
                dB = dB + (m->net_nu[2 * e] + -1.0 * m->net_nu[2 * e + 1]) * w->db[m->net_spec[e]];
            d = d + -1.0 * w->ropr[i] * (dkf + -1.0 * dB);
        }
        d = d * ci * Vj;
        /* last-species term through d c_ns / dT = -P / (R T^2) */
        int has_ns = 0;
        for (int e = o0; e < o1; ++e) has_ns |= m->net_spec[e] == last;
        if (has_ns) {
            double Sr = 0.0, Sf = 0.0;
            for (int e = o0; e < o1; ++e)
                if (m->net_spec[e] == last) {
                    Sr = m->net_nu[2 * e];
                    Sf = m->net_nu[2 * e + 1];
                }
            for (int e = o0; e < o1; ++e) {
                int nr_ = m->net_nu[2 * e], nf_ = m->net_nu[2 * e + 1];
                if (m->net_spec[e] == last) {
                    nr_ -= 1;
                    nf_ -= 1;
                }
                double c = fmax(SMALL, w->conc[m->net_spec[e]]);
                Sr = Sr * powi(c, nr_);
                Sf = Sf * powi(c, nf_);
            }
            double kr = m->rev_mask[i] >= 0 ? w->kr[i] : 0.0;
            d += (Sr * kr + -1.0 * Sf * w->kf[i]) * Vj * ci * P / (RU * Tj * Tj);
        }
        /* third-body / fall-off temperature dependence */
        if (t >= 0) {
            const double R = w->ropf[i] - (m->rev_mask[i] >= 0 ? w->ropr[i] : 0.0);
            const int ttype = m->thd_type[t];
            double mod = 1.0;
            const int tl = m->thd_off[t + 1] - 1;
            if (ttype == 2) mod = m->thd_spec[tl] == last;
            if (ttype == 1 && m->thd_off[t + 1] > m->thd_off[t] && m->thd_spec[tl] == last)
                mod = m->thd_eff[tl];
            const double dM = -1.0 * P * mod * (1.0 / RU) * Tjinv * Tjinv;
            if (f < 0) {
                d += dM * Vj * R;
            } else {
                double k0, kinf, b0, binf, Ta0, Tainf;
                if (!m->fall_ftype[f]) {
                    kinf = w->kf[i];
                    k0 = w->kf_fall[f];
                    binf = m->simple_b[si];
                    Tainf = m->simple_Ta[si];
                    b0 = m->fall_b[f];
                    Ta0 = m->fall_Ta[f];
                } else {
                    kinf = w->kf_fall[f];
                    k0 = w->kf[i];
                    b0 = m->simple_b[si];
                    Ta0 = m->simple_Ta[si];
                    binf = m->fall_b[f];
                    Tainf = m->fall_Ta[f];
                }
                const double theta = Tjinv * (b0 + -1.0 * binf + (Ta0 + -1.0 * Tainf) * Tjinv);
                const double theta_n = dM * k0 / kinf;
                double direct = 0.0;
                if (m->fall_troe[f] >= 0) {
                    int q = m->fall_troe[f];
                    double A = w->Atroe[f], B = w->Btroe[f], Fc = w->Fcent[f];
                    double absq = A * A + B * B;
                    double dFc = -1.0 * m->troe_a[q] * m->troe_T1[q] * gexp(-1.0 * Tj * m->troe_T1[q]) +
                                 (m->troe_a[q] + -1.0) * m->troe_T3[q] * gexp(-1.0 * Tj * m->troe_T3[q]) +
                                 m->troe_T2[q] * Tjinv * Tjinv * gexp(-1.0 * m->troe_T2[q] * Tjinv);
                    double lnFc = log(fmax(SMALL, Fc));
                    direct = -B * dFc * (2.0 * A * (1.1762 * A + -0.67 * B) * lnFc - B * absq * LN10) /
                             (Fc * absq * absq * LN10);
                } else if (m->fall_sri[f] >= 0) {
                    int q = m->fall_sri[f];
                    double X = w->Xsri[f];
                    double Q = m->sri_a[q] * gexp(-m->sri_b[q] / Tc) + gexp(-Tc / m->sri_c[q]);
                    double dQ = m->sri_a[q] * m->sri_b[q] * Tjinv * Tjinv * gexp(-m->sri_b[q] / Tc) -
                                gexp(-Tc / m->sri_c[q]) / m->sri_c[q];
                    direct = X * dQ / Q + m->sri_e[q] * Tjinv;
                }
                d += dci_fall(m, w, f, theta, theta_n, direct) * Vj * R;
            }
        }
        for (int e = o0; e < o1; ++e) {
            const int sk = m->net_spec[e];
            if (sk == last) continue;
            JAC(sk + 2, 0) += (m->net_nu[2 * e] + -1.0 * m->net_nu[2 * e + 1]) * d;
        }
    }

    /* dTdot_dT (:1847) and dEdot_dT (:2001) */
    {
        const double Vjinv = 1.0 / Vj;
        double dTsum = (w->cp[last] * Tjinv - w->dcp[last]) * w->conc[last];
        double rate_sum = 0.0;
        for (int k = 0; k < last; ++k) {
            rate_sum = rate_sum + Vjinv * JAC(2 + k, 0) * (-w->h[k] + w->h[last] * m->mw_post[k]);
            rate_sum = rate_sum + w->wdot[k] * (-w->cp[k] + m->mw_post[k] * w->cp[last]);
            dTsum = dTsum + (w->cp[last] * Tjinv - w->dcp[k]) * w->conc[k];
        }
        JAC(0, 0) += (Tdot * dTsum + rate_sum) / cp_tot;
        double sum = 0.0;
        if (conp) {
            for (int k = 0; k < last; ++k)
                sum = sum + (1.0 - m->mw_post[k]) * (Vjinv * JAC(2 + k, 0) + Tjinv * w->wdot[k]);
            JAC(1, 0) += Vj * Tjinv * (JAC(0, 0) - Tjinv * Tdot);
            JAC(1, 0) += RU * Tj * Vj * sum / P;
        } else {
            const double fac = Tj / Vj;
            for (int k = 0; k < last; ++k)
                sum = sum + (1.0 - m->mw_post[k]) * (JAC(2 + k, 0) * fac + w->wdot[k]);
            JAC(1, 0) += P * (JAC(0, 0) - Tdot * Tjinv) * Tjinv;
            JAC(1, 0) += RU * sum;
        }
    }

    /* extra-variable column: dRopi_dE (:1458-1594), dci_*_dE (:362-880) */
    for (int i = 0; i < nr; ++i) {
        const int o0 = m->net_off[i], o1 = m->net_off[i + 1];
        const int t = m->rxn_thd[i], f = m->rxn_fall[i];
        const double ci = t >= 0 ? w->pres_mod[t] : 1.0;
        const double kr = m->rev_mask[i] >= 0 ? w->kr[i] : 0.0;
        const double rr = m->rev_mask[i] >= 0 ? w->ropr[i] : 0.0;
        const double R = w->ropf[i] - rr;
        double d = 0.0;
        if (conp) {
            int nuf = -1, nur = -1;
            for (int e = o0; e < o1; ++e) {
                nur += m->net_nu[2 * e];
                nuf += m->net_nu[2 * e + 1];
            }
            d = -1.0 * nuf * w->ropf[i] + nur * rr;
            d = d * ci;
        } else if (m->rxn_plog[i] >= 0 || m->rxn_cheb[i] >= 0) {
            double dT_, dlnP;
            if (m->rxn_plog[i] >= 0) {
                plog_logk(m, m->rxn_plog[i], log(Tc), 1.0 / Tc, logP, Tjinv, &dT_, &dlnP);
            } else {
                cheb_log10k(m, m->rxn_cheb[i], 1.0 / Tc, logP, Tjinv, &dT_, &dlnP);
                dlnP *= LN10;
            }
            d = Vj * ci * R * dlnP / P;
        }
        int has_ns = 0;
        for (int e = o0; e < o1; ++e) has_ns |= m->net_spec[e] == last;
        if (has_ns) {
            double Sr = 0.0, Sf = 0.0;
            for (int e = o0; e < o1; ++e)
                if (m->net_spec[e] == last) {
                    Sr = m->net_nu[2 * e];
                    Sf = m->net_nu[2 * e + 1];
                }
            for (int e = o0; e < o1; ++e) {
                int nr_ = m->net_nu[2 * e], nf_ = m->net_nu[2 * e + 1];
                if (m->net_spec[e] == last) {
                    nr_ -= 1;
                    nf_ -= 1;
                }
                double c = fmax(SMALL, w->conc[m->net_spec[e]]);
                Sr = Sr * powi(c, nr_);
                Sf = Sf * powi(c, nf_);
            }
            /* d c_ns / dV = P / (R T V) beyond the -c/V of the mass-action term
             * (conp), d c_ns / dP = 1 / (R T) (conv) */
            const double g = conp ? P / (RU * Tj) : Vj / (RU * Tj);
            d += (w->kf[i] * Sf + -1.0 * kr * Sr) * ci * g;
        }
        if (t >= 0) {
            const int ttype = m->thd_type[t];
            double mod = conp ? (double)(ttype == 1) : 1.0;
            const int tl = m->thd_off[t + 1] - 1;
            if (ttype == 2) mod = m->thd_spec[tl] == last;
            if (ttype == 1 && m->thd_off[t + 1] > m->thd_off[t] && m->thd_spec[tl] == last)
                mod = m->thd_eff[tl];
            const double rt_inv = 1.0 / (RU * Tj);
            if (f < 0) {
                if (conp) {
                    double fac = 0.0;
                    if (ttype != 3) fac = mod * P * rt_inv + -1.0 * w->pres_mod[t];
                    d += fac * R;
                } else {
                    d += Vj * R * mod * rt_inv;
                }
            } else {
                double k0 = m->fall_ftype[f] ? w->kf[i] : w->kf_fall[f];
                double kinf = m->fall_ftype[f] ? w->kf_fall[f] : w->kf[i];
                double modp = mod * (conp ? P : 1.0) * rt_inv * k0 / kinf;
                double theta = conp ? -1.0 * (ttype != 3) : 0.0;
                double dc = dci_fall(m, w, f, theta, modp, 0.0);
                d += dc * (conp ? 1.0 : Vj) * R;
            }
        }
        for (int e = o0; e < o1; ++e) {
            const int sk = m->net_spec[e];
            if (sk == last) continue;
            JAC(sk + 2, 1) += (m->net_nu[2 * e] + -1.0 * m->net_nu[2 * e + 1]) * d;
        }
    }

    /* dTdot_dE (:1595) and dEdot_dE (:1740) */
    {
        if (conp) {
            double dTsum = 0.0, specsum = 0.0;
            for (int k = 0; k < last; ++k) {
                specsum = specsum + (w->h[k] - w->h[last] * m->mw_post[k]) * (JAC(k + 2, 1) - w->wdot[k]);
                dTsum = dTsum + (w->cp[k] - w->cp[last]) * w->conc[k];
            }
            double spec_inv = 1.0 / (cp_tot * Vj);
            JAC(0, 1) += (Tdot * dTsum - specsum) * spec_inv;
        } else {
            double sum = 0.0;
            for (int k = 0; k < last; ++k)
                sum = sum + (w->h[k] - w->h[last] * m->mw_post[k]) * JAC(k + 2, 1);
            double spec_inv = 1.0 / cp_tot;
            JAC(0, 1) -= (Tdot * w->cp[last] / (RU * Tj)) * spec_inv;
            JAC(0, 1) -= (sum * (1.0 / Vj)) * spec_inv;
        }
        double sum = 0.0;
        for (int k = 0; k < last; ++k) sum = sum + (1.0 - m->mw_post[k]) * JAC(k + 2, 1);
        const double pstr = conp ? P : Vj;
        JAC(1, 1) += RU * Tj * sum / pstr;
        JAC(1, 1) += (extra * JAC(0, 1) + Tdot) / Tj;
    }
#undef JAC
}

static int ws_alloc(const orc_mech* m, ws* w)
{
    int nf = 0, nt = 0;
    for (int i = 0; i < m->nr; ++i) {
        if (m->rxn_fall[i] + 1 > nf) nf = m->rxn_fall[i] + 1;
        if (m->rxn_thd[i] + 1 > nt) nt = m->rxn_thd[i] + 1;
    }
    w->n_fall = nf;
    w->n_thd = nt;
    const int ns = m->ns, nr = m->nr, NN = ns + 1;
    size_t tot = (size_t)ns * 10 + (size_t)nr * 4 + (size_t)(nf + 1) * 7 + (size_t)(nt + 1) * 2 + 2 * NN;
    double* p = (double*)calloc(tot, sizeof(double));
    if (!p) return -1;
    w->conc = p; p += ns;
    w->b = p; p += ns;
    w->wdot = p; p += ns;
    w->h = p; p += ns;
    w->cp = p; p += ns;
    w->dcp = p; p += ns;
    w->db = p; p += ns;
    w->gross = p; p += ns;
    p += 2 * ns;
    w->kf = p; p += nr;
    w->kr = p; p += nr;
    w->ropf = p; p += nr;
    w->ropr = p; p += nr;
    w->kf_fall = p; p += nf + 1;
    w->Pr = p; p += nf + 1;
    w->Fi = p; p += nf + 1;
    w->Fcent = p; p += nf + 1;
    w->Atroe = p; p += nf + 1;
    w->Btroe = p; p += nf + 1;
    w->Xsri = p; p += nf + 1;
    w->thd_conc = p; p += nt + 1;
    w->pres_mod = p; p += nt + 1;
    w->dphi = p; p += NN;
    w->scale = p;
    return 0;
}

static int run(const orc_mech* m, long n, int conp, const double* param, const double* phi,
               double* out, int nthreads, int jac)
{
    if (!m || n < 0 || (n > 0 && (!param || !phi || !out))) return -1;
    if (n == 0) return 0;
    const int NN = m->ns + 1;
    int err = 0;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads) reduction(| : err)
#endif
    {
        ws w;
        if (ws_alloc(m, &w)) {
            err |= 1;
        } else {
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
            for (long s = 0; s < n; ++s) {
                if (jac == 1) {
                    eval_jacobian(m, conp, param[s], phi + (size_t)s * NN, &w,
                                  out + (size_t)s * NN * NN);
                } else if (jac == 2) {
                    eval_rates(m, conp, param[s], phi + (size_t)s * NN, &w);
                    memcpy(out + (size_t)s * NN, w.scale, sizeof(double) * NN);
                } else {
                    eval_rates(m, conp, param[s], phi + (size_t)s * NN, &w);
                    memcpy(out + (size_t)s * NN, w.dphi, sizeof(double) * NN);
                }
            }
            free(w.conc);
        }
    }
    (void)nthreads;
    return err ? -2 : 0;
}

int orc_species_rates(const orc_mech* m, long n, int conp, const double* param,
                      const double* phi, double* dphi, int nthreads)
{
    return run(m, n, conp, param, phi, dphi, nthreads, 0);
}

int orc_jacobian(const orc_mech* m, long n, int conp, const double* param, const double* phi,
                 double* jac, int nthreads)
{
    return run(m, n, conp, param, phi, jac, nthreads, 1);
}

int orc_rates_detail(const orc_mech* m, int conp, double param, const double* phi, double* kf,
                     double* kr, double* Pr, double* Fi, double* wdot, double* dphi, double* conc)
{
    if (!m || !phi) return -1;
    ws w;
    if (ws_alloc(m, &w)) return -2;
    eval_rates(m, conp, param, phi, &w);
    if (kf) memcpy(kf, w.kf, sizeof(double) * m->nr);
    if (kr) memcpy(kr, w.kr, sizeof(double) * m->nr);
    if (Pr) memcpy(Pr, w.Pr, sizeof(double) * w.n_fall);
    if (Fi) memcpy(Fi, w.Fi, sizeof(double) * w.n_fall);
    if (wdot) memcpy(wdot, w.wdot, sizeof(double) * m->ns);
    if (dphi) memcpy(dphi, w.dphi, sizeof(double) * (m->ns + 1));
    if (conc) memcpy(conc, w.conc, sizeof(double) * m->ns);
    free(w.conc);
    return 0;
}

int orc_rates_scale(const orc_mech* m, long n, int conp, const double* param, const double* phi,
                    double* scale, int nthreads)
{
    return run(m, n, conp, param, phi, scale, nthreads, 2);
}

int orc_chem_utils(const orc_mech* m, long n, int conp, const double* phi, double* cp,
                   double* h, double* b)
{
    if (!m || n < 0 || (n && (!phi || !cp || !h || !b))) return -1;
    const int ns = m->ns, NN = ns + 1;
    for (long i = 0; i < n; ++i) {
        /* the temperature guard of polyfit_kernel_gen (TemperatureGuard) */
        const double Tc = fmin(10000.0, fmax(100.0, phi[i * NN]));
        const double logT = log(Tc), Tinv = 1.0 / Tc;
        for (int k = 0; k < ns; ++k) {
            const double* a;
            thermo_coeffs(m, k, Tc, &a);
            const double cpoly = Tc * (Tc * (Tc * (Tc * a[4] + a[3]) + a[2]) + a[1]) + a[0];
            const double hpoly =
                Tc * (Tc * (Tc * (Tc * (Tc * a[4] / 5.0 + a[3] / 4.0) + a[2] / 3.0) + a[1] / 2.0) + a[0]);
            cp[i * ns + k] = conp ? RU * cpoly : RU * (cpoly - 1.0);
            h[i * ns + k] = conp ? RU * (hpoly + a[5]) : RU * (hpoly - Tc + a[5]);
            b[i * ns + k] = Tc * (Tc * (Tc * (Tc * a[4] / 20.0 + a[3] / 12.0) + a[2] / 6.0) + a[1] / 2.0) +
                            (a[0] + -1.0) * logT + -1.0 * a[0] + a[6] + -1.0 * a[5] * Tinv;
        }
    }
    return 0;
}

/* ---- Newton-matrix LU of an implicit integrator step (no reference
 * counterpart; the algorithm is LAPACK's unblocked dgetf2 and dgetrs, with the
 * operation order of the CUDA kernels so that results agree bit for bit:
 * entries fma(-s h_i, J, delta), pivot = first largest |a| in the column,
 * whole-row interchange, scale by 1/pivot (or divide below DBL_MIN), rank-1
 * update a_rc = fma(-l_r, u_c, a_rc); solves in the column order of LAPACK's
 * dtrsv on a column-major matrix: the unit-lower pass subtracts each solved
 * y_c from the rows below in increasing c, the upper pass divides y_c by U's
 * diagonal and subtracts it from the rows above in decreasing c, each row
 * accumulating by FMA). */
int orc_lu_factor(int nn, long n, double s, const double* h, double h0, const double* jac,
                  double* lu, int* piv, int* info)
{
    if (nn < 1 || n < 0 || (n && (!jac || !lu || !piv))) return -1;
    for (long i = 0; i < n; ++i) {
        const double g = s * (h ? h[i] : h0);
        const double* J = jac + (size_t)i * nn * nn;
        double* a = lu + (size_t)i * nn * nn;
        int first_zero = 0;
        for (int r = 0; r < nn; ++r)
            for (int c = 0; c < nn; ++c) a[r * nn + c] = fma(-g, J[r * nn + c], r == c ? 1.0 : 0.0);
        for (int k = 0; k < nn; ++k) {
            int br = k;
            double best = fabs(a[k * nn + k]);
            for (int r = k + 1; r < nn; ++r)
                if (fabs(a[r * nn + k]) > best) {
                    best = fabs(a[r * nn + k]);
                    br = r;
                }
            piv[(size_t)i * nn + k] = br + 1;
            const double p = a[br * nn + k];
            if (p != 0.0) {
                if (br != k)
                    for (int c = 0; c < nn; ++c) {
                        const double t = a[k * nn + c];
                        a[k * nn + c] = a[br * nn + c];
                        a[br * nn + c] = t;
                    }
                if (fabs(p) >= DBL_MIN) {
                    const double inv = 1.0 / p;
                    for (int r = k + 1; r < nn; ++r) a[r * nn + k] *= inv;
                } else {
                    for (int r = k + 1; r < nn; ++r) a[r * nn + k] /= p;
                }
            } else if (!first_zero) {
                first_zero = k + 1;
            }
            for (int r = k + 1; r < nn; ++r)
                for (int c = k + 1; c < nn; ++c)
                    a[r * nn + c] = fma(-a[r * nn + k], a[k * nn + c], a[r * nn + c]);
        }
        if (info) info[i] = first_zero;
    }
    return 0;
}

int orc_lu_solve(int nn, long n, const double* lu, const int* piv, double* b)
{
    if (nn < 1 || n < 0 || (n && (!lu || !piv || !b))) return -1;
    for (long i = 0; i < n; ++i) {
        const double* a = lu + (size_t)i * nn * nn;
        double* y = b + (size_t)i * nn;
        for (int k = 0; k < nn; ++k) {
            const int p = piv[(size_t)i * nn + k] - 1;
            if (p != k) {
                const double t = y[k];
                y[k] = y[p];
                y[p] = t;
            }
        }
        for (int c = 0; c < nn; ++c)
            for (int r = c + 1; r < nn; ++r) y[r] = fma(-a[r * nn + c], y[c], y[r]);
        for (int c = nn - 1; c >= 0; --c) {
            y[c] = y[c] / a[c * nn + c];
            for (int r = 0; r < c; ++r) y[r] = fma(-a[r * nn + c], y[c], y[r]);
        }
    }
    return 0;
}

/* ROS2 stage arithmetic, element-wise with a per-state step (C order):
 * op 0: out = x + h k; op 1: out = x - 2 k; op 2: out = x + h (1.5 k + 0.5 z),
 * err = h (0.5 (k + z)). */
int orc_ros2_combine(int op, int nn, long n, const double* h, double h0, const double* x,
                     const double* k, const double* z, double* out, double* err)
{
    for (long i = 0; i < n; ++i) {
        const double hi = h ? h[i] : h0;
        for (int j = 0; j < nn; ++j) {
            const size_t e = (size_t)i * nn + j;
            if (op == 0) {
                out[e] = fma(hi, k[e], x[e]);
            } else if (op == 1) {
                out[e] = fma(-2.0, k[e], x[e]);
            } else {
                out[e] = fma(hi, fma(1.5, k[e], 0.5 * z[e]), x[e]);
                if (err) err[e] = hi * (0.5 * (k[e] + z[e]));
            }
        }
    }
    return 0;
}

/* ---- static-pivot sparse LU (no interchanges) on a precomputed plan: the
 * permuted matrix a[r][c] = fma(-s h_i, J[perm[r]][perm[c]], delta) is
 * eliminated in order; step k scales the rows R_k of column k by 1/pivot (or
 * divides below DBL_MIN) and updates R_k x C_k by FMA.  Dense C-order
 * storage of the permuted factors. */
int orc_lu_sparse_factor(int nn, long n, double s, const double* h, double h0, const double* jac,
                         const int* perm, const int* roff, const int* ridx, const int* coff,
                         const int* cidx, double* lu, int* info)
{
    if (nn < 1 || n < 0) return -1;
    for (long i = 0; i < n; ++i) {
        const double g = s * (h ? h[i] : h0);
        const double* J = jac + (size_t)i * nn * nn;
        double* a = lu + (size_t)i * nn * nn;
        int first_zero = 0;
        for (int r = 0; r < nn; ++r)
            for (int c = 0; c < nn; ++c)
                a[r * nn + c] = fma(-g, J[perm[r] * nn + perm[c]], r == c ? 1.0 : 0.0);
        for (int k = 0; k < nn; ++k) {
            const double p = a[k * nn + k];
            if (!first_zero) {
                if (p == 0.0) first_zero = k + 1;
                else if (!isfinite(p)) first_zero = -(k + 1);  /* overflow or NaN */
            }
            if (roff[k + 1] == roff[k]) continue;
            if (p != 0.0)
                for (int q = roff[k]; q < roff[k + 1]; ++q) {
                    const int r = ridx[q];
                    if (fabs(p) >= DBL_MIN)
                        a[r * nn + k] *= 1.0 / p;
                    else
                        a[r * nn + k] /= p;
                }
            for (int q = roff[k]; q < roff[k + 1]; ++q)
                for (int t = coff[k]; t < coff[k + 1]; ++t) {
                    const int r = ridx[q], c = cidx[t];
                    a[r * nn + c] = fma(-a[r * nn + k], a[k * nn + c], a[r * nn + c]);
                }
        }
        if (info) info[i] = first_zero;
    }
    return 0;
}

/* b [n][nn] (variables' order) <- M^-1 b from orc_lu_sparse_factor's factors */
int orc_lu_sparse_solve(int nn, long n, const double* lu, const int* perm, const int* loff,
                        const int* lidx, const int* uoff, const int* uidx, double* b)
{
    if (nn < 1 || n < 0) return -1;
    double* y = (double*)malloc(sizeof(double) * (size_t)nn);
    if (!y) return -2;
    for (long i = 0; i < n; ++i) {
        const double* a = lu + (size_t)i * nn * nn;
        double* x = b + (size_t)i * nn;
        for (int r = 0; r < nn; ++r) y[r] = x[perm[r]];
        for (int r = 1; r < nn; ++r) {
            double acc = y[r];
            for (int q = loff[r]; q < loff[r + 1]; ++q) acc = fma(-a[r * nn + lidx[q]], y[lidx[q]], acc);
            y[r] = acc;
        }
        for (int r = nn - 1; r >= 0; --r) {
            double acc = y[r];
            for (int q = uoff[r]; q < uoff[r + 1]; ++q) acc = fma(-a[r * nn + uidx[q]], y[uidx[q]], acc);
            y[r] = acc / a[r * nn + r];
        }
        for (int r = 0; r < nn; ++r) x[perm[r]] = y[r];
    }
    free(y);
    return 0;
}
