// Per-reaction evaluation of the evaluation kernels (pjg_eval.cu).
//
// rxn_terms() evaluates one reaction at one state: forward rate constant
// (get_simple_arrhenius_rates :2642, PLOG :2084, Chebyshev :1904 of
// pyjac/core/rate_subs.py), reverse rate through the equilibrium constant
// (:1627), mass-action rates of progress (:1170-1509), third-body and
// fall-off pressure modification (:1510-1626, :1788-2641), and, when DER is
// set, the reaction's analytical derivative terms (create_jacobian.py
// dRopi_dnj :4169-4522, dci_*_dnj :3558-4168, dRopidT :2589-3108,
// dRopidE :1458-1594, dci_*_dT :2117-2588, dci_*_dE :362-880).
//
// The caller owns the accumulation: species rates get nu_k * net, species row
// k of the Jacobian gets nu_k * (g_j ci) in column j, nu_k * d0 in column T,
// nu_k * d1 in column E, nu_k * coef_l * X in the columns of the third-body
// list, and nu_k * (gns ci + cns X) in every species column (the bath-gas
// terms, gathered per row).
//
// Per-state arrays are read through an accessor with operator[] (a strided
// view of global memory, or a shared-memory pointer).
#pragma once
#include "pjg_math.cuh"
#include "pjg_tables.cuh"

namespace pjg {

// nu * x for a warp-uniform small integer nu without an int->double conversion
// -x by flipping the sign bit on the integer pipe: a value that only feeds a
// reduction cannot fold the negation into an FP64 instruction
__device__ __forceinline__ double negi(double x)
{
    return __hiloint2double(__double2hiint(x) ^ 0x80000000, __double2loint(x));
}

__device__ __forceinline__ double nux(int nu, double x)
{
    switch (nu) {
    case 1: return x;
    case -1: return negi(x);
    case 2: return x + x;
    case -2: return negi(x + x);
    case 0: return 0.0;
    }
    return (double)nu * x;
}

// acc + nu * x
__device__ __forceinline__ double addnu(double acc, int nu, double x)
{
    switch (nu) {
    case 1: return acc + x;
    case -1: return acc - x;
    case 2: return fma(2.0, x, acc);
    case -2: return fma(-2.0, x, acc);
    case 0: return acc;
    }
    return fma((double)nu, x, acc);
}

// scalars of one thermochemical state used by every reaction
struct StateVars {
    double T;       // temperature (unclamped: explicit factors of the Jacobian)
    double Tc;      // T clamped to [100, 10000] K (rate evaluation)
    double logT, Tinv;  // of Tc
    double Tjinv;   // 1 / T
    double V, P;
    double PoRT;    // P / (R T)
    double rt_inv;  // 1 / (R T)
    double logP;    // ln P (PLOG / Chebyshev mechanisms only)
    bool conp;
    // every |b_k| <= EvalArgs::kc_split_max = 690 / (the mechanism's largest
    // sum |nu| of a reversible reaction): 1 / Kc is the product of the
    // participants' exp(+-b_k) (no partial product past e^690, so the
    // reference's clamp of sum nu b at 690.78 never acts); else
    // exp(-sum nu b) per reaction from b_k
    bool split;
    const double* etab;  // fexp table (shared memory)
};

// decoded reaction header
struct RxnHead {
    int flags, nsp, thd_off, thd_cnt, auxo, bint, fbint;
    unsigned ent[PJG_MAXSP];
    const double* p;
};

__device__ __forceinline__ void load_head(const PjgRxn* R, RxnHead& h)
{
    const int4 h0 = __ldg(reinterpret_cast<const int4*>(R));
    const int4 h1 = __ldg(reinterpret_cast<const int4*>(R) + 1);
    h.flags = h0.x;
    h.nsp = h0.y;
    h.thd_off = h0.z;
    h.thd_cnt = h0.w;
    h.auxo = h1.x;
    h.bint = h1.z;
    h.fbint = h1.w;
    const uint4 e0 = __ldg(reinterpret_cast<const uint4*>(R) + 2);
    const uint4 e1 = __ldg(reinterpret_cast<const uint4*>(R) + 3);
    h.ent[0] = e0.x; h.ent[1] = e0.y; h.ent[2] = e0.z; h.ent[3] = e0.w;
    h.ent[4] = e1.x; h.ent[5] = e1.y; h.ent[6] = e1.z; h.ent[7] = e1.w;
    h.p = R->p;
}

struct RxnTerms {
    double net;              // pressure-modified net rate of progress
    double g[PJG_MAXSP];          // d (rf - rr) / d c_j for participant j
    double gns;              // the same for the bath gas (0 if absent)
    double ci_;              // pressure modification (1 without third body)
    double d0, d1;           // temperature and extra-variable column terms
    double X;                // third-body column factor, Rnet d ci / d [M]
};

// mulpow with rounded products: the rates of progress must not depend on
// how the compiler contracts them into later FMAs, which differs between the
// kernel kinds (the Jacobian kernel's rates equal the rates kernel's bit for
// bit)
__device__ __forceinline__ double mulpow_rn(double acc, double v, int p)
{
    if (p == 0) return acc;
    if (p == 1) return __dmul_rn(acc, v);
    if (p == 2) return __dmul_rn(acc, __dmul_rn(v, v));
    return __dmul_rn(acc, powi(v, p));
}

// Stoichiometry of a reaction as rxn_terms() reads it: from the record
// (RunStoich) or fixed at compile time by a coefficient pattern
// (PatStoich<MaPattern<...>>, the record's entries stored in the pattern's
// order).
struct RunStoich {
    __device__ static int nsp(const RxnHead& h) { return h.nsp; }
    __device__ static int nuf(const RxnHead& h, int e) { return ent_nuf(h.ent[e]); }
    __device__ static int nur(const RxnHead& h, int e) { return ent_nur(h.ent[e]); }
};
template <class PT>
struct PatStoich {
    __device__ static constexpr int nsp(const RxnHead&) { return PT::n; }
    __device__ static constexpr int nuf(const RxnHead&, int e) { return PT::nuf(e); }
    __device__ static constexpr int nur(const RxnHead&, int e) { return PT::nur(e); }
};

// exp(-sum nu b) as the product of the participants' per-species factors
// exp(b_k)^-nu (nu < 0) and exp(-b_k)^nu (nu > 0), where StateVars::split
// holds (no partial product then passes e^690).
template <class ST, class ARR>
__device__ __forceinline__ double inv_kc_split(const RxnHead& h, const ARR& ep, const ARR& em)
{
    double r = 1.0;
    bool first = true;
#pragma unroll
    for (int e = 0; e < PJG_MAXSP; ++e) {
        if (e >= ST::nsp(h)) break;
        const int nu = ST::nur(h, e) - ST::nuf(h, e);
        if (nu == 0) continue;
        const int k = ent_spec(h.ent[e]);
        const double f = nu < 0 ? ep[k] : em[k];
        const int na = nu < 0 ? -nu : nu;
        const double fn = na == 1 ? f : (na == 2 ? __dmul_rn(f, f) : powi(f, na));
        r = first ? fn : __dmul_rn(r, fn);
        first = false;
    }
    return r;
}

// [M] of the last third-body reaction evaluated and ln [M] of the last
// fall-off reaction that formed it: the packing makes reactions with the
// same [M] adjacent and marks the repeats (RX_SAMEM, RX_SAMELNM)
struct MCache {
    double M = 0.0, logM = 0.0;
};

struct FallState {
    double Pr, Fi, A, B, Fc, lnFc, X, lnQ, kratio, logPr;
    double e1, e2, e3;  // Troe exponentials at the clamped temperature
};

template <bool DER, class ST = RunStoich, class ARR>
__device__ __forceinline__ void rxn_terms(const RxnHead& h, const double* aux,
                                          const int* thd_spec, const double* thd_coef, int last,
                                          const StateVars& sv, const ARR& conc, const ARR& bk,
                                          const ARR& ep, const ARR& em, const ARR& db, MCache& mc,
                                          RxnTerms& o)
{
    const int flags = h.flags, nsp = ST::nsp(h);
    const double* p = h.p;
    const int form = RX_FORM(flags);
    const bool rev = flags & RX_REV;
    const double Tc = sv.Tc, logT = sv.logT, Tinv = sv.Tinv, Tjinv = sv.Tjinv;
    const double* et = sv.etab;

    // forward rate constant and its log-derivatives
    double kf, dlnkf_dT = 0.0, dlnkf_dlnP = 0.0, lnkf = 0.0;
    bool has_lnkf = false;
    if (form <= FORM_ARR) {
        kf = arrhenius_ln(form, ldg(p + P_A), ldg(p + P_B), ldg(p + P_TA), h.bint, Tc, logT, Tinv,
                          et, lnkf, has_lnkf);
        if (DER) dlnkf_dT = (ldg(p + P_B) + ldg(p + P_TA) * Tjinv) * Tjinv;
    } else if (form == FORM_PLOG) {
        kf = gexp(plog_logk(aux + h.auxo, logT, Tinv, sv.logP, Tjinv, &dlnkf_dT, &dlnkf_dlnP), et);
    } else {
        const double l10 = cheb_log10k(aux + h.auxo, Tinv, sv.logP, Tjinv, &dlnkf_dT, &dlnkf_dlnP);
        kf = fexp(LN10 * min_pos(EXP_MAX, l10), et);
        dlnkf_dT *= LN10;
        dlnkf_dlnP *= LN10;
    }
    // reverse rate: kr = kf / Kc, Kc = (P_atm/R)^nu_sum exp(sum nu b)
    double kr = 0.0, dB = 0.0;
    if (rev) {
        if (DER) {
#pragma unroll
            for (int e = 0; e < PJG_MAXSP; ++e) {
                if (e >= nsp) break;
                const int nu = ST::nur(h, e) - ST::nuf(h, e);
                if (nu != 0) dB = addnu(dB, nu, db[ent_spec(h.ent[e])]);
            }
        }
        double ikc;
        if (sv.split) {
            ikc = inv_kc_split<ST>(h, ep, em);
        } else {
            double Bsum = 0.0;
#pragma unroll
            for (int e = 0; e < PJG_MAXSP; ++e) {
                if (e >= nsp) break;
                const int nu = ST::nur(h, e) - ST::nuf(h, e);
                if (nu != 0) Bsum = addnu(Bsum, nu, bk[ent_spec(h.ent[e])]);
            }
            ikc = fexp(-min_pos(EXP_MAX, Bsum), et);
        }
        kr = kf * ldg(p + P_PSUM) * ikc;
    }
    // rates of progress (mass action on raw concentrations)
    double rf = kf, rr = kr;
#pragma unroll
    for (int e = 0; e < PJG_MAXSP; ++e) {
        if (e >= nsp) break;
        const double c = conc[ent_spec(h.ent[e])];
        rf = mulpow_rn(rf, c, ST::nuf(h, e));
        if (rev) rr = mulpow_rn(rr, c, ST::nur(h, e));
    }
    // third-body / fall-off pressure modification
    const int thd = RX_THD(flags);
    const int blend = RX_BLEND(flags);
    const bool chem = flags & RX_CHEM;
    double ci = 1.0, M = 0.0;
    FallState fs;
    fs.Pr = 0.0; fs.Fi = 1.0; fs.A = 0.0; fs.B = 0.0; fs.Fc = 1.0; fs.lnFc = 0.0; fs.X = 0.0;
    fs.lnQ = 0.0; fs.kratio = 0.0; fs.e1 = 0.0; fs.e2 = 0.0; fs.e3 = 0.0; fs.logPr = 0.0;
    if (thd) {
        if (flags & RX_SAMEM) {
            M = mc.M;
        } else {
            M = sv.PoRT * ldg(p + P_FLAG);
            for (int l = 0; l < h.thd_cnt; ++l)
                M = fma(__ldg(thd_coef + h.thd_off + l), conc[__ldg(thd_spec + h.thd_off + l)], M);
            mc.M = M;
        }
        if (blend == BL_NONE) {
            ci = M;
        } else {
            double lnkfall = 0.0;
            bool has_lnkfall = false;
            const double kfall = arrhenius_ln(RX_FFORM(flags), ldg(p + P_FA), ldg(p + P_FB),
                                              ldg(p + P_FTA), h.fbint, Tc, logT, Tinv, et,
                                              lnkfall, has_lnkfall);
            fs.kratio = chem ? kf / kfall : kfall / kf;  // k0 / kinf
            fs.Pr = M * fs.kratio;
            // log10 Pr: ln [M] (formed once per run of reactions sharing [M])
            // + ln k0 - ln kinf where both rate constants are exponentials
            // (the packing's rule for RX_SAMELNM) and Pr >= 1e-300; else the
            // logarithm of the guarded Pr
            if (blend == BL_TROE || blend == BL_SRI) {
                double lnPr;
                if (has_lnkf && has_lnkfall) {
                    if (!(flags & RX_SAMELNM)) mc.logM = log(M);
                    lnPr = __double_as_longlong(fs.Pr) >= __double_as_longlong(SMALL)
                               ? mc.logM + (chem ? lnkf - lnkfall : lnkfall - lnkf)
                               : log(SMALL);
                } else {
                    lnPr = log(gsmall(fs.Pr));
                }
                fs.logPr = lnPr * INV_LN10;
            }
            if (blend == BL_TROE) {
                const double logPr = fs.logPr;
                const double ta = ldg(p + P_F0);
                fs.e1 = gexp(-1.0 * Tc * ldg(p + P_F1), et);
                fs.e3 = gexp(-1.0 * Tc * ldg(p + P_F3), et);
                double Fc = ta * fs.e1 + (1.0 + -1.0 * ta) * fs.e3;
                if (flags & RX_T2) {
                    fs.e2 = gexp(-1.0 * ldg(p + P_F2) * Tinv, et);
                    Fc = Fc + fs.e2;
                }
                fs.lnFc = log(gsmall(Fc));
                const double logFc = fs.lnFc * INV_LN10;
                fs.B = -1.1762 * logFc + -0.14 * logPr + 0.806;
                fs.A = -0.67 * logFc + logPr + -0.4;
                fs.Fc = Fc;
                const double B2 = fs.B * fs.B;
                fs.Fi = fexp(B2 / (fs.A * fs.A + B2) * fs.lnFc, et);
            } else if (blend == BL_SRI) {
                const double logPr = fs.logPr;
                fs.X = 1.0 / (logPr * logPr + 1.0);
                fs.e1 = gexp(-ldg(p + P_F1) * Tinv, et);
                fs.e3 = gexp(-Tc / ldg(p + P_F2), et);
                const double Q = ldg(p + P_F0) * fs.e1 + fs.e3;
                fs.lnQ = log(Q);
                double Fi = fexp(fs.X * fs.lnQ, et);
                if (flags & RX_SRID) Fi = Fi * ldg(p + P_F3);
                if (flags & RX_SRIE) {
                    const double e = ldg(p + P_F4);
                    const int ie = (int)e;
                    Fi = Fi * ((flags & RX_SRIEINT) ? (ie < 0 ? powi(Tinv, -ie) : powi(Tc, ie))
                                                    : pow(Tc, e));
                }
                fs.Fi = Fi;
            }
            ci = fs.Fi / (1.0 + fs.Pr);
            if (!chem) ci = ci * fs.Pr;
        }
    }
    double Rnet = rf;
    if (rev) Rnet = __dsub_rn(Rnet, rr);
    o.net = thd ? Rnet * ci : Rnet;
    if (!DER) return;

    const double T = sv.T, V = sv.V, P = sv.P, PoRT = sv.PoRT, rt_inv = sv.rt_inv;
    const bool conp = sv.conp;
    const double kr_ = rev ? kr : 0.0;
    double cg[PJG_MAXSP];
#pragma unroll
    for (int e = 0; e < PJG_MAXSP; ++e) cg[e] = e < nsp ? gsmall(conc[ent_spec(h.ent[e])]) : 1.0;
    // d R / d c_j for every participant j (dRopidnj :4169-4522)
    double gns = 0.0;
#pragma unroll
    for (int j = 0; j < PJG_MAXSP; ++j) {
        if (j >= nsp) break;
        const int nfj = ST::nuf(h, j), nrj = ST::nur(h, j);
        double gf = 0.0, gr = 0.0;
        if (nfj) {
            double S = nux(nfj, kf);
#pragma unroll
            for (int e = 0; e < PJG_MAXSP; ++e) {
                if (e >= nsp) break;
                S = mulpow(S, cg[e], ST::nuf(h, e) - (e == j));
            }
            gf = S;
        }
        if (rev && nrj) {
            double S = nux(nrj, kr_);
#pragma unroll
            for (int e = 0; e < PJG_MAXSP; ++e) {
                if (e >= nsp) break;
                S = mulpow(S, cg[e], ST::nur(h, e) - (e == j));
            }
            gr = S;
        }
        o.g[j] = gf - gr;
        if (ent_spec(h.ent[j]) == last) gns = o.g[j];
    }
    o.gns = gns;
    const double ci_ = thd ? ci : 1.0;
    o.ci_ = ci_;
    // fall-off derivative pieces shared by the n, T and E columns
    double inv1 = 0.0, dlnFi_dPr = 0.0;
    if (thd && blend != BL_NONE) {
        inv1 = 1.0 / (fs.Pr + 1.0);
        if (blend == BL_TROE) {
            const double absq = fs.A * fs.A + fs.B * fs.B;
            dlnFi_dPr = -2.0 * fs.A * fs.B * fs.lnFc * (0.14 * fs.A + fs.B) /
                        (gsmall(fs.Pr) * absq * absq * LN10);
        } else if (blend == BL_SRI) {
            dlnFi_dPr = -2.0 * fs.X * fs.X * fs.logPr / (gsmall(fs.Pr) * LN10) * fs.lnQ;
        }
    }
    // d ci / dx given d Pr / dx = Pr theta + theta_n and the direct part of d ln Fi / dx
    auto dci = [&](double theta, double theta_n, double direct) -> double {
        const double dPr = fs.Pr * theta + theta_n;
        double d = ci * (dlnFi_dPr * dPr + direct - dPr * inv1);
        if (!chem) d = d + theta * ci + fs.Fi * theta_n * inv1;
        return d;
    };
    const double dMfac = (thd && blend != BL_NONE) ? dci(0.0, fs.kratio, 0.0) : 1.0;
    o.X = Rnet * dMfac;
    const double mod = ldg(p + P_MOD);
    const bool hasns = flags & RX_HASNS;
    // temperature column (dRopi_dT :2589-3108, dci_*_dT :2117-2588)
    // rf dlnkf - rr (dlnkf - dB) = Rnet dlnkf + rr dB
    double d0 = rev ? fma(rr, dB, Rnet * dlnkf_dT) : rf * dlnkf_dT;
    d0 = d0 * ci_ * V;
    if (hasns) d0 += -gns * V * ci_ * PoRT * Tjinv;
    // extra-variable column (dRopi_dE :1458-1594, dci_*_dE :362-880)
    double d1 = 0.0;
    if (conp) {
        int nuf = -1, nur = -1;
#pragma unroll
        for (int e = 0; e < PJG_MAXSP; ++e) {
            if (e >= nsp) break;
            nuf += ST::nuf(h, e);
            nur += ST::nur(h, e);
        }
        d1 = (-nux(nuf, rf) + (rev ? nux(nur, rr) : 0.0)) * ci_;
    } else if (form >= FORM_PLOG) {
        d1 = V * ci_ * Rnet * dlnkf_dlnP / P;
    }
    if (hasns) d1 += gns * ci_ * (conp ? PoRT : V * rt_inv);
    if (thd) {
        const double dM = -1.0 * PoRT * mod * Tjinv;
        if (blend == BL_NONE) {
            d0 += dM * V * Rnet;
            if (conp) {
                if (thd != THD_UNITY) d1 += (mod * PoRT + -1.0 * M) * Rnet;
            } else {
                d1 += V * Rnet * mod * rt_inv;
            }
        } else {
            double b0, binf, Ta0, Tainf;
            if (!chem) {
                binf = ldg(p + P_B); Tainf = ldg(p + P_TA);
                b0 = ldg(p + P_FB); Ta0 = ldg(p + P_FTA);
            } else {
                b0 = ldg(p + P_B); Ta0 = ldg(p + P_TA);
                binf = ldg(p + P_FB); Tainf = ldg(p + P_FTA);
            }
            const double theta = Tjinv * (b0 + -1.0 * binf + (Ta0 + -1.0 * Tainf) * Tjinv);
            const double theta_n = dM * fs.kratio;
            double direct = 0.0;
            if (blend == BL_TROE) {
                const double absq = fs.A * fs.A + fs.B * fs.B;
                const double ta = ldg(p + P_F0), t1 = ldg(p + P_F1), t2 = ldg(p + P_F2),
                             t3 = ldg(p + P_F3);
                // the explicit T derivative uses the unclamped T, as the reference
                const bool same = T == Tc;
                const double x1 = same ? fs.e1 : gexp(-1.0 * T * t1, et);
                const double x3 = same ? fs.e3 : gexp(-1.0 * T * t3, et);
                double dFc = -1.0 * ta * t1 * x1 + (ta + -1.0) * t3 * x3;
                if (flags & RX_T2)
                    dFc += t2 * Tjinv * Tjinv * (same ? fs.e2 : gexp(-1.0 * t2 * Tjinv, et));
                direct = -fs.B * dFc *
                         (2.0 * fs.A * (1.1762 * fs.A + -0.67 * fs.B) * fs.lnFc - fs.B * absq * LN10) /
                         (fs.Fc * absq * absq * LN10);
            } else if (blend == BL_SRI) {
                const double sa = ldg(p + P_F0), sb = ldg(p + P_F1), sc = ldg(p + P_F2);
                const double Q = sa * fs.e1 + fs.e3;
                const double dQ = sa * sb * Tjinv * Tjinv * fs.e1 - fs.e3 / sc;
                direct = fs.X * dQ / Q + ldg(p + P_F4) * Tjinv;
            }
            d0 += dci(theta, theta_n, direct) * V * Rnet;
            const double modp = (conp ? (thd == THD_UNITY ? 0.0 : mod) * PoRT : mod * rt_inv) * fs.kratio;
            const double th = conp ? -1.0 * (thd != THD_UNITY) : 0.0;
            d1 += dci(th, modp, 0.0) * (conp ? 1.0 : V) * Rnet;
        }
    }
    o.d0 = d0;
    o.d1 = d1;
}

// ------------------------------------------------------------------------
// Reactions A + B <=> C + D (is_e22 in pjg_capi.cu: four distinct species
// with unit coefficients, reversible, Arrhenius form, no third body,
// nu_sum = 0), entries stored reactants first.  The same arithmetic as
// rxn_terms() for this case with every stoichiometric branch resolved at
// compile time: kr = kf exp(-sum nu b) (the (P_atm/R)^0 factor is 1),
// d R / d c_j is one product per participant, and ci = 1.
struct E22Head {
    int flags, bint;
    int s[4];  // reactant, reactant, product, product
    const double* p;
};

__device__ __forceinline__ void load_e22(const PjgRxn* R, E22Head& h)
{
    const int4 h0 = __ldg(reinterpret_cast<const int4*>(R));
    const int4 h1 = __ldg(reinterpret_cast<const int4*>(R) + 1);
    const uint4 e0 = __ldg(reinterpret_cast<const uint4*>(R) + 2);
    h.flags = h0.x;
    h.bint = h1.z;
    h.s[0] = ent_spec(e0.x);
    h.s[1] = ent_spec(e0.y);
    h.s[2] = ent_spec(e0.z);
    h.s[3] = ent_spec(e0.w);
    h.p = R->p;
}

struct E22Terms {
    double net;   // rate of progress
    double g[4];  // d net / d c_j of the four participants
    double gns;   // the same for the bath gas (0 if it does not take part)
    double d0, d1;
};

// the per-state values one elementary reaction reads (loaded ahead of use):
// concentrations, the 1 / Kc factors exp(b) of the reactants and exp(-b) of
// the products (in a split state; else the four b), d b / dT
struct E22Vals {
    double c[4], x[4], db[4];
};

template <bool DER, class ARR>
__device__ __forceinline__ void e22_fetch(const E22Head& h, bool split, const ARR& conc,
                                          const ARR& ep, const ARR& em, const ARR& db, E22Vals& v)
{
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        v.c[q] = conc[h.s[q]];
        v.x[q] = (q < 2 || !split) ? ep[h.s[q]] : em[h.s[q]];  // ep holds b if !split
        if (DER) v.db[q] = db[h.s[q]];
    }
}

template <bool DER>
__device__ __forceinline__ void e22_terms_v(const E22Head& h, const E22Vals& vv, int last,
                                            const StateVars& sv, E22Terms& o)
{
    const double* p = h.p;
    const double b = ldg(p + P_B), Ta = ldg(p + P_TA);
    const double kf = arrhenius(RX_FORM(h.flags), ldg(p + P_A), b, Ta, h.bint, sv.Tc, sv.logT,
                                sv.Tinv, sv.etab);
    double ikc;  // 1 / Kc = exp(-sum nu b)
    if (sv.split) {
        ikc = __dmul_rn(__dmul_rn(vv.x[0], vv.x[1]), __dmul_rn(vv.x[2], vv.x[3]));
    } else {
        const double Bsum = (vv.x[2] + vv.x[3]) - (vv.x[0] + vv.x[1]);
        ikc = fexp(-min_pos(EXP_MAX, Bsum), sv.etab);
    }
    const double kr = kf * ikc;
    const double c0 = vv.c[0], c1 = vv.c[1], c2 = vv.c[2], c3 = vv.c[3];
    // rounded products and difference (no contraction into an FMA): the rate
    // of progress must be the same in every kernel kind, whatever else uses
    // rf and rr (the Jacobian's rates equal the rates kernel's bit for bit)
    const double rf = __dmul_rn(__dmul_rn(kf, c0), c1), rr = __dmul_rn(__dmul_rn(kr, c2), c3);
    o.net = __dsub_rn(rf, rr);
    if (!DER) return;
    const double dlnkf_dT = (b + Ta * sv.Tjinv) * sv.Tjinv;
    const double dB = (vv.db[2] + vv.db[3]) - (vv.db[0] + vv.db[1]);
    o.g[0] = kf * gsmall(c1);
    o.g[1] = kf * gsmall(c0);
    o.g[2] = -(kr * gsmall(c3));
    o.g[3] = -(kr * gsmall(c2));
    double gns = 0.0;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (h.s[j] == last) gns = o.g[j];
    o.gns = gns;
    const bool hasns = h.flags & RX_HASNS;
    // rf dlnkf - rr (dlnkf - dB) = net dlnkf + rr dB
    double d0 = fma(rr, dB, o.net * dlnkf_dT) * sv.V;
    if (hasns) d0 += -gns * sv.V * sv.PoRT * sv.Tjinv;
    double d1 = sv.conp ? -rf + rr : 0.0;
    if (hasns) d1 += gns * (sv.conp ? sv.PoRT : sv.V * sv.rt_inv);
    o.d0 = d0;
    o.d1 = d1;
}

// ------------------------------------------------------------------------
// Other mass-action reactions without a third body, in a few fixed
// stoichiometric patterns (MaPattern below; pjg_capi.cu order_reactions packs
// each pattern's reactions together, entries in the pattern's order:
// reactants by coefficient, then species on both sides, then products by
// coefficient).  The arithmetic
// of rxn_terms() for such a reaction with every coefficient known at compile
// time.  Up to five entries.
template <bool REV, int F0, int R0, int F1, int R1, int F2 = 0, int R2 = 0, int F3 = 0, int R3 = 0,
          int F4 = 0, int R4 = 0>
struct MaPattern {
    static constexpr bool rev = REV;
    static constexpr int n = 2 + (F2 || R2) + (F3 || R3) + (F4 || R4);
    __host__ __device__ static constexpr int nuf(int e)
    {
        return e == 0 ? F0 : e == 1 ? F1 : e == 2 ? F2 : e == 3 ? F3 : F4;
    }
    __host__ __device__ static constexpr int nur(int e)
    {
        return e == 0 ? R0 : e == 1 ? R1 : e == 2 ? R2 : e == 3 ? R3 : R4;
    }
    __host__ __device__ static constexpr int sumf() { return F0 + F1 + F2 + F3 + F4; }
    __host__ __device__ static constexpr int sumr() { return R0 + R1 + R2 + R3 + R4; }
};

// the patterns, in the order their reactions are packed (kMaPatterns of them)
using MaP0 = MaPattern<false, 1, 0, 1, 0, 0, 1, 0, 1, 0, 1>;  // A + B => C + D + E
using MaP1 = MaPattern<true, 1, 0, 1, 0, 0, 1, 0, 1, 0, 1>;   // A + B <=> C + D + E
using MaP2 = MaPattern<true, 1, 0, 1, 0, 0, 2>;               // A + B <=> 2 C
using MaP3 = MaPattern<true, 2, 0, 0, 1, 0, 1>;               // 2 A <=> B + C
using MaP4 = MaPattern<true, 1, 0, 1, 0, 1, 0, 0, 1, 0, 1>;   // A + B + C <=> D + E
using MaP5 = MaPattern<true, 1, 0, 1, 0, 0, 1, 0, 2>;         // A + B <=> C + 2 D
using MaP6 = MaPattern<true, 1, 0, 2, 0, 0, 1, 0, 1>;         // A + 2 B <=> C + D
using MaP7 = MaPattern<false, 1, 0, 1, 0, 0, 1, 0, 1>;        // A + B => C + D
using MaP8 = MaPattern<true, 1, 0, 1, 1, 0, 1>;               // A + X <=> B + X
using MaP9 = MaPattern<true, 1, 0, 1, 0, 1, 1, 0, 1>;         // A + B + X <=> C + X
constexpr int kMaPatterns = 10;

// coefficient patterns of reactions with a third body or fall-off, evaluated
// by the general code (rxn_terms) compiled per pattern (PatStoich)
using TpP0 = MaPattern<true, 1, 0, 1, 0, 0, 1>;  // A + B (+M) <=> C
using TpP1 = MaPattern<true, 1, 0, 0, 1, 0, 1>;  // A (+M) <=> B + C
using TpP2 = MaPattern<true, 2, 0, 0, 1>;        // 2 A (+M) <=> B
constexpr int kTpPatterns = 3;

// acc * v^p for a compile-time p (0, 1 or 2), rounded products
template <int P>
__device__ __forceinline__ double mulpow_rn(double acc, double v)
{
    if (P == 0) return acc;
    if (P == 1) return __dmul_rn(acc, v);
    return __dmul_rn(acc, __dmul_rn(v, v));
}

struct MaTerms {
    double net;
    double g[5];
    double gns;
    double d0, d1;
};

template <class PT, bool DER, class ARR>
__device__ __forceinline__ void ma_terms(const RxnHead& h, int last, const StateVars& sv,
                                         const ARR& conc, const ARR& bk, const ARR& ep,
                                         const ARR& em, const ARR& db, MaTerms& o)
{
    constexpr int N = PT::n;
    const double* p = h.p;
    const double b = ldg(p + P_B), Ta = ldg(p + P_TA);
    const double kf = arrhenius(RX_FORM(h.flags), ldg(p + P_A), b, Ta, h.bint, sv.Tc, sv.logT,
                                sv.Tinv, sv.etab);
    int sp[N];
    double c[N];
#pragma unroll
    for (int e = 0; e < N; ++e) {
        sp[e] = ent_spec(h.ent[e]);
        c[e] = conc[sp[e]];
    }
    double kr = 0.0, dB = 0.0;
    if (PT::rev) {
        // the first term starts the sums (no addition to zero)
        bool first = true;
#pragma unroll
        for (int e = 0; e < N; ++e) {
            const int nu = PT::nur(e) - PT::nuf(e);
            if (nu == 0 || !DER) continue;
            dB = first ? nux(nu, db[sp[e]]) : addnu(dB, nu, db[sp[e]]);
            first = false;
        }
        double ikc;
        if (sv.split) {
            ikc = inv_kc_split<PatStoich<PT>>(h, ep, em);
        } else {
            double Bsum = 0.0;
            first = true;
#pragma unroll
            for (int e = 0; e < N; ++e) {
                const int nu = PT::nur(e) - PT::nuf(e);
                if (nu == 0) continue;
                Bsum = first ? nux(nu, bk[sp[e]]) : addnu(Bsum, nu, bk[sp[e]]);
                first = false;
            }
            ikc = fexp(-min_pos(EXP_MAX, Bsum), sv.etab);
        }
        kr = kf * ldg(p + P_PSUM) * ikc;
    }
    // rounded products and difference: the rate of progress is the same in
    // every kernel kind (see e22_terms)
    double rf = kf, rr = kr;
#pragma unroll
    for (int e = 0; e < N; ++e) {
        if (PT::nuf(e) == 1) rf = mulpow_rn<1>(rf, c[e]);
        if (PT::nuf(e) == 2) rf = mulpow_rn<2>(rf, c[e]);
        if (PT::rev && PT::nur(e) == 1) rr = mulpow_rn<1>(rr, c[e]);
        if (PT::rev && PT::nur(e) == 2) rr = mulpow_rn<2>(rr, c[e]);
    }
    o.net = PT::rev ? __dsub_rn(rf, rr) : rf;
    if (!DER) return;
    const double dlnkf_dT = (b + Ta * sv.Tjinv) * sv.Tjinv;
    double cg[N];
#pragma unroll
    for (int e = 0; e < N; ++e) cg[e] = gsmall(c[e]);
    double gns = 0.0;
#pragma unroll
    for (int j = 0; j < N; ++j) {
        double gf = 0.0, gr = 0.0;
        if (PT::nuf(j)) {
            double S = PT::nuf(j) == 2 ? kf + kf : kf;
#pragma unroll
            for (int e = 0; e < N; ++e) {
                const int q = PT::nuf(e) - (e == j);
                if (q == 1) S = S * cg[e];
                if (q == 2) S = S * (cg[e] * cg[e]);
            }
            gf = S;
        }
        if (PT::rev && PT::nur(j)) {
            double S = PT::nur(j) == 2 ? kr + kr : kr;
#pragma unroll
            for (int e = 0; e < N; ++e) {
                const int q = PT::nur(e) - (e == j);
                if (q == 1) S = S * cg[e];
                if (q == 2) S = S * (cg[e] * cg[e]);
            }
            gr = S;
        }
        o.g[j] = gf - gr;
        if (sp[j] == last) gns = o.g[j];
    }
    o.gns = gns;
    const bool hasns = h.flags & RX_HASNS;
    // rf dlnkf - rr (dlnkf - dB) = net dlnkf + rr dB
    double d0 = (PT::rev ? fma(rr, dB, o.net * dlnkf_dT) : rf * dlnkf_dT) * sv.V;
    if (hasns) d0 += -gns * sv.V * sv.PoRT * sv.Tjinv;
    double d1 = 0.0;
    if (sv.conp) d1 = -nux(PT::sumf() - 1, rf) + (PT::rev ? nux(PT::sumr() - 1, rr) : 0.0);
    if (hasns) d1 += gns * (sv.conp ? sv.PoRT : sv.V * sv.rt_inv);
    o.d0 = d0;
    o.d1 = d1;
}

}  // namespace pjg
