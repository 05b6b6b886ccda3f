// Fused FP64 species-rate and analytical-Jacobian kernels for sm_103a.
//
// One thread evaluates one thermochemical state end to end.  All threads of a
// warp walk the same reaction list, so mechanism records are read with
// warp-uniform addresses (broadcast loads, no divergence on reaction type);
// state data are laid out state-innermost so that every per-state access of a
// warp is one coalesced 256-byte transaction.
//
// Species rates restate pyJac's sub-kernel chain (pyjac/core/rate_subs.py
// get_specrates_kernel :3026-3278) as one pass over the reactions: forward rate
// (get_simple_arrhenius_rates :2642, PLOG :2084, Chebyshev :1904), third-body
// concentration (:1788), reduced pressure and Lindemann/Troe/SRI blending
// (:2251-2641), equilibrium constant and reverse rate (:1627), rates of progress
// (:1170-1509) and the net-production scatter (:1079), then molar, temperature and
// extra-variable rates (:709-1076).  Intermediates stay in registers instead of a
// global working buffer.
//
// The Jacobian restates create_jacobian.py (:285-4522) the same way: in the
// reaction pass each reaction adds its d(rop)/dn_j block, its third-body /
// fall-off terms and its T / extra-variable column terms; terms through the
// bath-gas concentration (the "_ns" kernels) are the same for every species
// column and are gathered per row; rows T and E are assembled afterwards from
// the species block (dTdot_dnj :3382, dEdot_dnj :3266, dTdotdT :1847,
// dEdotdT :2001, dTdotdE :1595, dEdotdE :1740).
//
// Numeric guards are the reference's (pyjac/core/instruction_creator.py:370-478):
// T clamped to [100, 10000] K for rate evaluation, V >= 1e-30, moles and
// concentrations in derivative products >= 1e-300, exp(min(x, 690.775527898)),
// log(max(x, 1e-300)).  As in the reference, the explicit T, V, P factors of the
// Jacobian blocks use the unclamped state values.
//
// FP64 instruction count is the cost that matters on GB300 (2 FP64 FMA per clock
// per SM): quotients of the NASA polynomials come precomputed in the species
// records, Troe's Fcent^(1/(1+(A/B)^2)) is exp(X ln Fcent) with ln Fcent shared
// with log10 Fcent, fall-off derivative factors are formed once per reaction,
// stoichiometric multiplications by +-1/+-2 are adds, and d(rop)/dc products
// skip zero exponents instead of dividing.
#include <cuda_runtime.h>
#include "pjg_eval.cuh"
#include "pjg_math.cuh"

using namespace pjg;

namespace {

// per-state array view: element k at base[k * stride]
struct SV {
    double* b;
    int64_t st;
    __device__ __forceinline__ double& operator[](int k) const { return b[(int64_t)k * st]; }
};

// nu * x for a warp-uniform small integer nu without an int->double conversion
__device__ __forceinline__ double nux(int nu, double x)
{
    switch (nu) {
    case 1: return x;
    case -1: return -x;
    case 2: return x + x;
    case -2: return -(x + x);
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

struct FallState {
    double Pr, Fi, A, B, Fc, lnFc, X, lnQ, kratio;
    double e1, e2, e3;   // Troe exponentials at the clamped temperature
};

#ifndef PJG_JAC_MINB
#define PJG_JAC_MINB 3  // resident 128-thread blocks per SM requested for the Jacobian kernel
#endif

template <int KIND>  // 0 species rates, 1 Jacobian, 2 J^T v
__global__ void __launch_bounds__(PJG_BLOCK, KIND == 1 ? PJG_JAC_MINB : (KIND == 2 ? 3 : 4))
    eval_kernel(const EvalArgs a)
{
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.n) return;  // no block-wide synchronisation below
    constexpr bool JAC = KIND == 1;
    constexpr bool VJP = KIND == 2;
    constexpr bool DER = KIND >= 1;  // derivative terms needed
    extern __shared__ double smem[];
    const int ns = a.ns, last = ns - 1;
    auto arr = [&](int which) -> SV {
        if (a.use_smem)
            return SV{smem + (int64_t)which * ns * blockDim.x + threadIdx.x, (int64_t)blockDim.x};
        return SV{a.scratch + (int64_t)which * ns * a.sc_ld + s, a.sc_ld};
    };
    SV conc = arr(ARR_CONC), bk = arr(ARR_B), wdot = arr(ARR_WDOT);
    SV db{nullptr, 0}, nsrow{nullptr, 0}, hw{nullptr, 0}, cpa{nullptr, 0}, dcpa{nullptr, 0},
        ha{nullptr, 0};
    if (DER) {
        db = arr(ARR_DB);
        nsrow = arr(ARR_NSROW);
        hw = arr(ARR_HW);
        cpa = arr(ARR_CP);
        dcpa = arr(ARR_DCP);
        ha = arr(ARR_H);
    }
    const bool conp = a.conp;
    const double* ph = a.phi + s * a.phi_ss;
    const double T = ph[0];
    const double Tc = fmin(10000.0, fmax(100.0, T));
    const double logT = log(Tc), Tinv = 1.0 / Tc;
    const double E = ph[a.phi_sj];
    const double prm = a.param[s];
    const double V = conp ? E : prm;
    const double P = conp ? prm : E;
    const double Vinv = 1.0 / fmax(1e-30, V);
    const double logP = a.need_logP ? log(P) : 0.0;
    const double Tjinv = DER ? 1.0 / T : 0.0;
    const double rt_inv = 1.0 / (RU * T);  // unclamped, as the reference's thd concentration
    const double PoRT = P * rt_inv;

    // concentrations (rate_subs.py get_concentrations :597-706)
    double nsum = 0.0;
    for (int k = 0; k < last; ++k) {
        const double nk = fmax(SMALL, ph[(int64_t)(2 + k) * a.phi_sj]);
        nsum = nsum + nk;
        conc[k] = nk * Vinv;
        wdot[k] = 0.0;
        if (DER) nsrow[k] = 0.0;
    }
    conc[last] = P / (RU * Tc) + -1.0 * fmax(SMALL, nsum) * Vinv;
    wdot[last] = 0.0;

    // thermo: Gibbs functions for Kc (+ derivatives and cp, h for the Jacobian)
    double h_ns = 0.0, cp_ns = 0.0, dcp_ns = 0.0;
    if (DER) {
        const Thermo tl = thermo<true>(a.sp + (int64_t)last * PJG_SP_DOUBLES, Tc, logT, Tinv, conp);
        h_ns = tl.h;
        cp_ns = tl.cp;
        dcp_ns = tl.dcp;
        for (int k = 0; k < ns; ++k) {
            const double* rec = a.sp + (int64_t)k * PJG_SP_DOUBLES;
            const Thermo t = k == last ? tl : thermo<true>(rec, Tc, logT, Tinv, conp);
            bk[k] = t.b;
            db[k] = t.db;
            ha[k] = t.h;
            if (k < last) {
                hw[k] = t.h - h_ns * ldg(rec + SP_MW);
                cpa[k] = t.cp;
                dcpa[k] = t.dcp;
            }
        }
    } else {
        for (int k = 0; k < ns; ++k)
            bk[k] = thermo<false>(a.sp + (int64_t)k * PJG_SP_DOUBLES, Tc, logT, Tinv, conp).b;
    }

    // J^T v: rows T and E of J are linear in the species rows, so v folds into
    // species weights vt_k = v_k + alpha * hw_k + beta * (1 - W_k/W_ns) known
    // before the reaction pass (cp_tot needs no rates); vt overwrites hw and the
    // species part of the product accumulates in nsrow.
    double vt_c0 = 0.0, v1 = 0.0, vout0 = 0.0, vout1 = 0.0, vNS = 0.0, cp_tot_v = 0.0;
    if (VJP) {
        const double* vv = a.v + s * a.phi_ss;
        const double v0 = vv[0];
        v1 = vv[a.phi_sj];
        double ct = 0.0;
        for (int k = 0; k < last; ++k) ct = fma(conc[k], cpa[k], ct);
        ct = fma(conc[last], cp_ns, ct);
        cp_tot_v = ct;
        const double extra = conp ? V : P, fixed = conp ? P : V;
        vt_c0 = v0 + v1 * extra * Tjinv;
        const double alpha = -vt_c0 / (V * ct), beta = v1 * T * RU / fixed;
        for (int k = 0; k < last; ++k) {
            const double omw = ldg(a.sp + (int64_t)k * PJG_SP_DOUBLES + SP_OMW);
            hw[k] = vv[(int64_t)(2 + k) * a.phi_sj] + alpha * hw[k] + beta * omw;
        }
    }

    // ---------------------------------------------------------------- reactions
    for (int i = 0; i < a.nr; ++i) {
        const PjgRxn* R = a.rxn + i;
        const int4 h0 = __ldg(reinterpret_cast<const int4*>(R));
        const int4 h1 = __ldg(reinterpret_cast<const int4*>(R) + 1);
        const int flags = h0.x, nsp = h0.y, thd_off = h0.z, thd_cnt = h0.w;
        const int auxo = h1.x, bint = h1.z, fbint = h1.w;
        unsigned ent[PJG_MAXSP];
        {
            const uint4 e0 = __ldg(reinterpret_cast<const uint4*>(R) + 2);
            const uint4 e1 = __ldg(reinterpret_cast<const uint4*>(R) + 3);
            ent[0] = e0.x; ent[1] = e0.y; ent[2] = e0.z; ent[3] = e0.w;
            ent[4] = e1.x; ent[5] = e1.y; ent[6] = e1.z; ent[7] = e1.w;
        }
        const double* p = R->p;
        const int form = RX_FORM(flags);
        const bool rev = flags & RX_REV;

        // forward rate constant and its log-derivatives
        double kf, dlnkf_dT = 0.0, dlnkf_dlnP = 0.0;
        if (form <= FORM_ARR) {
            kf = arrhenius(form, ldg(p + P_A), ldg(p + P_B), ldg(p + P_TA), bint, Tc, logT, Tinv);
            if (DER) dlnkf_dT = (ldg(p + P_B) + ldg(p + P_TA) * Tjinv) * Tjinv;
        } else if (form == FORM_PLOG) {
            kf = gexp(plog_logk(a.aux + auxo, logT, Tinv, logP, Tjinv, &dlnkf_dT, &dlnkf_dlnP));
        } else {
            const double l10 = cheb_log10k(a.aux + auxo, Tinv, logP, Tjinv, &dlnkf_dT, &dlnkf_dlnP);
            kf = exp(LN10 * fmin(EXP_MAX, l10));
            dlnkf_dT *= LN10;
            dlnkf_dlnP *= LN10;
        }
        // reverse rate: kr = kf / Kc, Kc = (P_atm/R)^nu_sum exp(sum nu b)
        double kr = 0.0, dB = 0.0;
        if (rev) {
            double Bsum = 0.0;
#pragma unroll
            for (int e = 0; e < PJG_MAXSP; ++e) {
                if (e >= nsp) break;
                const int nu = ent_nur(ent[e]) - ent_nuf(ent[e]);
                if (nu != 0) {
                    Bsum = addnu(Bsum, nu, bk[ent_spec(ent[e])]);
                    if (DER) dB = addnu(dB, nu, db[ent_spec(ent[e])]);
                }
            }
            kr = kf * ldg(p + P_PSUM) * exp(-fmin(EXP_MAX, Bsum));
        }
        // rates of progress (mass action on raw concentrations)
        double rf = kf, rr = kr;
#pragma unroll
        for (int e = 0; e < PJG_MAXSP; ++e) {
            if (e >= nsp) break;
            const double c = conc[ent_spec(ent[e])];
            rf = mulpow(rf, c, ent_nuf(ent[e]));
            if (rev) rr = mulpow(rr, c, ent_nur(ent[e]));
        }
        // third-body / fall-off pressure modification
        const int thd = RX_THD(flags);
        const int blend = RX_BLEND(flags);
        const bool chem = flags & RX_CHEM;
        double ci = 1.0, M = 0.0;
        FallState fs;
        fs.Pr = 0.0; fs.Fi = 1.0; fs.A = 0.0; fs.B = 0.0; fs.Fc = 1.0; fs.lnFc = 0.0; fs.X = 0.0;
        fs.lnQ = 0.0; fs.kratio = 0.0; fs.e1 = 0.0; fs.e2 = 0.0; fs.e3 = 0.0;
        if (thd) {
            M = PoRT * ldg(p + P_FLAG);
            for (int l = 0; l < thd_cnt; ++l)
                M = fma(__ldg(a.thd_coef + thd_off + l), conc[__ldg(a.thd_spec + thd_off + l)], M);
            if (blend == BL_NONE) {
                ci = M;
            } else {
                const double kfall = arrhenius(RX_FFORM(flags), ldg(p + P_FA), ldg(p + P_FB),
                                               ldg(p + P_FTA), fbint, Tc, logT, Tinv);
                fs.kratio = chem ? kf / kfall : kfall / kf;  // k0 / kinf
                fs.Pr = M * fs.kratio;
                if (blend == BL_TROE) {
                    const double logPr = log(fmax(SMALL, fs.Pr)) * INV_LN10;
                    const double ta = ldg(p + P_F0);
                    fs.e1 = gexp(-1.0 * Tc * ldg(p + P_F1));
                    fs.e3 = gexp(-1.0 * Tc * ldg(p + P_F3));
                    double Fc = ta * fs.e1 + (1.0 + -1.0 * ta) * fs.e3;
                    if (flags & RX_T2) {
                        fs.e2 = gexp(-1.0 * ldg(p + P_F2) * Tinv);
                        Fc = Fc + fs.e2;
                    }
                    fs.lnFc = log(fmax(SMALL, Fc));
                    const double logFc = fs.lnFc * INV_LN10;
                    fs.B = -1.1762 * logFc + -0.14 * logPr + 0.806;
                    fs.A = -0.67 * logFc + logPr + -0.4;
                    fs.Fc = Fc;
                    const double B2 = fs.B * fs.B;
                    fs.Fi = exp(B2 / (fs.A * fs.A + B2) * fs.lnFc);
                } else if (blend == BL_SRI) {
                    const double logPr = log(fmax(SMALL, fs.Pr)) * INV_LN10;
                    fs.X = 1.0 / (logPr * logPr + 1.0);
                    fs.e1 = gexp(-ldg(p + P_F1) * Tinv);
                    fs.e3 = gexp(-Tc / ldg(p + P_F2));
                    const double Q = ldg(p + P_F0) * fs.e1 + fs.e3;
                    fs.lnQ = log(Q);
                    double Fi = exp(fs.X * fs.lnQ);
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
        if (rev) Rnet = Rnet + -1.0 * rr;
        const double net = thd ? Rnet * ci : Rnet;
        {
            // participants are distinct species: load all, then update
            double wv[PJG_MAXSP];
#pragma unroll
            for (int e = 0; e < PJG_MAXSP; ++e)
                if (e < nsp) wv[e] = wdot[ent_spec(ent[e])];
#pragma unroll
            for (int e = 0; e < PJG_MAXSP; ++e) {
                if (e >= nsp) break;
                wdot[ent_spec(ent[e])] = addnu(wv[e], ent_nur(ent[e]) - ent_nuf(ent[e]), net);
            }
        }
        if (!DER) continue;

        // ------------------------------------------------- Jacobian terms
        const int* slots = JAC ? a.rxn_slots + __ldg(a.rxn_slot_off + i) : nullptr;
        const double kr_ = rev ? kr : 0.0;
        double cg[PJG_MAXSP];
#pragma unroll
        for (int e = 0; e < PJG_MAXSP; ++e) cg[e] = e < nsp ? gsmall(conc[ent_spec(ent[e])]) : 1.0;
        // d R / d c_j for every participant j (dRopidnj :4169-4522)
        double g[PJG_MAXSP];
        double gns = 0.0;
#pragma unroll
        for (int j = 0; j < PJG_MAXSP; ++j) {
            if (j >= nsp) break;
            const int nfj = ent_nuf(ent[j]), nrj = ent_nur(ent[j]);
            double gf = 0.0, gr = 0.0;
            if (nfj) {
                double S = nux(nfj, kf);
#pragma unroll
                for (int e = 0; e < PJG_MAXSP; ++e) {
                    if (e >= nsp) break;
                    S = mulpow(S, cg[e], ent_nuf(ent[e]) - (e == j));
                }
                gf = S;
            }
            if (rev && nrj) {
                double S = nux(nrj, kr_);
#pragma unroll
                for (int e = 0; e < PJG_MAXSP; ++e) {
                    if (e >= nsp) break;
                    S = mulpow(S, cg[e], ent_nur(ent[e]) - (e == j));
                }
                gr = S;
            }
            g[j] = gf - gr;
            if (ent_spec(ent[j]) == last) gns = g[j];
        }
        const bool hasns = flags & RX_HASNS;
        const double ci_ = thd ? ci : 1.0;
        // fall-off derivative pieces shared by the n, T and E columns
        double inv1 = 0.0, dlnFi_dPr = 0.0;
        if (thd && blend != BL_NONE) {
            inv1 = 1.0 / (fs.Pr + 1.0);
            if (blend == BL_TROE) {
                const double absq = fs.A * fs.A + fs.B * fs.B;
                dlnFi_dPr = -2.0 * fs.A * fs.B * fs.lnFc * (0.14 * fs.A + fs.B) /
                            (fmax(SMALL, fs.Pr) * absq * absq * LN10);
            } else if (blend == BL_SRI) {
                const double logPr = log(fmax(SMALL, fs.Pr)) * INV_LN10;
                dlnFi_dPr = -2.0 * fs.X * fs.X * logPr / (fmax(SMALL, fs.Pr) * LN10) * fs.lnQ;
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
        const double X = Rnet * dMfac;
        const double mod = ldg(p + P_MOD);
        // temperature column (dRopi_dT :2589-3108, dci_*_dT :2117-2588)
        double d0 = rf * dlnkf_dT;
        if (rev) d0 = d0 + -1.0 * rr * (dlnkf_dT + -1.0 * dB);
        d0 = d0 * ci_ * V;
        if (hasns) d0 += -gns * V * ci_ * PoRT * Tjinv;
        // extra-variable column (dRopi_dE :1458-1594, dci_*_dE :362-880)
        double d1 = 0.0;
        if (conp) {
            int nuf = -1, nur = -1;
#pragma unroll
            for (int e = 0; e < PJG_MAXSP; ++e) {
                if (e >= nsp) break;
                nuf += ent_nuf(ent[e]);
                nur += ent_nur(ent[e]);
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
                    const double x1 = same ? fs.e1 : gexp(-1.0 * T * t1);
                    const double x3 = same ? fs.e3 : gexp(-1.0 * T * t3);
                    double dFc = -1.0 * ta * t1 * x1 + (ta + -1.0) * t3 * x3;
                    if (flags & RX_T2) dFc += t2 * Tjinv * Tjinv * (same ? fs.e2 : gexp(-1.0 * t2 * Tjinv));
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
        const double cns = ldg(p + P_CNS);
        const bool nslist = flags & RX_NSLIST;
        if (VJP) {
            // w = sum_k nu_k vt_k over the species rows of this reaction
            double w = 0.0;
#pragma unroll
            for (int ka = 0; ka < PJG_MAXSP; ++ka) {
                if (ka >= nsp) break;
                const int k = ent_spec(ent[ka]);
                if (k == last) continue;
                w = addnu(w, ent_nur(ent[ka]) - ent_nuf(ent[ka]), hw[k]);
            }
            if (w != 0.0) {
                const double wc = w * ci_;
                double vo[PJG_MAXSP];
#pragma unroll
                for (int jb = 0; jb < PJG_MAXSP; ++jb)
                    if (jb < nsp && ent_spec(ent[jb]) != last) vo[jb] = nsrow[ent_spec(ent[jb])];
#pragma unroll
                for (int jb = 0; jb < PJG_MAXSP; ++jb) {
                    if (jb >= nsp) break;
                    if (ent_spec(ent[jb]) != last) nsrow[ent_spec(ent[jb])] = fma(wc, g[jb], vo[jb]);
                }
                if (hasns) vNS = fma(wc, gns, vNS);
                if (thd) {
                    const double wx = w * X;
                    for (int l = 0; l < thd_cnt; ++l) {
                        const int j = __ldg(a.thd_spec + thd_off + l);
                        if (j != last) nsrow[j] = fma(__ldg(a.thd_coef + thd_off + l), wx, nsrow[j]);
                    }
                    if (nslist) vNS = fma(cns, wx, vNS);
                }
                vout0 = fma(w, d0, vout0);
                vout1 = fma(w, d1, vout1);
            }
            continue;
        }
        // scatter into the species rows of this reaction
#pragma unroll
        for (int ka = 0; ka < PJG_MAXSP; ++ka) {
            if (ka >= nsp) break;
            const int k = ent_spec(ent[ka]);
            if (k == last) continue;
            const int nuk = ent_nur(ent[ka]) - ent_nuf(ent[ka]);
            if (nuk == 0) continue;
            // all loads of this row's accumulators first, so they are in flight together
            double* ap[PJG_MAXSP + 2];
            double av[PJG_MAXSP + 2];
#pragma unroll
            for (int jb = 0; jb < PJG_MAXSP + 2; ++jb) {
                if (jb >= nsp + 2) break;
                const int sl = jb < nsp ? __ldg(slots + ka * nsp + jb)
                                        : __ldg(slots + nsp * nsp + 2 * ka + (jb - nsp));
                ap[jb] = sl >= 0 ? a.acc + (int64_t)sl * a.acc_ld + s : nullptr;
                av[jb] = sl >= 0 ? *ap[jb] : 0.0;
            }
#pragma unroll
            for (int jb = 0; jb < PJG_MAXSP; ++jb) {
                if (jb >= nsp) break;
                if (ap[jb]) *ap[jb] = addnu(av[jb], nuk, g[jb] * ci_);
            }
            if (ap[nsp]) *ap[nsp] = addnu(av[nsp], nuk, d0);
            if (ap[nsp + 1]) *ap[nsp + 1] = addnu(av[nsp + 1], nuk, d1);
            double nsacc = 0.0;
            if (hasns) nsacc = gns * ci_;
            if (thd) {
                const double wx = nux(nuk, X);
                for (int l = 0; l < thd_cnt; ++l) {
                    const int sl = __ldg(slots + nsp * nsp + 2 * nsp + l * nsp + ka);
                    if (sl >= 0) {
                        double& r = a.acc[(int64_t)sl * a.acc_ld + s];
                        r = fma(__ldg(a.thd_coef + thd_off + l), wx, r);
                    }
                }
                if (nslist) nsacc = fma(cns, X, nsacc);
            }
            if (hasns || (thd && nslist)) nsrow[k] = addnu(nsrow[k], nuk, nsacc);
        }
    }

    // ------------------------------------------- temperature and E rates
    double upper = 0.0, lower = 0.0;
    if (DER) {
        for (int k = 0; k < last; ++k) {
            lower = fma(conc[k], cpa[k], lower);
            upper = fma(ha[k], wdot[k], upper);
        }
        lower = fma(conc[last], cp_ns, lower);
        upper = fma(h_ns, wdot[last], upper);
    } else {
        for (int k = 0; k < ns; ++k) {
            const Thermo t = thermo<false>(a.sp + (int64_t)k * PJG_SP_DOUBLES, Tc, logT, Tinv, conp);
            lower = fma(conc[k], t.cp, lower);
            upper = fma(t.h, wdot[k], upper);
        }
    }
    const double Tdot = 0.0 + -1.0 * upper / lower;
    double dE = 0.0;
    for (int k = 0; k < last; ++k)
        dE = fma(ldg(a.sp + (int64_t)k * PJG_SP_DOUBLES + SP_OMW), wdot[k], dE);
    const double Vval = fmax(1e-30, V);
    double Edot;
    if (conp) {
        Edot = Vval * Tdot / Tc;
        Edot = Edot + Vval * dE * Tc * RU / P;
    } else {
        Edot = P * Tdot / Tc;
        Edot = Edot + Tc * RU * dE;
    }
    if (a.dphi) {
        double* o = a.dphi + s * a.dphi_ss;
        o[0] = Tdot;
        o[a.dphi_sj] = Edot;
        for (int k = 0; k < last; ++k) o[(int64_t)(2 + k) * a.dphi_sj] = Vval * wdot[k];
    }
    if (VJP) {
        // constant parts of columns T and E (from rows T, E of dTdot_dT :1847,
        // dEdotdT :2001, dTdotdE :1595, dEdotdE :1740) and the species columns'
        // bath-gas and d cp_tot / dn_j terms
        const double extra = conp ? V : P;
        double dTsum = (cp_ns * Tjinv - dcp_ns) * conc[last];
        double wsum = 0.0, omws = 0.0, dTsum1 = 0.0, hws = 0.0;
        for (int k = 0; k < last; ++k) {
            const double* rec = a.sp + (int64_t)k * PJG_SP_DOUBLES;
            const double mw = ldg(rec + SP_MW), omw = ldg(rec + SP_OMW);
            const double wk = wdot[k], ck = conc[k], cpk = cpa[k];
            dTsum = dTsum + (cp_ns * Tjinv - dcpa[k]) * ck;
            wsum = wsum + wk * (-cpk + mw * cp_ns);
            omws = fma(omw, wk, omws);
            dTsum1 = dTsum1 + (cpk - cp_ns) * ck;
            hws = fma(ha[k] - h_ns * mw, wk, hws);
        }
        const double ct = cp_tot_v;
        double C0 = vt_c0 * (Tdot * dTsum + wsum) / ct - v1 * extra * Tdot * Tjinv * Tjinv +
                    v1 * RU * (conp ? V / P : 1.0) * omws;
        double C1 = conp ? vt_c0 * (Tdot * dTsum1 + hws) / (ct * V)
                         : -vt_c0 * Tdot * cp_ns * rt_inv / ct;
        C1 += v1 * Tdot * Tjinv;
        const double gam = -vt_c0 * Tdot / (V * ct);
        double* o = a.vjp + s * a.phi_ss;
        o[0] = vout0 + C0;
        o[a.phi_sj] = vout1 + C1;
        for (int j = 0; j < last; ++j)
            o[(int64_t)(2 + j) * a.phi_sj] = nsrow[j] - vNS + gam * (cpa[j] - cp_ns);
        return;
    }
    if (!JAC) return;

    // ------------------------------------------- assemble rows T and E
    double* acc = a.acc + s;
    const int64_t ld = a.acc_ld;
    // bath-gas terms: subtract the per-row sums from every species column
    for (int k = 0; k < last; ++k) {
        const double v = nsrow[k];
        if (v == 0.0) continue;
        const int r0 = __ldg(a.row_off + k), r1 = __ldg(a.row_off + k + 1);
        for (int q = r0; q < r1; ++q) {
            const int2 e = __ldg(a.row_list + q);
            acc[(int64_t)e.y * ld] -= v;
        }
    }
    const double cp_tot = lower;
    const double fixed = conp ? P : V, extra = conp ? V : P;
    const double inv_vcp = 1.0 / (V * cp_tot);
    const double TRf = T * RU / fixed, eTj = extra * Tjinv;
    for (int j = 0; j < last; ++j) {
        double sum = 0.0, sumE = 0.0;
        const int c0 = __ldg(a.col_off + j), c1 = __ldg(a.col_off + j + 1);
        for (int q = c0; q < c1; ++q) {
            const int2 e = __ldg(a.col_list + q);
            const double Jkj = acc[(int64_t)e.y * ld];
            sum = fma(hw[e.x], Jkj, sum);
            sumE = fma(ldg(a.sp + (int64_t)e.x * PJG_SP_DOUBLES + SP_OMW), Jkj, sumE);
        }
        const double J0 = -1.0 * (sum + Tdot * (cpa[j] + -1.0 * cp_ns)) * inv_vcp;
        acc[(int64_t)__ldg(a.cj_slots + 2 * j) * ld] = J0;
        acc[(int64_t)__ldg(a.cj_slots + 2 * j + 1) * ld] = TRf * sumE + eTj * J0;
    }
    // T column of rows T, E and E column of rows T, E
    double dTsum = (cp_ns * Tjinv - dcp_ns) * conc[last];
    double rate_sum = 0.0, sumT = 0.0, sumE1 = 0.0, spec1 = 0.0, dTsum1 = 0.0;
    const double Vjinv = 1.0 / V;
    for (int k = 0; k < last; ++k) {
        const double* rec = a.sp + (int64_t)k * PJG_SP_DOUBLES;
        const double mw = ldg(rec + SP_MW), omw = ldg(rec + SP_OMW);
        const int sl0 = __ldg(a.sp_slots + 2 * k), sl1 = __ldg(a.sp_slots + 2 * k + 1);
        const double Jk0 = sl0 >= 0 ? acc[(int64_t)sl0 * ld] : 0.0;
        const double Jk1 = sl1 >= 0 ? acc[(int64_t)sl1 * ld] : 0.0;
        const double wk = wdot[k], ck = conc[k], cpk = cpa[k], hwk = hw[k];
        rate_sum = rate_sum + Vjinv * Jk0 * (-1.0 * hwk);
        rate_sum = rate_sum + wk * (-cpk + mw * cp_ns);
        dTsum = dTsum + (cp_ns * Tjinv - dcpa[k]) * ck;
        if (conp) {
            sumT = sumT + omw * (Vjinv * Jk0 + Tjinv * wk);
            spec1 = spec1 + hwk * (Jk1 - wk);
            dTsum1 = dTsum1 + (cpk - cp_ns) * ck;
        } else {
            sumT = sumT + omw * (Jk0 * (T * Vjinv) + wk);
            spec1 = spec1 + hwk * Jk1;
        }
        sumE1 = fma(omw, Jk1, sumE1);
    }
    const double inv_cp = 1.0 / cp_tot;
    const double J00 = (Tdot * dTsum + rate_sum) * inv_cp;
    double J10;
    if (conp) {
        J10 = V * Tjinv * (J00 - Tjinv * Tdot);
        J10 = J10 + RU * T * V * sumT / P;
    } else {
        J10 = P * (J00 - Tdot * Tjinv) * Tjinv;
        J10 = J10 + RU * sumT;
    }
    double J01;
    if (conp) {
        J01 = (Tdot * dTsum1 - spec1) * inv_vcp;
    } else {
        J01 = -((Tdot * cp_ns * rt_inv) * inv_cp);
        J01 = J01 - (spec1 * Vjinv) * inv_cp;
    }
    double J11 = TRf * sumE1;
    J11 = J11 + (extra * J01 + Tdot) * Tjinv;
    acc[(int64_t)a.s00 * ld] = J00;
    acc[(int64_t)a.s10 * ld] = J10;
    acc[(int64_t)a.s01 * ld] = J01;
    acc[(int64_t)a.s11 * ld] = J11;
}

}  // namespace

int pjg_launch_eval(const EvalArgs& a, int kind, void* stream, size_t smem_bytes)
{
    if (a.n <= 0) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned grid = (unsigned)((a.n + PJG_BLOCK - 1) / PJG_BLOCK);
    if (kind == 1) {
        if (smem_bytes > 48 * 1024)
            cudaFuncSetAttribute(eval_kernel<1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem_bytes);
        eval_kernel<1><<<grid, PJG_BLOCK, smem_bytes, st>>>(a);
    } else if (kind == 2) {
        if (smem_bytes > 48 * 1024)
            cudaFuncSetAttribute(eval_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem_bytes);
        eval_kernel<2><<<grid, PJG_BLOCK, smem_bytes, st>>>(a);
    } else {
        if (smem_bytes > 48 * 1024)
            cudaFuncSetAttribute(eval_kernel<0>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)smem_bytes);
        eval_kernel<0><<<grid, PJG_BLOCK, smem_bytes, st>>>(a);
    }
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}
