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
#include "pjg_rxn.cuh"

using namespace pjg;

namespace {

// per-state array view: element k at base[k * stride]
struct SV {
    double* b;
    int64_t st;
    __device__ __forceinline__ double& operator[](int k) const { return b[(int64_t)k * st]; }
};

#ifndef PJG_VJP_MINB
#define PJG_VJP_MINB 3  // resident 128-thread blocks per SM requested for the J^T v kernel
#endif

#ifndef PJG_JAC_MINB
#define PJG_JAC_MINB 4  // resident 128-thread blocks per SM requested for the Jacobian kernel
#endif

// Species-rate kernel: 6 blocks per SM fit its 80 registers without spills.
// Measured on 1M GRI states (F): 4 blocks 22.35 ms, 5: 22.34, 6: 21.86, 8:
// 21.75 (64 registers, with spills); the Jacobian at 5 blocks 68.7 against
// 68.2 ms at 4, J^T v at 4 blocks 13.8 against 13.6 ms at 3.
#ifndef PJG_RATES_MINB
#define PJG_RATES_MINB 6  // resident 128-thread blocks per SM requested for the species-rate kernel
#endif

// Rows T and E of the output and the bath-gas terms of its species block
// (the assembly step of eval_kernel<1>), out of line so that its registers do
// not shape the reaction loops' allocation.  One pass over the species block
// in chunks of kCols columns whose row-T and row-E sums stay in registers,
// visiting only the rows with a structurally nonzero entry in the chunk
// (dchunk_list; GRI: 1,774 of 2,704 entries).  A row's entries are loaded
// together, have the row's bath-gas sum subtracted (stored back only then)
// and are summed into their columns' sums in increasing row order.  Slots:
// (2 + k) rs + (2 + j) cs for a dense output, dchunk_slots (one quadruple per
// listed row) and cj_slots for a sparse one.  Software-pipelined: the next
// listed row's entries and weights are loaded before this row's are summed.
// Measured on 1M GRI states (dense F): chunks of 4 columns 92.1 ms, 6: 92.8,
// 8: 93.3, 10: 96.1, 16: 101.1 (register pressure), against 96.3 ms for two
// passes (subtract, then sum); loads and stores interleaved entry by entry
// serialised on possible aliasing (100.4 ms).  Later, with the row lists
// 70.3 ms against every entry visited, pipelined 68.35 against 69.11 ms, out
// of line 68.3 against 68.4 ms inlined.
__device__ __noinline__ void rows_te(bool sparse, double* acc, int64_t ld, int rs, int cs,
                                     const int* dchunk_off, const int* dchunk_list,
                                     const int4* dchunk_slots, const int* cj_slots,
                                     const double* sp, SV nsrow, SV hw, SV cpa, int last,
                                     double cp_ns, double Tdot, double inv_vcp, double TRf,
                                     double eTj)
{
    constexpr int kCols = PJG_DENSE_COLS;
    static_assert(kCols == 4, "one int4 of slots per listed row");
    for (int c = 0, j0 = 0; j0 < last; ++c, j0 += kCols) {
        double sT[kCols], sE[kCols];
#pragma unroll
        for (int q = 0; q < kCols; ++q) {
            sT[q] = 0.0;
            sE[q] = 0.0;
        }
        auto fetch = [&](int t, int e, double (&J)[kCols], int (&sl)[kCols], double& v_,
                         double& hw_, double& om_) {
            const int k = e >> 4, mask = e & 15;
            if (sparse) {
                const int4 q4 = __ldg(dchunk_slots + t);
                sl[0] = q4.x;
                sl[1] = q4.y;
                sl[2] = q4.z;
                sl[3] = q4.w;
            } else {
#pragma unroll
                for (int q = 0; q < kCols; ++q) sl[q] = (2 + k) * rs + (2 + j0 + q) * cs;
            }
#pragma unroll
            for (int q = 0; q < kCols; ++q)
                J[q] = (mask >> q & 1) ? __ldcg(acc + (int64_t)sl[q] * ld) : 0.0;
            v_ = __ldcg(&nsrow[k]);
            hw_ = hw[k];
            om_ = ldg(sp + (int64_t)k * PJG_SP_DOUBLES + SP_OMW);
        };
        int t = __ldg(dchunk_off + c);
        const int t1 = __ldg(dchunk_off + c + 1);
        int en = 0;
        int sln[kCols] = {0, 0, 0, 0};
        double Jn[kCols], vn = 0.0, hwn = 0.0, omn = 0.0;
        if (t < t1) {
            en = __ldg(dchunk_list + t);  // the same for every thread
            fetch(t, en, Jn, sln, vn, hwn, omn);
        }
        for (; t < t1; ++t) {
            const int mask = en & 15;
            double Jv[kCols];
            int sl[kCols];
#pragma unroll
            for (int q = 0; q < kCols; ++q) {
                Jv[q] = Jn[q];
                sl[q] = sln[q];
            }
            const double v = vn, hwk = hwn, omk = omn;
            if (t + 1 < t1) {
                en = __ldg(dchunk_list + t + 1);
                fetch(t + 1, en, Jn, sln, vn, hwn, omn);
            }
            if (mask == (1 << kCols) - 1) {
                if (nonzero(v)) {
#pragma unroll
                    for (int q = 0; q < kCols; ++q) {
                        Jv[q] = Jv[q] - v;
                        acc[(int64_t)sl[q] * ld] = Jv[q];
                    }
                }
#pragma unroll
                for (int q = 0; q < kCols; ++q) {
                    sT[q] = fma(hwk, Jv[q], sT[q]);
                    sE[q] = fma(omk, Jv[q], sE[q]);
                }
            } else {
                if (nonzero(v)) {
#pragma unroll
                    for (int q = 0; q < kCols; ++q) {
                        if (mask >> q & 1) {
                            Jv[q] = Jv[q] - v;
                            acc[(int64_t)sl[q] * ld] = Jv[q];
                        }
                    }
                }
#pragma unroll
                for (int q = 0; q < kCols; ++q) {
                    if (mask >> q & 1) {
                        sT[q] = fma(hwk, Jv[q], sT[q]);
                        sE[q] = fma(omk, Jv[q], sE[q]);
                    }
                }
            }
        }
#pragma unroll
        for (int q = 0; q < kCols; ++q) {
            const int j = j0 + q;
            if (j < last) {
                const int s0 = sparse ? __ldg(cj_slots + 2 * j) : (2 + j) * cs;
                const int s1 = sparse ? __ldg(cj_slots + 2 * j + 1) : rs + (2 + j) * cs;
                const double J0 = -1.0 * (sT[q] + Tdot * (cpa[j] + -1.0 * cp_ns)) * inv_vcp;
                acc[(int64_t)s0 * ld] = J0;
                acc[(int64_t)s1 * ld] = TRf * sE[q] + eTj * J0;
            }
        }
    }
}

template <int KIND>  // 0 species rates, 1 Jacobian, 2 J^T v
__global__ void __launch_bounds__(PJG_BLOCK, KIND == 1 ? PJG_JAC_MINB : (KIND == 2 ? PJG_VJP_MINB : PJG_RATES_MINB))
    eval_kernel(const EvalArgs a)
{
    __shared__ double etab[PJG_EXP_TAB];
    fill_exp_table(etab);
    __syncthreads();
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= a.n) return;  // no block-wide synchronisation below
    constexpr bool JAC = KIND == 1;
    constexpr bool VJP = KIND == 2;
    constexpr bool DER = KIND >= 1;  // derivative terms needed
    const int ns = a.ns, last = ns - 1;
    auto arr = [&](int which) -> SV {
        return SV{a.scratch + (int64_t)which * ns * a.sc_ld + s, a.sc_ld};
    };
    // ep holds b_k until the state's split is known (then exp(b_k) if it
    // holds); the per-reaction fallback reads b_k from it as bk
    SV conc = arr(ARR_CONC), ep = arr(ARR_EP), em = arr(ARR_EM), wdot = arr(ARR_WDOT);
    const SV& bk = ep;
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
    // The per-state arrays live in global scratch (state-innermost, so a
    // warp's accesses are coalesced) and stay in L1/L2: shared memory would
    // hold too few states per SM to keep the FP64 pipe busy.  Accumulators
    // take fire-and-forget reductions, performed in L2, and are read back
    // from L2 after a fence.
    auto accum = [&](const SV& v, int k, double x) { atomicAdd(&v[k], x); };
    auto rd = [&](const SV& v, int k) -> double { return __ldcg(&v[k]); };
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
    StateVars sv;
    sv.T = T; sv.Tc = Tc; sv.logT = logT; sv.Tinv = Tinv; sv.Tjinv = Tjinv;
    sv.V = V; sv.P = P; sv.PoRT = PoRT; sv.rt_inv = rt_inv; sv.logP = logP; sv.conp = conp;
    sv.etab = etab;

    // concentrations (rate_subs.py get_concentrations :597-706)
    double nsum = 0.0;
    for (int k = 0; k < last; ++k) {
        const double nk = gsmall(ph[(int64_t)(2 + k) * a.phi_sj]);
        nsum = nsum + nk;
        conc[k] = nk * Vinv;
        wdot[k] = 0.0;
        if (DER) nsrow[k] = 0.0;
    }
    conc[last] = P / (RU * Tc) + -1.0 * gsmall(nsum) * Vinv;
    wdot[last] = 0.0;

    // thermo: Gibbs functions for Kc (+ derivatives and cp, h for the Jacobian),
    // and their exponentials, the factors of 1 / Kc (StateVars::split)
    double h_ns = 0.0, cp_ns = 0.0, dcp_ns = 0.0;
    bool split = true;
    auto gibbs = [&](int k, double b) {
        ep[k] = b;
        split = split && abs_le(b, a.kc_split_max);
    };
    if (DER) {
        const Thermo tl = thermo<true>(a.sp + (int64_t)last * PJG_SP_DOUBLES, Tc, logT, Tinv, conp);
        h_ns = tl.h;
        cp_ns = tl.cp;
        dcp_ns = tl.dcp;
        for (int k = 0; k < ns; ++k) {
            const double* rec = a.sp + (int64_t)k * PJG_SP_DOUBLES;
            const Thermo t = k == last ? tl : thermo<true>(rec, Tc, logT, Tinv, conp);
            gibbs(k, t.b);
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
            gibbs(k, thermo<false>(a.sp + (int64_t)k * PJG_SP_DOUBLES, Tc, logT, Tinv, conp).b);
    }
    if (split) {
        for (int k = 0; k < ns; ++k) {
            const double b = ep[k];
            ep[k] = fexp(b, etab);
            em[k] = fexp(-b, etab);
        }
    }
    sv.split = split;

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

    // ------------------------------------- reactions A + B <=> C + D (packed first)
    // the next reaction's record and per-state values are loaded while this
    // one computes
    E22Head hn;
    E22Vals vn;
    if (a.nr_e22 > 0) {
        load_e22(a.rxn, hn);
        e22_fetch<DER>(hn, split, conc, ep, em, db, vn);
    }
    for (int i = 0; i < a.nr_e22; ++i) {
        const E22Head h = hn;
        const E22Vals vv = vn;
        if (i + 1 < a.nr_e22) {
            load_e22(a.rxn + i + 1, hn);
            e22_fetch<DER>(hn, split, conc, ep, em, db, vn);
        }
        E22Terms o;
        e22_terms_v<DER>(h, vv, last, sv, o);
        accum(wdot, h.s[0], negi(o.net));
        accum(wdot, h.s[1], negi(o.net));
        accum(wdot, h.s[2], o.net);
        accum(wdot, h.s[3], o.net);
        if (!DER) continue;
        const bool hasns = (h.flags & RX_HASNS) && !a.jac_approx;
        if (VJP) {
            double w = 0.0;
#pragma unroll
            for (int ka = 0; ka < 4; ++ka)
                if (h.s[ka] != last) w = ka < 2 ? w - hw[h.s[ka]] : w + hw[h.s[ka]];
            if (nonzero(w)) {
#pragma unroll
                for (int jb = 0; jb < 4; ++jb)
                    if (h.s[jb] != last) accum(nsrow, h.s[jb], w * o.g[jb]);
                if (hasns) vNS = fma(w, o.gns, vNS);
                vout0 = fma(w, o.d0, vout0);
                vout1 = fma(w, o.d1, vout1);
            }
            continue;
        }
        const int* slots = a.rxn_slots + __ldg(a.rxn_slot_off + i);
        double* accs = a.acc + s;
#pragma unroll
        for (int ka = 0; ka < 4; ++ka) {
            const int k = h.s[ka];
            if (k == last) continue;
            // row k gets -v (reactants) or +v (products); reductions as below
#pragma unroll
            for (int jb = 0; jb < 6; ++jb) {
                const int sl = jb < 4 ? __ldg(slots + ka * 4 + jb) : __ldg(slots + 16 + 2 * ka + (jb - 4));
                const double v = jb < 4 ? o.g[jb] : (jb == 4 ? o.d0 : o.d1);
                if (sl >= 0) atomicAdd(accs + (int64_t)sl * a.acc_ld, ka < 2 ? negi(v) : v);
            }
            if (hasns) accum(nsrow, k, ka < 2 ? negi(o.gns) : o.gns);
        }
    }

    // ------------------------- other mass-action reactions in fixed patterns
    auto ma_range = [&](auto tag, int i0, int i1) {
        using PT = decltype(tag);
        constexpr int N = PT::n;
        for (int i = i0; i < i1; ++i) {
            RxnHead h;
            load_head(a.rxn + i, h);
            MaTerms o;
            ma_terms<PT, DER>(h, last, sv, conc, bk, ep, em, db, o);
            int sp[N];
#pragma unroll
            for (int e = 0; e < N; ++e) {
                sp[e] = ent_spec(h.ent[e]);
                if (PT::nur(e) != PT::nuf(e)) accum(wdot, sp[e], nux(PT::nur(e) - PT::nuf(e), o.net));
            }
            if (!DER) continue;
            const bool hasns = (h.flags & RX_HASNS) && !a.jac_approx;
            if (VJP) {
                double w = 0.0;
#pragma unroll
                for (int ka = 0; ka < N; ++ka)
                    if (sp[ka] != last) w = addnu(w, PT::nur(ka) - PT::nuf(ka), hw[sp[ka]]);
                if (nonzero(w)) {
#pragma unroll
                    for (int jb = 0; jb < N; ++jb)
                        if (sp[jb] != last) accum(nsrow, sp[jb], w * o.g[jb]);
                    if (hasns) vNS = fma(w, o.gns, vNS);
                    vout0 = fma(w, o.d0, vout0);
                    vout1 = fma(w, o.d1, vout1);
                }
                continue;
            }
            const int* slots = a.rxn_slots + __ldg(a.rxn_slot_off + i);
            double* accs = a.acc + s;
#pragma unroll
            for (int ka = 0; ka < N; ++ka) {
                const int nuk = PT::nur(ka) - PT::nuf(ka);
                if (nuk == 0 || sp[ka] == last) continue;
#pragma unroll
                for (int jb = 0; jb < N + 2; ++jb) {
                    const int sl = jb < N ? __ldg(slots + ka * N + jb)
                                          : __ldg(slots + N * N + 2 * ka + (jb - N));
                    const double v = jb < N ? o.g[jb] : (jb == N ? o.d0 : o.d1);
                    if (sl >= 0) atomicAdd(accs + (int64_t)sl * a.acc_ld, nux(nuk, v));
                }
                if (hasns) accum(nsrow, sp[ka], nux(nuk, o.gns));
            }
        }
    };
    ma_range(MaP0{}, a.ma_off[0], a.ma_off[1]);
    ma_range(MaP1{}, a.ma_off[1], a.ma_off[2]);
    ma_range(MaP2{}, a.ma_off[2], a.ma_off[3]);
    ma_range(MaP3{}, a.ma_off[3], a.ma_off[4]);
    ma_range(MaP4{}, a.ma_off[4], a.ma_off[5]);
    ma_range(MaP5{}, a.ma_off[5], a.ma_off[6]);
    ma_range(MaP6{}, a.ma_off[6], a.ma_off[7]);
    ma_range(MaP7{}, a.ma_off[7], a.ma_off[8]);
    ma_range(MaP8{}, a.ma_off[8], a.ma_off[9]);
    ma_range(MaP9{}, a.ma_off[9], a.ma_off[10]);

    // ------------------------------------------------------- other reactions
    // (the general code; third-body and fall-off reactions of the patterns
    // TpP0..TpP2 compiled per pattern, the rest reading their coefficients)
    auto general = [&](auto st_tag, int i0, int i1) {
        using ST = decltype(st_tag);
        MCache mc;
        for (int i = i0; i < i1; ++i) {
            RxnHead h;
            load_head(a.rxn + i, h);
            RxnTerms o;
            rxn_terms<DER, ST>(h, a.aux, a.thd_spec, a.thd_coef, last, sv, conc, bk, ep, em, db, mc, o);
            const int flags = h.flags, nsp = ST::nsp(h), thd_off = h.thd_off, thd_cnt = h.thd_cnt;
            const unsigned* ent = h.ent;
            const double* p = h.p;
#pragma unroll
            for (int e = 0; e < PJG_MAXSP; ++e) {
                if (e >= nsp) break;
                const int nu = ST::nur(h, e) - ST::nuf(h, e);
                if (nu != 0) accum(wdot, ent_spec(ent[e]), nux(nu, o.net));
            }
            if (!DER) continue;

            // ------------------------------------------------- Jacobian terms
            const int* slots = JAC ? a.rxn_slots + __ldg(a.rxn_slot_off + i) : nullptr;
            const int thd = RX_THD(flags);
            const bool hasns = flags & RX_HASNS;
            const double ci_ = o.ci_, X = o.X, d0 = o.d0, d1 = o.d1, gns = o.gns;
            const double* g = o.g;
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
                    w = addnu(w, ST::nur(h, ka) - ST::nuf(h, ka), hw[k]);
                }
                if (nonzero(w)) {
                    const double wc = w * ci_;
#pragma unroll
                    for (int jb = 0; jb < PJG_MAXSP; ++jb) {
                        if (jb >= nsp) break;
                        if (ent_spec(ent[jb]) != last) accum(nsrow, ent_spec(ent[jb]), wc * g[jb]);
                    }
                    if (hasns && !a.jac_approx) vNS = fma(wc, gns, vNS);
                    if (thd) {
                        const double wx = w * X;
                        for (int l = 0; l < thd_cnt; ++l) {
                            const int j = __ldg(a.thd_spec + thd_off + l);
                            if (j != last) accum(nsrow, j, __ldg(a.thd_coef + thd_off + l) * wx);
                        }
                        if (nslist && !a.jac_approx) vNS = fma(cns, wx, vNS);
                    }
                    vout0 = fma(w, d0, vout0);
                    vout1 = fma(w, d1, vout1);
                }
                continue;
            }
            // d R / d c_j times the pressure modification, once per reaction (ci is
            // exactly 1 without a third body)
            double gci[PJG_MAXSP];
#pragma unroll
            for (int e = 0; e < PJG_MAXSP; ++e) gci[e] = e < nsp ? (thd ? g[e] * ci_ : g[e]) : 0.0;
            // scatter into the species rows of this reaction
#pragma unroll
            for (int ka = 0; ka < PJG_MAXSP; ++ka) {
                if (ka >= nsp) break;
                const int k = ent_spec(ent[ka]);
                if (k == last) continue;
                const int nuk = ST::nur(h, ka) - ST::nuf(h, ka);
                if (nuk == 0) continue;
                // Fire-and-forget reductions (red.global.add.f64): the thread does not
                // wait for the accumulator's old value.  Only this thread updates its
                // state's entries, and one thread's operations on one address apply
                // in program order, so every entry sums its reactions in a fixed order.
                double* accs = a.acc + s;
#pragma unroll
                for (int jb = 0; jb < PJG_MAXSP + 2; ++jb) {
                    if (jb >= nsp + 2) break;
                    const int sl = jb < nsp ? __ldg(slots + ka * nsp + jb)
                                            : __ldg(slots + nsp * nsp + 2 * ka + (jb - nsp));
                    const double v = jb < nsp ? gci[jb] : (jb == nsp ? d0 : d1);
                    if (sl >= 0) atomicAdd(accs + (int64_t)sl * a.acc_ld, nux(nuk, v));
                }
                double nsacc = 0.0;
                if (hasns) nsacc = gns * ci_;
                if (thd && nslist) nsacc = fma(cns, X, nsacc);
                if ((hasns || (thd && nslist)) && !a.jac_approx) accum(nsrow, k, nux(nuk, nsacc));
            }
            // third-body list columns: coefficient x X formed once per list
            // entry, then +-it (or twice it) into every row of the reaction
            // (each entry still takes this reaction's terms after its
            // species-column terms, the order of the rows' own loops)
            if (thd) {
                double* accs = a.acc + s;
                for (int l = 0; l < thd_cnt; ++l) {
                    const double cw = __ldg(a.thd_coef + thd_off + l) * X;
#pragma unroll
                    for (int ka = 0; ka < PJG_MAXSP; ++ka) {
                        if (ka >= nsp) break;
                        if (ent_spec(ent[ka]) == last) continue;
                        const int nuk = ST::nur(h, ka) - ST::nuf(h, ka);
                        if (nuk == 0) continue;
                        const int sl = __ldg(slots + nsp * nsp + 2 * nsp + l * nsp + ka);
                        if (sl >= 0) atomicAdd(accs + (int64_t)sl * a.acc_ld, nux(nuk, cw));
                    }
                }
            }
        }
    };
    general(PatStoich<TpP0>{}, a.tp_off[0], a.tp_off[1]);
    general(PatStoich<TpP1>{}, a.tp_off[1], a.tp_off[2]);
    general(PatStoich<TpP2>{}, a.tp_off[2], a.tp_off[3]);
    general(RunStoich{}, a.tp_off[kTpPatterns], a.nr);

    __threadfence();

    // ------------------------------------------- temperature and E rates
    double upper = 0.0, lower = 0.0;
    if (DER) {
        for (int k = 0; k < last; ++k) {
            lower = fma(conc[k], cpa[k], lower);
            upper = fma(ha[k], rd(wdot, k), upper);
        }
        lower = fma(conc[last], cp_ns, lower);
        upper = fma(h_ns, rd(wdot, last), upper);
    } else {
        for (int k = 0; k < ns; ++k) {
            const Thermo t = thermo<false>(a.sp + (int64_t)k * PJG_SP_DOUBLES, Tc, logT, Tinv, conp);
            lower = fma(conc[k], t.cp, lower);
            upper = fma(t.h, rd(wdot, k), upper);
        }
    }
    const double Tdot = 0.0 + -1.0 * upper / lower;
    double dE = 0.0;
    for (int k = 0; k < last; ++k)
        dE = fma(ldg(a.sp + (int64_t)k * PJG_SP_DOUBLES + SP_OMW), rd(wdot, k), dE);
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
        for (int k = 0; k < last; ++k) o[(int64_t)(2 + k) * a.dphi_sj] = Vval * rd(wdot, k);
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
            const double wk = rd(wdot, k), ck = conc[k], cpk = cpa[k];
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
            o[(int64_t)(2 + j) * a.phi_sj] = rd(nsrow, j) - vNS + gam * (cpa[j] - cp_ns);
        return;
    }
    if (!JAC) return;

    // ------------------------------------------- assemble rows T and E
    double* acc = a.acc + s;
    const int64_t ld = a.acc_ld;
    // the reductions are performed in L2: read the accumulator there
    __threadfence();
    auto accr = [&](int64_t sl) { return __ldcg(acc + sl * ld); };
    const double cp_tot = lower;
    const double fixed = conp ? P : V, extra = conp ? V : P;
    const double inv_vcp = 1.0 / (V * cp_tot);
    const double TRf = T * RU / fixed, eTj = extra * Tjinv;
    if (a.dense_rs || a.dchunk_slots) {
        rows_te(a.dense_rs == 0, acc, ld, a.dense_rs, a.dense_cs, a.dchunk_off, a.dchunk_list,
                a.dchunk_slots, a.cj_slots, a.sp, nsrow, hw, cpa, last, cp_ns, Tdot, inv_vcp, TRf,
                eTj);
    } else {
        // sparse output whose pattern fills under half of the chunk lists' slots
        // (dchunk_slots null; large sparse mechanisms): the bath-gas terms (per-row
        // sums subtracted from every species column of the pattern), then the
        // column sums of rows T and E, two passes over the pattern
        for (int k = 0; k < last; ++k) {
            const double v = rd(nsrow, k);
            if (!nonzero(v)) continue;
            const int r0 = __ldg(a.row_off + k), r1 = __ldg(a.row_off + k + 1);
            for (int q = r0; q < r1; ++q) {
                const int2 e = __ldg(a.row_list + q);
                acc[(int64_t)e.y * ld] = accr(e.y) - v;
            }
        }
        for (int j = 0; j < last; ++j) {
            double sum = 0.0, sumE = 0.0;
            const int c0 = __ldg(a.col_off + j), c1 = __ldg(a.col_off + j + 1);
            for (int q = c0; q < c1; ++q) {
                const int2 e = __ldg(a.col_list + q);
                const double Jkj = accr(e.y);
                sum = fma(hw[e.x], Jkj, sum);
                sumE = fma(ldg(a.sp + (int64_t)e.x * PJG_SP_DOUBLES + SP_OMW), Jkj, sumE);
            }
            const double J0 = -1.0 * (sum + Tdot * (cpa[j] + -1.0 * cp_ns)) * inv_vcp;
            acc[(int64_t)__ldg(a.cj_slots + 2 * j) * ld] = J0;
            acc[(int64_t)__ldg(a.cj_slots + 2 * j + 1) * ld] = TRf * sumE + eTj * J0;
        }
    }

    // T column of rows T, E and E column of rows T, E
    double dTsum = (cp_ns * Tjinv - dcp_ns) * conc[last];
    double rate_sum = 0.0, sumT = 0.0, sumE1 = 0.0, spec1 = 0.0, dTsum1 = 0.0;
    const double Vjinv = 1.0 / V;
    for (int k = 0; k < last; ++k) {
        const double* rec = a.sp + (int64_t)k * PJG_SP_DOUBLES;
        const double mw = ldg(rec + SP_MW), omw = ldg(rec + SP_OMW);
        const int sl0 = __ldg(a.sp_slots + 2 * k), sl1 = __ldg(a.sp_slots + 2 * k + 1);
        const double Jk0 = sl0 >= 0 ? accr(sl0) : 0.0;
        const double Jk1 = sl1 >= 0 ? accr(sl1) : 0.0;
        const double wk = rd(wdot, k), ck = conc[k], cpk = cpa[k], hwk = hw[k];
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

// Species thermo of the chem_utils kernel type (rate_subs.py write_chem_utils
// :3391-3444, polyfit_kernel_gen :3281-3388): at the guarded temperature,
// cp (cv), h (u) and the Gibbs function b of every species.  Entry (s, k) of
// each output at out[s * out_ss + k * out_sk].
__global__ void __launch_bounds__(PJG_BLOCK) chem_utils_kernel(const double* __restrict__ sp, int ns,
                                                               int64_t n, int conp,
                                                               const double* __restrict__ phi,
                                                               int64_t phi_ss, double* cp, double* h,
                                                               double* b, int64_t out_ss,
                                                               int64_t out_sk)
{
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const double Tc = fmin(10000.0, fmax(100.0, phi[s * phi_ss]));
    const double logT = log(Tc), Tinv = 1.0 / Tc;
    for (int k = 0; k < ns; ++k) {
        const Thermo t = thermo<false>(sp + (int64_t)k * PJG_SP_DOUBLES, Tc, logT, Tinv, conp);
        const int64_t o = s * out_ss + (int64_t)k * out_sk;
        cp[o] = t.cp;
        h[o] = t.h;
        b[o] = t.b;
    }
}

}  // namespace

int pjg_launch_chem_utils(const double* sp, int ns, int64_t n, int conp, const double* phi,
                          int64_t phi_ss, double* cp, double* h, double* b, int64_t out_ss,
                          int64_t out_sk, void* stream)
{
    if (n <= 0) return 0;
    chem_utils_kernel<<<(unsigned)((n + PJG_BLOCK - 1) / PJG_BLOCK), PJG_BLOCK, 0, (cudaStream_t)stream>>>(
        sp, ns, n, conp, phi, phi_ss, cp, h, b, out_ss, out_sk);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

namespace {

template <int KIND>
void launch(const EvalArgs& a, unsigned grid, cudaStream_t st)
{
    eval_kernel<KIND><<<grid, PJG_BLOCK, 0, st>>>(a);
}

}  // namespace

int pjg_eval_blocks_per_sm(int kind)
{
    int b = 0;
    cudaError_t e;
    if (kind == 1)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, eval_kernel<1>, PJG_BLOCK, 0);
    else if (kind == 2)
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, eval_kernel<2>, PJG_BLOCK, 0);
    else
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, eval_kernel<0>, PJG_BLOCK, 0);
    return e == cudaSuccess && b > 0 ? b : 1;
}

namespace {
thread_local cudaError_t g_launch_err = cudaSuccess;  // of this thread's last evaluation launch
}

const char* pjg_launch_error_string() { return cudaGetErrorString(g_launch_err); }

int pjg_launch_eval(const EvalArgs& a, int kind, void* stream)
{
    if (a.n <= 0) return 0;
    cudaStream_t st = (cudaStream_t)stream;
    const unsigned grid = (unsigned)((a.n + PJG_BLOCK - 1) / PJG_BLOCK);
    if (kind == 1) launch<1>(a, grid, st);
    else if (kind == 2) launch<2>(a, grid, st);
    else launch<0>(a, grid, st);
    g_launch_err = cudaGetLastError();
    return g_launch_err == cudaSuccess ? 0 : -2;
}
