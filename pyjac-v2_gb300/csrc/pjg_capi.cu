// C ABI of pyjac-v2_gb300 (declared in include/pyjac_gb300.h).
//
// Host responsibilities: validate and upload the mechanism tables, derive the
// Jacobian slot tables for each output layout (dense/sparse x C/F), size the
// per-state working arrays, chunk large problems, and launch the kernels of
// pjg_eval.cu.  Mirrors the reference's generated Kernel class
// (pyjac/kernel_utils/common/kernel.hpp.in:86-335, kernel.cpp.in:539-633):
// problems are evaluated in chunks (the reference's max_per_run) with a
// per-kernel-object device working buffer (the reference's rwk).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <vector>

#include "../../include/pyjac_gb300.h"
#include "../../include/pyjac_gb300_internal.h"
#include "pjg_eval.cuh"
#include "pjg_rxn.cuh"
#include "pjg_mlp.cuh"

namespace {

constexpr int PJG_KIND_VJP = 2;  // internal kernel kind of pjg_vjp
thread_local char g_err[512] = "";
// kernel launches issued by this library, and optional per-launch timing of
// the evaluation kernels (pjg_profile_begin / pjg_profile_end)
std::atomic<int64_t> g_launches{0};
std::atomic<bool> g_prof_on{false};
std::mutex g_prof_mu;
std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_prof_events;

int fail(int code, const char* fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

#define CUDA_TRY(x)                                                                   \
    do {                                                                              \
        cudaError_t e_ = (x);                                                         \
        if (e_ != cudaSuccess)                                                        \
            return fail(PJG_ERR_CUDA, "%s failed: %s", #x, cudaGetErrorString(e_));   \
    } while (0)

template <class T>
int upload(const std::vector<T>& h, T** d)
{
    *d = nullptr;
    size_t bytes = std::max<size_t>(h.size(), 1) * sizeof(T);
    CUDA_TRY(cudaMalloc((void**)d, bytes));
    if (!h.empty()) CUDA_TRY(cudaMemcpy(*d, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice));
    return 0;
}

struct SlotTables {
    int nslot = 0;
    int *rxn_slot_off = nullptr, *rxn_slots = nullptr;
    int *row_off = nullptr, *col_off = nullptr;
    int2 *row_list = nullptr, *col_list = nullptr;
    int *sp_slots = nullptr, *cj_slots = nullptr;
    int *dchunk_off = nullptr, *dchunk_list = nullptr;
    int4* dchunk_slots = nullptr;  // sparse output only
    int s00 = 0, s01 = 0, s10 = 0, s11 = 0;
    size_t bytes = 0;
};

}  // namespace

extern "C" int pjg_internal_lu_plan_create(int32_t nn, const int32_t* row_ptr, const int32_t* col_ind,
                                           void** out);
extern "C" void pjg_internal_lu_plan_destroy(void* p);
extern "C" void pjg_internal_lu_plan_info(const void* p, int32_t* perm, int32_t* nnz_lu, int64_t* fma);
extern "C" int pjg_internal_lu_factor_sparse(const void* p, int64_t n, char order, double s,
                                             const double* h, double h0, const double* jac, double* lu,
                                             int32_t* info, cudaStream_t st);
extern "C" int pjg_internal_lu_solve_sparse(const void* p, int64_t n, char order, const double* lu,
                                            double* b, cudaStream_t st);

struct pjg_mech {
    int ns = 0, nr = 0, nn = 0, need_logP = 0, nnz = 0, jac_approx = 0;
    int nr_e22 = 0;  // leading reactions of the class A + B <=> C + D
    double kc_split_max = 138.0;  // EvalArgs::kc_split_max
    int ma_off[11] = {};                          // then the mass-action patterns (EvalArgs)
    int tp_off[4] = {0, 0, 0, 0};                 // then the third-body patterns (EvalArgs)
    int device = 0;
    PjgRxn* rxn = nullptr;
    double* sp = nullptr;
    int* thd_spec = nullptr;
    double* thd_coef = nullptr;
    double* aux = nullptr;
    // host copies used to derive slot tables
    std::vector<PjgRxn> h_rxn;
    std::vector<int> h_thd_spec;
    std::vector<double> h_thd_coef;
    std::vector<int> crs_ptr, crs_ind, ccs_ptr, ccs_ind;
    std::map<int, SlotTables> slots;  // key: (order == 'F') * 2 + sparse
    std::mutex lock;
    // working buffer shared by device-pointer calls on this mechanism
    double* work = nullptr;
    size_t work_bytes = 0;
    // static-pivot sparse LU plan of the Newton matrix (built on first use)
    void* lu_plan = nullptr;
};

// Kernel object (host-pointer calls).  A call streams the problem through
// kRing device buffers: while chunk c is evaluated, chunk c+1 is copied in
// and chunk c-1 copied out (the copy engines run beside the kernels), on
// three streams ordered by events.  A chunk is PJG_CHUNK_WAVES full waves of
// resident Jacobian blocks: a launch of a fraction of a wave takes as long as
// a whole one.
constexpr int kRing = 3;
#ifndef PJG_CHUNK_WAVES
#define PJG_CHUNK_WAVES 2
#endif
constexpr size_t kKernelBudget = size_t(32) << 30;  // device bytes of one kernel object

struct pjg_kernel {
    pjg_mech* mech = nullptr;
    int kind = 0, conp = 1, jac_format = 0;
    char order = 'C';
    size_t problem_size = 0, work_size = 0;
    int64_t chunk = 0;                 // states per device buffer
    double* d_param[kRing] = {};
    double* d_phi[kRing] = {};
    double* d_out[kRing] = {};
    double* work = nullptr;            // per-state working arrays of one chunk
    size_t work_bytes = 0;
    size_t out_per_state = 0;
    cudaStream_t s_in = nullptr, s_comp = nullptr, s_out = nullptr;
    cudaEvent_t ev_in[kRing] = {}, ev_k[kRing] = {}, ev_out[kRing] = {};
};

namespace {

int slot_of(const pjg_mech* m, bool F, bool sparse, int r, int c)
{
    const int NN = m->nn;
    if (!sparse) return F ? r + NN * c : r * NN + c;
    if (!F) {
        for (int q = m->crs_ptr[r]; q < m->crs_ptr[r + 1]; ++q)
            if (m->crs_ind[q] == c) return q;
        return -1;
    }
    for (int q = m->ccs_ptr[c]; q < m->ccs_ptr[c + 1]; ++q)
        if (m->ccs_ind[q] == r) return q;
    return -1;
}

int build_slots(pjg_mech* m, bool F, bool sparse, SlotTables** out)
{
    const int key = (F ? 2 : 0) + (sparse ? 1 : 0);
    std::lock_guard<std::mutex> g(m->lock);
    auto it = m->slots.find(key);
    if (it != m->slots.end()) {
        *out = &it->second;
        return 0;
    }
    const int ns = m->ns, last = ns - 1, NN = m->nn;
    SlotTables t;
    t.nslot = sparse ? m->nnz : NN * NN;
    std::vector<int> off(m->nr + 1, 0), list;
    for (int i = 0; i < m->nr; ++i) {
        const PjgRxn& R = m->h_rxn[i];
        const int nsp = R.nspec;
        off[i] = (int)list.size();
        for (int a = 0; a < nsp; ++a)
            for (int b = 0; b < nsp; ++b) {
                const int k = ent_spec(R.ent[a]), j = ent_spec(R.ent[b]);
                list.push_back(k == last || j == last ? -1 : slot_of(m, F, sparse, 2 + k, 2 + j));
            }
        for (int a = 0; a < nsp; ++a) {
            const int k = ent_spec(R.ent[a]);
            list.push_back(k == last ? -1 : slot_of(m, F, sparse, 2 + k, 0));
            list.push_back(k == last ? -1 : slot_of(m, F, sparse, 2 + k, 1));
        }
        for (int l = 0; l < R.thd_cnt; ++l) {
            const int j = m->h_thd_spec[R.thd_off + l];
            for (int a = 0; a < nsp; ++a) {
                const int k = ent_spec(R.ent[a]);
                list.push_back(k == last || j == last ? -1 : slot_of(m, F, sparse, 2 + k, 2 + j));
            }
        }
    }
    off[m->nr] = (int)list.size();
    std::vector<int> row_off(ns, 0), col_off(ns, 0), sp_slots(2 * std::max(last, 1), -1),
        cj_slots(2 * std::max(last, 1), -1);
    std::vector<int2> row_list, col_list;
    for (int k = 0; k < last; ++k) {
        row_off[k] = (int)row_list.size();
        for (int j = 0; j < last; ++j) {
            const int sl = slot_of(m, F, sparse, 2 + k, 2 + j);
            if (sl >= 0) row_list.push_back(make_int2(j, sl));
        }
        sp_slots[2 * k] = slot_of(m, F, sparse, 2 + k, 0);
        sp_slots[2 * k + 1] = slot_of(m, F, sparse, 2 + k, 1);
    }
    for (int j = 0; j < last; ++j) {
        col_off[j] = (int)col_list.size();
        for (int k = 0; k < last; ++k) {
            const int sl = slot_of(m, F, sparse, 2 + k, 2 + j);
            if (sl >= 0) col_list.push_back(make_int2(k, sl));
        }
        cj_slots[2 * j] = slot_of(m, F, sparse, 0, 2 + j);
        cj_slots[2 * j + 1] = slot_of(m, F, sparse, 1, 2 + j);
        if (cj_slots[2 * j] < 0 || cj_slots[2 * j + 1] < 0)
            return fail(PJG_ERR_TABLES, "Jacobian pattern lacks entries of rows T/E");
    }
    row_off[last] = (int)row_list.size();
    col_off[last] = (int)col_list.size();
    // the structurally nonzero entries of the species block (the pattern's;
    // for a dense output also every entry a reaction adds to) in chunks of
    // PJG_DENSE_COLS columns, the assembly's row lists; a sparse output's
    // slots of each listed row
    static_assert(PJG_DENSE_COLS == 4, "one int4 of slots per listed row");
    std::vector<int> doff, dlist;
    std::vector<int4> dslots;
    if (last > 0) {
        std::vector<char> nz((size_t)last * last, 0);
        for (int k = 0; k < last; ++k)
            for (int q = m->crs_ptr[2 + k]; q < m->crs_ptr[3 + k]; ++q) {
                const int c = m->crs_ind[q] - 2;
                if (c >= 0 && c < last) nz[(size_t)k * last + c] = 1;
            }
        if (!sparse)
            for (int sl : list) {
                if (sl < 0) continue;
                const int r = F ? sl % NN : sl / NN, c = F ? sl / NN : sl % NN;
                if (r >= 2 && c >= 2) nz[(size_t)(r - 2) * last + (c - 2)] = 1;
            }
        for (int j0 = 0; j0 < last; j0 += PJG_DENSE_COLS) {
            doff.push_back((int)dlist.size());
            for (int k = 0; k < last; ++k) {
                int mask = 0, sl[PJG_DENSE_COLS] = {-1, -1, -1, -1};
                for (int q = 0; q < PJG_DENSE_COLS && j0 + q < last; ++q)
                    if (nz[(size_t)k * last + j0 + q]) {
                        mask |= 1 << q;
                        sl[q] = slot_of(m, F, sparse, 2 + k, 2 + j0 + q);
                        if (sparse && sl[q] < 0)
                            return fail(PJG_ERR_TABLES, "Jacobian pattern inconsistent");
                    }
                if (mask) {
                    dlist.push_back(k << 4 | mask);
                    if (sparse) dslots.push_back(make_int4(sl[0], sl[1], sl[2], sl[3]));
                }
            }
        }
        doff.push_back((int)dlist.size());
        // a sparse output takes the chunk lists where the pattern fills at
        // least half of the listed rows' slots (GRI: 1,774 of 2,100); else
        // its two passes over the pattern (the 500-species mechanism: about a
        // third, where the lists ran 19 % slower)
        if (sparse && (size_t)m->nnz * 2 < dlist.size() * PJG_DENSE_COLS) dslots.clear();
    }
    t.s00 = slot_of(m, F, sparse, 0, 0);
    t.s01 = slot_of(m, F, sparse, 0, 1);
    t.s10 = slot_of(m, F, sparse, 1, 0);
    t.s11 = slot_of(m, F, sparse, 1, 1);
    if (t.s00 < 0 || t.s01 < 0 || t.s10 < 0 || t.s11 < 0)
        return fail(PJG_ERR_TABLES, "Jacobian pattern lacks the T/E block");
    int rc;
    if ((rc = upload(off, &t.rxn_slot_off)) || (rc = upload(list, &t.rxn_slots)) ||
        (rc = upload(row_off, &t.row_off)) || (rc = upload(row_list, &t.row_list)) ||
        (rc = upload(col_off, &t.col_off)) || (rc = upload(col_list, &t.col_list)) ||
        (rc = upload(sp_slots, &t.sp_slots)) || (rc = upload(cj_slots, &t.cj_slots)) ||
        (rc = upload(doff, &t.dchunk_off)) || (rc = upload(dlist, &t.dchunk_list)) ||
        (!dslots.empty() && (rc = upload(dslots, &t.dchunk_slots))))
        return rc;
    t.bytes = (off.size() + list.size() + row_off.size() + col_off.size() + sp_slots.size() +
               cj_slots.size() + doff.size() + dlist.size()) * sizeof(int) +
              (row_list.size() + col_list.size()) * sizeof(int2) + dslots.size() * sizeof(int4);
    auto res = m->slots.emplace(key, t);
    *out = &res.first->second;
    return 0;
}

// per-state bytes of working arrays for one evaluation
size_t state_bytes(const pjg_mech* m, int kind, bool c_order_jac, int nslot)
{
    size_t arrs = kind == PJG_SPECIES_RATES ? ARR_N_RATES : ARR_N_JAC;
    size_t b = arrs * m->ns * sizeof(double);
    if (kind == PJG_JACOBIAN && c_order_jac) b += (size_t)nslot * sizeof(double);
    return b;
}

constexpr size_t kWorkBudget = size_t(8) << 30;  // bytes of working buffer per call

// States one launch can take with per_state bytes of working arrays: a whole
// number of waves of resident blocks within the budget (a launch of a
// fraction of a wave takes as long as a full wave).  Where one wave needs
// more than the budget (large mechanisms in order 'C'), a full wave if half
// the free device memory holds it, else as much as fits.  At most n.
int64_t chunk_states(size_t per_state, int64_t n, int64_t wave)
{
    if (per_state == 0) return n;
    int64_t c = (int64_t)(kWorkBudget / per_state);
    if (c >= wave) {
        c = c / wave * wave;
    } else {
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = 0;
        const int64_t fit = (int64_t)(free_b / 2 / per_state);
        c = std::max<int64_t>(c, std::min<int64_t>(fit, wave));
        c = std::max<int64_t>(PJG_BLOCK, c / PJG_BLOCK * PJG_BLOCK);
    }
    return std::min<int64_t>(c, n);
}

// States of one full wave of the evaluation kernel of `kind` on the mechanism's device.
int64_t wave_states(const pjg_mech* m, int kind)
{
    int sms = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, m->device);
    return (int64_t)sms * pjg_eval_blocks_per_sm(kind) * PJG_BLOCK;
}

int ensure_work(pjg_mech* m, size_t bytes)
{
    if (bytes <= m->work_bytes) return 0;
    if (m->work) cudaFree(m->work);
    m->work = nullptr;
    m->work_bytes = 0;
    CUDA_TRY(cudaMalloc((void**)&m->work, bytes));
    m->work_bytes = bytes;
    return 0;
}

// The mechanism's tables live on the device that was current at
// pjg_mech_create; a launch on another device would read them through
// foreign addresses, so such calls are rejected.
int check_device(const pjg_mech* m)
{
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess) return fail(PJG_ERR_CUDA, "cudaGetDevice failed");
    if (cur != m->device)
        return fail(PJG_ERR_ARG, "mechanism was created on device %d, current device is %d",
                    m->device, cur);
    return 0;
}

void fill_common(const pjg_mech* m, EvalArgs& a)
{
    memset(&a, 0, sizeof(a));
    a.rxn = m->rxn;
    a.sp = m->sp;
    a.thd_spec = m->thd_spec;
    a.thd_coef = m->thd_coef;
    a.aux = m->aux;
    a.ns = m->ns;
    a.nr = m->nr;
    a.nr_e22 = m->nr_e22;
    for (int q = 0; q <= pjg::kMaPatterns; ++q) a.ma_off[q] = m->ma_off[q];
    for (int q = 0; q <= pjg::kTpPatterns; ++q) a.tp_off[q] = m->tp_off[q];
    a.need_logP = m->need_logP;
    a.jac_approx = m->jac_approx;
    a.kc_split_max = m->kc_split_max;
}

// Per-state bytes of working arrays one evaluation needs.  The Jacobian
// accumulates in scratch for order 'C' (then transposed); an output of order
// 'F' is its own accumulator.
size_t eval_state_bytes(const pjg_mech* m, int kind, bool F, const SlotTables* t)
{
    return state_bytes(m, kind, kind == PJG_JACOBIAN && !F, t ? t->nslot : 0);
}

// Evaluate n states.  The per-state working arrays go to ext_work (ext_bytes)
// when given, else to the mechanism's shared buffer, grown on demand; larger
// problems run as several launches.
// For the Jacobian, dphi (optional, laid out like phi) also receives the
// species rates of the same pass.
int run_eval(pjg_mech* m, int kind, int64_t n, char order, int conp, int jac_format,
             const double* param, const double* phi, double* out, cudaStream_t st,
             const double* v = nullptr, double* ext_work = nullptr, size_t ext_bytes = 0,
             double* dphi = nullptr)
{
    if (!m) return fail(PJG_ERR_ARG, "null mechanism");
    if (n < 0) return fail(PJG_ERR_ARG, "negative problem size");
    if (order != 'C' && order != 'F') return fail(PJG_ERR_ARG, "order must be 'C' or 'F'");
    if (jac_format != PJG_JAC_FULL && jac_format != PJG_JAC_SPARSE)
        return fail(PJG_ERR_ARG, "jac_format must be 0 (full) or 1 (sparse)");
    if (n == 0) return 0;
    if (!param || !phi || !out) return fail(PJG_ERR_ARG, "null array");
    if (kind == PJG_KIND_VJP && !v) return fail(PJG_ERR_ARG, "null vector");
    if (int rc = check_device(m)) return rc;
    const bool F = order == 'F';
    const int NN = m->nn;
    SlotTables* t = nullptr;
    if (kind == PJG_JACOBIAN) {
        int rc = build_slots(m, F, jac_format == PJG_JAC_SPARSE, &t);
        if (rc) return rc;
    }
    const size_t per_state = eval_state_bytes(m, kind, F, t);
    int64_t ch;
    double* work = ext_work;
    if (ext_work) {
        ch = per_state ? (int64_t)(ext_bytes / per_state) / PJG_BLOCK * PJG_BLOCK : n;
        if (ch < PJG_BLOCK && ch < n) return fail(PJG_ERR_ARG, "working buffer too small");
        ch = std::min<int64_t>(std::max<int64_t>(ch, 1), n);
    } else {
        ch = chunk_states(per_state, n, wave_states(m, kind));
        if (per_state) {
            int rc = ensure_work(m, per_state * (size_t)ch);
            if (rc) return rc;
        }
        work = m->work;
    }
    for (int64_t off = 0; off < n; off += ch) {
        const int64_t cnt = std::min<int64_t>(ch, n - off);
        EvalArgs a;
        fill_common(m, a);
        a.n = cnt;
        a.conp = conp;
        a.param = param + off;
        if (F) {
            a.phi = phi + off;
            a.phi_ss = 1;
            a.phi_sj = n;
        } else {
            a.phi = phi + off * NN;
            a.phi_ss = NN;
            a.phi_sj = 1;
        }
        a.scratch = work;
        a.sc_ld = ch;
        if (kind == PJG_SPECIES_RATES) {
            a.dphi = F ? out + off : out + off * NN;
            a.dphi_ss = a.phi_ss;
            a.dphi_sj = a.phi_sj;
        } else if (kind == PJG_KIND_VJP) {
            a.v = F ? v + off : v + off * NN;
            a.vjp = F ? out + off : out + off * NN;
        } else {
            if (dphi) {
                a.dphi = F ? dphi + off : dphi + off * NN;
                a.dphi_ss = a.phi_ss;
                a.dphi_sj = a.phi_sj;
            }
            a.nslot = t->nslot;
            if (F) {
                a.acc = out + off;
                a.acc_ld = n;
            } else {
                a.acc = work + (size_t)ARR_N_JAC * m->ns * ch;
                a.acc_ld = ch;
            }
            a.rxn_slot_off = t->rxn_slot_off;
            a.rxn_slots = t->rxn_slots;
            a.row_off = t->row_off;
            a.row_list = t->row_list;
            a.col_off = t->col_off;
            a.col_list = t->col_list;
            a.sp_slots = t->sp_slots;
            a.cj_slots = t->cj_slots;
            a.dchunk_off = t->dchunk_off;
            a.dchunk_list = t->dchunk_list;
            a.dchunk_slots = t->dchunk_slots;
            a.s00 = t->s00;
            a.s01 = t->s01;
            a.s10 = t->s10;
            a.s11 = t->s11;
            if (jac_format != PJG_JAC_SPARSE) {
                a.dense_rs = F ? 1 : NN;
                a.dense_cs = F ? NN : 1;
            }
        }
        int rc = 0;
        if (kind == PJG_JACOBIAN) {
            rc = pjg_launch_zero(a.acc, a.acc_ld, cnt, a.nslot, st);
            if (rc) return fail(PJG_ERR_CUDA, "zero launch failed");
            g_launches.fetch_add(1);
        }
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        const bool prof = g_prof_on.load();
        if (prof) {
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            cudaEventRecord(e0, st);
        }
        rc = pjg_launch_eval(a, kind, st);
        if (rc) return fail(PJG_ERR_CUDA, "kernel launch failed: %s", pjg_launch_error_string());
        g_launches.fetch_add(1);
        if (prof) {
            cudaEventRecord(e1, st);
            std::lock_guard<std::mutex> g(g_prof_mu);
            g_prof_events.emplace_back(e0, e1);
        }
        if (kind == PJG_JACOBIAN && !F) {
            rc = pjg_launch_transpose(a.acc, a.acc_ld, cnt, t->nslot, out + off * (int64_t)t->nslot,
                                      st);
            if (rc) return fail(PJG_ERR_CUDA, "transpose launch failed");
            g_launches.fetch_add(1);
        }
    }
    return 0;
}

// A reaction of the class A + B <=> C + D: four distinct species with unit
// coefficients, reversible, an Arrhenius rate form, no third body, and
// (P_atm / R)^nu_sum = 1 (nu_sum = 0).  232 of GRI-Mech 3.0's 325 reactions.
bool is_e22(const PjgRxn& R)
{
    if (R.nspec != 4 || RX_FORM(R.flags) > FORM_ARR || !(R.flags & RX_REV) ||
        RX_THD(R.flags) != THD_NONE || R.nu_sum != 0 || R.p[P_PSUM] != 1.0)
        return false;
    int nre = 0, npr = 0;
    for (int e = 0; e < 4; ++e) {
        const int f = ent_nuf(R.ent[e]), r = ent_nur(R.ent[e]);
        if (f == 1 && r == 0) ++nre;
        else if (f == 0 && r == 1) ++npr;
        else return false;
    }
    return nre == 2 && npr == 2;
}

// whether a canonical coefficient list (pattern_key) and reversibility are
// those of the pattern PT (pjg_rxn.cuh)
template <class PT>
bool ma_matches(const std::vector<std::pair<int, int>>& key, bool rev)
{
    if (PT::rev != rev || (int)key.size() != PT::n) return false;
    for (int e = 0; e < PT::n; ++e)
        if (key[e].first != PT::nuf(e) || key[e].second != PT::nur(e)) return false;
    return true;
}

// The canonical order of a record's entries: reactant-only entries by
// coefficient, then entries on both sides by (reactant, product)
// coefficients, then product-only entries by coefficient; species order kept
// among equal coefficients.  Coefficients above 2 have no canonical order.
bool canonical_order(const PjgRxn& R, int* idx)
{
    int k = 0;
    for (int pass = 0; pass < 3; ++pass)
        for (int a = 1; a <= 2; ++a)
            for (int b = pass == 1 ? 1 : 0; b <= (pass == 1 ? 2 : 0); ++b)
                for (int e = 0; e < R.nspec; ++e) {
                    const int f = ent_nuf(R.ent[e]), r = ent_nur(R.ent[e]);
                    if ((pass == 0 && f == a && r == 0) || (pass == 1 && f == a && r == b) ||
                        (pass == 2 && f == 0 && r == a))
                        idx[k++] = e;
                }
    return k == R.nspec;
}

// the canonical (reactant, product) coefficient list of a record; empty if a
// coefficient is above 2
std::vector<std::pair<int, int>> pattern_key(const PjgRxn& R)
{
    std::vector<std::pair<int, int>> key;
    int idx[PJG_MAXSP];
    if (!canonical_order(R, idx)) return key;
    for (int k = 0; k < R.nspec; ++k)
        key.push_back({ent_nuf(R.ent[idx[k]]), ent_nur(R.ent[idx[k]])});
    return key;
}

// TpP0..TpP2: third-body or fall-off reactions of an Arrhenius form
int tp_pattern_of(const PjgRxn& R)
{
    if (RX_FORM(R.flags) > FORM_ARR || RX_THD(R.flags) == THD_NONE) return -1;
    const auto key = pattern_key(R);
    const bool rev = R.flags & RX_REV;
    if (key.empty()) return -1;
    if (ma_matches<pjg::TpP0>(key, rev)) return 0;
    if (ma_matches<pjg::TpP1>(key, rev)) return 1;
    if (ma_matches<pjg::TpP2>(key, rev)) return 2;
    return -1;
}

// the record with its entries in the canonical order (a pattern's record)
PjgRxn canonical_entries(const PjgRxn& R)
{
    PjgRxn c = R;
    int idx[PJG_MAXSP];
    if (canonical_order(R, idx))
        for (int k = 0; k < R.nspec; ++k) c.ent[k] = R.ent[idx[k]];
    return c;
}

// MaP0..MaP9: reactions without third body, of an Arrhenius form, whose
// canonical coefficient list matches a pattern; -1 otherwise (other shapes,
// coefficients above 2, third bodies, fall-off, PLOG and Chebyshev keep the
// general code)
int ma_pattern_of(const PjgRxn& R)
{
    if (RX_FORM(R.flags) > FORM_ARR || RX_THD(R.flags) != THD_NONE || R.nspec < 3 || R.nspec > 5)
        return -1;
    const auto key = pattern_key(R);
    if (key.empty()) return -1;  // a coefficient > 2
    const bool rev = R.flags & RX_REV;
    if (ma_matches<pjg::MaP0>(key, rev)) return 0;
    if (ma_matches<pjg::MaP1>(key, rev)) return 1;
    if (ma_matches<pjg::MaP2>(key, rev)) return 2;
    if (ma_matches<pjg::MaP3>(key, rev)) return 3;
    if (ma_matches<pjg::MaP4>(key, rev)) return 4;
    if (ma_matches<pjg::MaP5>(key, rev)) return 5;
    if (ma_matches<pjg::MaP6>(key, rev)) return 6;
    if (ma_matches<pjg::MaP7>(key, rev)) return 7;
    if (ma_matches<pjg::MaP8>(key, rev)) return 8;
    if (ma_matches<pjg::MaP9>(key, rev)) return 9;
    return -1;
}

// The packed reaction order of the device tables: the class above first,
// each with its entries reordered reactants first (species order kept within
// each side); then the mass-action patterns MaP0..MaP9 and the third-body
// patterns TpP0..TpP2 (pjg_rxn.cuh), each reaction with its entries in the
// pattern's order (canonical_entries); then the rest in mechanism order.
// The kernels evaluate each group by code compiled for it.  Nothing outside
// the kernels depends on the reaction order: the species rates and the
// Jacobian are sums over reactions, and the slot tables are built from these
// records.  orig[p] is the mechanism index of packed record p, cls[p] its
// group: 0 the elementary class, 1 + q pattern MaPq, 1 + kMaPatterns + t
// pattern TpPt, -1 the general code.
struct Packing {
    std::vector<PjgRxn> rx;
    std::vector<int> orig, cls;
    int nr_e22 = 0;
    int ma_off[pjg::kMaPatterns + 1] = {};
    int tp_off[pjg::kTpPatterns + 1] = {};
};

// Reactions with a third body whose [M] is the same function of the state
// (default efficiency, then the same (species, efficiency) list) share one
// key: the mechanism-order index of the first such reaction.  -1 without a
// third body.  canon receives that first reaction's list offset.
std::vector<int> third_body_keys(const std::vector<PjgRxn>& in, const int* thd_spec,
                                 const double* thd_coef, std::vector<int>& canon)
{
    std::map<std::vector<long long>, int> seen;
    std::vector<int> key(in.size(), -1);
    canon.assign(in.size(), 0);
    for (int i = 0; i < (int)in.size(); ++i) {
        const PjgRxn& R = in[i];
        canon[i] = R.thd_off;
        if (RX_THD(R.flags) == THD_NONE) continue;
        std::vector<long long> k;
        double flag = R.p[P_FLAG];
        long long fb;
        memcpy(&fb, &flag, sizeof fb);
        k.push_back(fb);
        for (int l = 0; l < R.thd_cnt; ++l) {
            long long cb;
            memcpy(&cb, thd_coef + R.thd_off + l, sizeof cb);
            k.push_back(thd_spec[R.thd_off + l]);
            k.push_back(cb);
        }
        auto it = seen.emplace(k, i).first;
        key[i] = it->second;
        canon[i] = in[it->second].thd_off;
    }
    return key;
}

void pack_reactions(const std::vector<PjgRxn>& in, const int* thd_spec, const double* thd_coef,
                    Packing& pk)
{
    const int nma = pjg::kMaPatterns, ntp = pjg::kTpPatterns;
    std::vector<std::vector<int>> groups(1 + nma + ntp + 1);  // indices into `in`
    for (int i = 0; i < (int)in.size(); ++i) {
        const PjgRxn& R = in[i];
        int g;
        if (is_e22(R)) {
            g = 0;
        } else {
            const int q = ma_pattern_of(R), t = q < 0 ? tp_pattern_of(R) : -1;
            g = q >= 0 ? 1 + q : t >= 0 ? 1 + nma + t : 1 + nma + ntp;
        }
        groups[g].push_back(i);
    }
    // third-body groups and the general group: the later reactions sharing
    // [M] with a reaction are moved up to follow it (every other reaction
    // keeps its place in mechanism order), so that the kernels reuse [M] and
    // ln [M]; identical lists share one stored copy
    std::vector<int> canon;
    const std::vector<int> key = third_body_keys(in, thd_spec, thd_coef, canon);
    for (int g = 1 + nma; g < (int)groups.size(); ++g) {
        std::vector<int> ordered;
        std::vector<char> placed(groups[g].size(), 0);
        for (size_t x = 0; x < groups[g].size(); ++x) {
            if (placed[x]) continue;
            const int i = groups[g][x];
            ordered.push_back(i);
            if (key[i] < 0) continue;
            for (size_t y = x + 1; y < groups[g].size(); ++y)
                if (!placed[y] && key[groups[g][y]] == key[i]) {
                    ordered.push_back(groups[g][y]);
                    placed[y] = 1;
                }
        }
        groups[g].swap(ordered);
    }
    pk.rx.clear();
    pk.orig.clear();
    pk.cls.clear();
    for (int g = 0; g < (int)groups.size(); ++g) {
        if (g >= 1 && g <= nma) pk.ma_off[g - 1] = (int)pk.rx.size();
        if (g > nma && g <= nma + ntp) pk.tp_off[g - 1 - nma] = (int)pk.rx.size();
        for (int i : groups[g]) {
            const PjgRxn& R = in[i];
            PjgRxn c = R;
            c.thd_off = canon[i];
            if (g == 0) {
                int q = 0;
                for (int side = 0; side < 2; ++side)
                    for (int e = 0; e < 4; ++e)
                        if ((ent_nuf(R.ent[e]) == 1) == (side == 0)) c.ent[q++] = R.ent[e];
            } else if (g <= nma + ntp) {
                c = canonical_entries(R);
                c.thd_off = canon[i];
            }
            pk.rx.push_back(c);
            pk.orig.push_back(i);
            pk.cls.push_back(g <= nma + ntp ? g : -1);
        }
        if (g == 0) pk.nr_e22 = (int)pk.rx.size();
        if (g == nma) pk.ma_off[nma] = (int)pk.rx.size();
        if (g == nma + ntp) pk.tp_off[ntp] = (int)pk.rx.size();
    }
    // RX_SAMEM: [M] equals the previous reaction's in the same group;
    // RX_SAMELNM: and an earlier reaction of that run formed ln [M] (a Troe or
    // SRI fall-off with both rate constants in exponential form, which forms
    // it whatever Pr)
    const int nr = (int)pk.rx.size();
    bool run_log = false;
    for (int q = 0; q < nr; ++q) {
        PjgRxn& c = pk.rx[q];
        c.flags &= ~(RX_SAMEM | RX_SAMELNM);
        const int g = pk.cls[q];
        const bool same = q > 0 && key[pk.orig[q]] >= 0 && key[pk.orig[q]] == key[pk.orig[q - 1]] &&
                          g == pk.cls[q - 1];
        if (!same) run_log = false;
        if (same) c.flags |= RX_SAMEM;
        if (same && run_log) c.flags |= RX_SAMELNM;
        const int blend = RX_BLEND(c.flags);
        if (RX_THD(c.flags) != THD_NONE && (blend == BL_TROE || blend == BL_SRI) &&
            RX_FORM(c.flags) == FORM_ARR && RX_FFORM(c.flags) == FORM_ARR)
            run_log = true;
    }
}

void order_reactions(pjg_mech* m)
{
    Packing pk;
    pack_reactions(m->h_rxn, m->h_thd_spec.data(), m->h_thd_coef.data(), pk);
    m->h_rxn.swap(pk.rx);
    m->nr_e22 = pk.nr_e22;
    for (int q = 0; q <= pjg::kMaPatterns; ++q) m->ma_off[q] = pk.ma_off[q];
    for (int q = 0; q <= pjg::kTpPatterns; ++q) m->tp_off[q] = pk.tp_off[q];
    // bound on a state's |b_k| under which 1 / Kc is formed from per-species
    // factors: 690 / (largest sum |nu| of a reversible reaction), at most
    // 690 / 5 (every coefficient pattern has sum |nu| <= 5)
    int numax = 5;
    for (const PjgRxn& R : m->h_rxn) {
        if (!(R.flags & RX_REV)) continue;
        int n = 0;
        for (int e = 0; e < R.nspec; ++e) {
            const int nu = ent_nur(R.ent[e]) - ent_nuf(R.ent[e]);
            n += nu < 0 ? -nu : nu;
        }
        numax = std::max(numax, n);
    }
    m->kc_split_max = 690.0 / numax;
}

}  // namespace

// Internal accessors for other translation units of this library.
int pjg_internal_fail(int code, const char* msg) { return fail(code, "%s", msg); }
void pjg_internal_fill_args(const pjg_mech* m, EvalArgs* a) { fill_common(m, *a); }
int pjg_internal_mech_ns(const pjg_mech* m) { return m->ns; }
int pjg_internal_check_device(const pjg_mech* m) { return check_device(m); }
void pjg_internal_count_launch() { g_launches.fetch_add(1); }

extern "C" {

int pjg_last_error(char* buf, size_t len)
{
    if (!buf || len == 0) return PJG_ERR_ARG;
    snprintf(buf, len, "%s", g_err);
    return 0;
}

int pjg_mlp_linear(const void* X, int64_t ldx, const void* W, int64_t ldw, int64_t M, int N, int K,
                   const float* bias, int act, const void* zprev, int64_t ldzp, void* Y, int64_t ldy,
                   void* YT, int64_t ldyt, void* Z, int64_t ldz, float* Y32, int64_t ldy32,
                   float* colsum, void* stream)
{
    if (M < 0) return fail(PJG_ERR_ARG, "negative row count");
    const int rc = mlp_launch_rows(X, ldx, W, ldw, M, N, K, bias, act, zprev, ldzp, Y, ldy, YT, ldyt,
                                   Z, ldz, Y32, ldy32, colsum, stream);
    if (rc == -1)
        return fail(PJG_ERR_ARG, "pjg_mlp_linear: unsupported shape or misaligned operand "
                                 "(N %% 32, K %% 16, N, K <= 256, leading dims %% 8, 16-byte aligned)");
    if (rc) return fail(PJG_ERR_CUDA, "pjg_mlp_linear launch failed: %s",
                        cudaGetErrorString(cudaGetLastError()));
    g_launches.fetch_add(1);
    return 0;
}

int pjg_mlp_wgrad(const void* A, int64_t lda, const void* B, int64_t ldb, int Mo, int No, int64_t Kb,
                  float* C, int64_t ldc, void* stream)
{
    const int rc = mlp_launch_wgrad(A, lda, B, ldb, Mo, No, Kb, C, ldc, stream);
    if (rc == -1)
        return fail(PJG_ERR_ARG, "pjg_mlp_wgrad: unsupported shape or misaligned operand "
                                 "(No %% 32, No <= 256, Kb %% 64, leading dims %% 8)");
    if (rc) return fail(PJG_ERR_CUDA, "pjg_mlp_wgrad launch failed: %s",
                        cudaGetErrorString(cudaGetLastError()));
    g_launches.fetch_add(1);
    return 0;
}

int pjg_mlp_status(int clear) { return mlp_error_flag(clear); }

int pjg_surrogate_features(int64_t n, int32_t nn, const double* phi, const double* param,
                           const double* stats, void* X, double floor_c, void* stream)
{
    if (n < 0 || (n && (!phi || !param || !stats || !X)))
        return fail(PJG_ERR_ARG, "pjg_surrogate_features: bad arguments");
    const int rc = surr_launch_features(n, nn, phi, param, stats, X, (float)floor_c, stream);
    if (rc == -1) return fail(PJG_ERR_ARG, "pjg_surrogate_features: 3 <= nn <= 64, X 16-byte aligned");
    if (rc) return fail(PJG_ERR_CUDA, "pjg_surrogate_features launch failed");
    if (n > 0) g_launches.fetch_add(1);
    return 0;
}

int pjg_surrogate_outputs(int64_t n, int32_t nn, const float* Y, const double* phi,
                          const double* param, const double* stats, int32_t err_col, double* dphi,
                          float* lerr, void* stream)
{
    if (n < 0 || (n && (!Y || !phi || !param || !stats || !dphi || !lerr)))
        return fail(PJG_ERR_ARG, "pjg_surrogate_outputs: bad arguments");
    const int rc = surr_launch_outputs(n, nn, Y, phi, param, stats, err_col, dphi, lerr, stream);
    if (rc == -1) return fail(PJG_ERR_ARG, "pjg_surrogate_outputs: 3 <= nn <= 65, 0 <= err_col < 64");
    if (rc) return fail(PJG_ERR_CUDA, "pjg_surrogate_outputs launch failed");
    if (n > 0) g_launches.fetch_add(1);
    return 0;
}

int pjg_mlp_forward(const void* X, int64_t ldx, int64_t M, const void* const* W,
                    const float* const* b, float* Y, int64_t ldy, void* stream)
{
    if (M < 0 || !W || !b) return fail(PJG_ERR_ARG, "pjg_mlp_forward: bad arguments");
    int rc = mlp_launch_fused(X, ldx, M, W, b, Y, ldy, stream);
    if (rc == -1)
        return fail(PJG_ERR_ARG, "pjg_mlp_forward: operands must be 16-byte aligned, ldx %% 8, "
                                 "ldy %% 4, ldx and ldy >= 64");
    if (rc) return fail(PJG_ERR_CUDA, "pjg_mlp_forward launch failed: %s",
                        cudaGetErrorString(cudaGetLastError()));
    if (M > 0) g_launches.fetch_add(1);
    return 0;
}

int pjg_fp64_peak(double* tflops)
{
    if (!tflops) return fail(PJG_ERR_ARG, "null argument");
    int dev = 0, sms = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    CUDA_TRY(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    double* out = nullptr;
    CUDA_TRY(cudaMalloc((void**)&out, sizeof(double) * 64 * sms));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int blocks = 8 * sms, threads = 256, iters = 4096;
    int rc = pjg_fp64_probe(blocks, threads, 64, out, nullptr);  // warm-up
    cudaEventRecord(e0, nullptr);
    rc |= pjg_fp64_probe(blocks, threads, iters, out, nullptr);
    cudaEventRecord(e1, nullptr);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (rc) return fail(PJG_ERR_CUDA, "fp64 probe launch failed");
    *tflops = 2.0 * 8.0 * iters * (double)blocks * threads / (ms * 1e-3) / 1e12;
    return 0;
}

int pjg_chem_utils(pjg_mech* m, int64_t n, char order, int conp, const double* phi, double* cp,
                   double* h, double* b, void* stream)
{
    if (!m) return fail(PJG_ERR_ARG, "null mechanism");
    if (n < 0) return fail(PJG_ERR_ARG, "negative problem size");
    if (order != 'C' && order != 'F') return fail(PJG_ERR_ARG, "order must be 'C' or 'F'");
    if (n == 0) return 0;
    if (!phi || !cp || !h || !b) return fail(PJG_ERR_ARG, "null array");
    const bool F = order == 'F';
    if (pjg_launch_chem_utils(m->sp, m->ns, n, conp, phi, F ? 1 : m->nn, cp, h, b, F ? 1 : m->ns,
                              F ? n : 1, stream))
        return fail(PJG_ERR_CUDA, "chem_utils launch failed");
    g_launches.fetch_add(1);
    return 0;
}

int pjg_math_exp(const double* x, double* y, int64_t n, void* stream)
{
    if (n < 0) return fail(PJG_ERR_ARG, "negative size");
    if (n == 0) return 0;
    if (!x || !y) return fail(PJG_ERR_ARG, "null array");
    if (pjg_launch_fexp(x, y, n, stream)) return fail(PJG_ERR_CUDA, "exp launch failed");
    g_launches.fetch_add(1);
    return 0;
}

int pjg_host_register(void* ptr, size_t bytes)
{
    if (!ptr || !bytes) return fail(PJG_ERR_ARG, "null or empty host range");
    CUDA_TRY(cudaHostRegister(ptr, bytes, cudaHostRegisterDefault));
    return 0;
}

int pjg_host_unregister(void* ptr)
{
    if (!ptr) return fail(PJG_ERR_ARG, "null host pointer");
    CUDA_TRY(cudaHostUnregister(ptr));
    return 0;
}

int pjg_launch_count(int64_t* count)
{
    if (!count) return fail(PJG_ERR_ARG, "null argument");
    *count = g_launches.load();
    return 0;
}

int pjg_profile_begin(void)
{
    std::lock_guard<std::mutex> g(g_prof_mu);
    for (auto& e : g_prof_events) {
        cudaEventDestroy(e.first);
        cudaEventDestroy(e.second);
    }
    g_prof_events.clear();
    g_prof_on.store(true);
    return 0;
}

int pjg_profile_end(int64_t* launches, double* total_ms)
{
    g_prof_on.store(false);
    std::lock_guard<std::mutex> g(g_prof_mu);
    double tot = 0.0;
    int rc = 0;
    for (auto& e : g_prof_events) {
        float ms = 0.0f;
        if (cudaEventSynchronize(e.second) != cudaSuccess ||
            cudaEventElapsedTime(&ms, e.first, e.second) != cudaSuccess)
            rc = fail(PJG_ERR_CUDA, "profiling event query failed");
        tot += ms;
        cudaEventDestroy(e.first);
        cudaEventDestroy(e.second);
    }
    if (launches) *launches = (int64_t)g_prof_events.size();
    if (total_ms) *total_ms = tot;
    g_prof_events.clear();
    return rc;
}


int pjg_mech_create(const pjg_tables* tb, pjg_mech** out)
{
    if (!tb || !out) return fail(PJG_ERR_ARG, "null argument");
    *out = nullptr;
    if (tb->ns < 2 || tb->nr < 0 || !tb->species || (tb->nr > 0 && !tb->rxn))
        return fail(PJG_ERR_TABLES, "invalid species/reaction counts");
    const int NN = tb->ns + 1;
    if (tb->nnz <= 0 || !tb->crs_row_ptr || !tb->crs_col_ind || !tb->ccs_col_ptr || !tb->ccs_row_ind)
        return fail(PJG_ERR_TABLES, "missing Jacobian pattern");
    pjg_mech* m = new pjg_mech();
    m->ns = tb->ns;
    m->nr = tb->nr;
    m->nn = NN;
    m->need_logP = tb->flags & 1;
    m->jac_approx = (tb->flags >> 1) & 1;
    m->nnz = tb->nnz;
    cudaGetDevice(&m->device);
    const PjgRxn* r = (const PjgRxn*)tb->rxn;
    m->h_rxn.assign(r, r + tb->nr);
    m->h_thd_spec.assign(tb->thd_spec, tb->thd_spec + std::max(tb->n_thd, 0));
    m->h_thd_coef.assign(tb->thd_coef, tb->thd_coef + std::max(tb->n_thd, 0));
    for (const PjgRxn& R : m->h_rxn) {
        if (R.nspec < 1 || R.nspec > PJG_MAXSP || R.thd_off < 0 || R.thd_cnt < 0 ||
            R.thd_off + R.thd_cnt > tb->n_thd) {
            delete m;
            return fail(PJG_ERR_TABLES, "reaction record out of range");
        }
        for (int e = 0; e < R.nspec; ++e)
            if (ent_spec(R.ent[e]) >= tb->ns) {
                delete m;
                return fail(PJG_ERR_TABLES, "species index out of range");
            }
        if (RX_FORM(R.flags) >= FORM_PLOG && (R.aux < 0 || R.aux >= tb->n_aux)) {
            delete m;
            return fail(PJG_ERR_TABLES, "PLOG/Chebyshev block out of range");
        }
    }
    for (int l = 0; l < tb->n_thd; ++l)
        if (tb->thd_spec[l] < 0 || tb->thd_spec[l] >= tb->ns) {
            delete m;
            return fail(PJG_ERR_TABLES, "third-body species out of range");
        }
    order_reactions(m);
    m->crs_ptr.assign(tb->crs_row_ptr, tb->crs_row_ptr + NN + 1);
    m->crs_ind.assign(tb->crs_col_ind, tb->crs_col_ind + tb->nnz);
    m->ccs_ptr.assign(tb->ccs_col_ptr, tb->ccs_col_ptr + NN + 1);
    m->ccs_ind.assign(tb->ccs_row_ind, tb->ccs_row_ind + tb->nnz);
    if (m->crs_ptr[NN] != tb->nnz || m->ccs_ptr[NN] != tb->nnz) {
        delete m;
        return fail(PJG_ERR_TABLES, "pattern pointers inconsistent with nnz");
    }
    std::vector<PjgRxn> rx(m->h_rxn);
    std::vector<double> sp(tb->species, tb->species + (size_t)tb->ns * PJG_SP_DOUBLES);
    std::vector<double> coef(tb->thd_coef, tb->thd_coef + std::max(tb->n_thd, 0));
    std::vector<double> aux(tb->aux ? tb->aux : (const double*)nullptr,
                            tb->aux ? tb->aux + std::max(tb->n_aux, 0) : (const double*)nullptr);
    int rc;
    if ((rc = upload(rx, &m->rxn)) || (rc = upload(sp, &m->sp)) ||
        (rc = upload(m->h_thd_spec, &m->thd_spec)) || (rc = upload(coef, &m->thd_coef)) ||
        (rc = upload(aux, &m->aux))) {
        pjg_mech_destroy(m);
        return rc;
    }
    *out = m;
    return 0;
}

int pjg_mech_destroy(pjg_mech* m)
{
    if (!m) return 0;
    cudaFree(m->rxn);
    cudaFree(m->sp);
    cudaFree(m->thd_spec);
    cudaFree(m->thd_coef);
    cudaFree(m->aux);
    cudaFree(m->work);
    pjg_internal_lu_plan_destroy(m->lu_plan);
    for (auto& kv : m->slots) {
        SlotTables& t = kv.second;
        cudaFree(t.rxn_slot_off);
        cudaFree(t.rxn_slots);
        cudaFree(t.row_off);
        cudaFree(t.row_list);
        cudaFree(t.col_off);
        cudaFree(t.col_list);
        cudaFree(t.sp_slots);
        cudaFree(t.cj_slots);
        cudaFree(t.dchunk_off);
        cudaFree(t.dchunk_list);
        cudaFree(t.dchunk_slots);
    }
    delete m;
    return 0;
}

int pjg_reaction_order(const pjg_tables* tb, int32_t* orig, int32_t* cls, int32_t* flags)
{
    if (!tb || tb->nr < 0 || (tb->nr > 0 && (!tb->rxn || !orig || !cls)))
        return fail(PJG_ERR_ARG, "invalid tables or null output");
    const PjgRxn* r = (const PjgRxn*)tb->rxn;
    for (int i = 0; i < tb->nr; ++i)
        if (r[i].nspec < 1 || r[i].nspec > PJG_MAXSP)
            return fail(PJG_ERR_TABLES, "reaction record out of range");
    for (int i = 0; i < tb->nr; ++i)
        if (r[i].thd_off < 0 || r[i].thd_cnt < 0 || r[i].thd_off + r[i].thd_cnt > std::max(tb->n_thd, 0) ||
            (r[i].thd_cnt > 0 && (!tb->thd_spec || !tb->thd_coef)))
            return fail(PJG_ERR_TABLES, "reaction record out of range");
    Packing pk;
    pack_reactions(std::vector<PjgRxn>(r, r + tb->nr), tb->thd_spec, tb->thd_coef, pk);
    for (int p = 0; p < tb->nr; ++p) {
        orig[p] = pk.orig[p];
        cls[p] = pk.cls[p];
        if (flags) flags[p] = pk.rx[p].flags;
    }
    return 0;
}

int pjg_mech_info(const pjg_mech* m, int32_t* ns, int32_t* nr, int32_t* nnz)
{
    if (!m) return fail(PJG_ERR_ARG, "null mechanism");
    if (ns) *ns = m->ns;
    if (nr) *nr = m->nr;
    if (nnz) *nnz = m->nnz;
    return 0;
}

int pjg_jacobian_indices(const pjg_mech* m, char order, int32_t* ptr, int32_t* ind, int32_t* nnz)
{
    if (!m) return fail(PJG_ERR_ARG, "null mechanism");
    if (order != 'C' && order != 'F') return fail(PJG_ERR_ARG, "order must be 'C' or 'F'");
    const std::vector<int>& p = order == 'C' ? m->crs_ptr : m->ccs_ptr;
    const std::vector<int>& q = order == 'C' ? m->crs_ind : m->ccs_ind;
    if (nnz) *nnz = m->nnz;
    if (ptr) memcpy(ptr, p.data(), p.size() * sizeof(int32_t));
    if (ind) memcpy(ind, q.data(), q.size() * sizeof(int32_t));
    return 0;
}

int pjg_species_rates(pjg_mech* m, int64_t n, char order, int conp, const double* param,
                      const double* phi, double* dphi, void* stream)
{
    return run_eval(m, PJG_SPECIES_RATES, n, order, conp, 0, param, phi, dphi, (cudaStream_t)stream);
}

int pjg_jacobian(pjg_mech* m, int64_t n, char order, int conp, int jac_format, const double* param,
                 const double* phi, double* jac, void* stream)
{
    return run_eval(m, PJG_JACOBIAN, n, order, conp, jac_format, param, phi, jac,
                    (cudaStream_t)stream);
}

int pjg_jacobian_rates(pjg_mech* m, int64_t n, char order, int conp, int jac_format,
                       const double* param, const double* phi, double* jac, double* dphi, void* stream)
{
    if (n > 0 && !dphi) return fail(PJG_ERR_ARG, "null array");
    return run_eval(m, PJG_JACOBIAN, n, order, conp, jac_format, param, phi, jac, (cudaStream_t)stream,
                    nullptr, nullptr, 0, dphi);
}

int pjg_eval_chunk(pjg_mech* m, int kind, int64_t n, char order, int jac_format, int64_t* states)
{
    if (!states) return fail(PJG_ERR_ARG, "null argument");
    if (kind < 0 || kind > 2) return fail(PJG_ERR_ARG, "bad kind");
    *states = 0;
    if (!m) return fail(PJG_ERR_ARG, "null mechanism");
    if (order != 'C' && order != 'F') return fail(PJG_ERR_ARG, "order must be 'C' or 'F'");
    if (n <= 0) return 0;
    SlotTables* t = nullptr;
    if (kind == PJG_JACOBIAN) {
        int rc = build_slots(m, order == 'F', jac_format == PJG_JAC_SPARSE, &t);
        if (rc) return rc;
    }
    *states = chunk_states(eval_state_bytes(m, kind, order == 'F', t), n, wave_states(m, kind));
    return 0;
}

int pjg_vjp(pjg_mech* m, int64_t n, char order, int conp, const double* param, const double* phi,
            const double* v, double* out, void* stream)
{
    return run_eval(m, PJG_KIND_VJP, n, order, conp, 0, param, phi, out, (cudaStream_t)stream, v);
}

int pjg_internal_lu_factor(int32_t nn, int64_t n, char order, double s, const double* h, double h0,
                           const double* jac, double* lu, int32_t* piv, int32_t* info,
                           cudaStream_t st);
int pjg_internal_lu_solve(int32_t nn, int64_t n, char order, const double* lu, const int32_t* piv,
                          double* b, cudaStream_t st);
int pjg_internal_ros2_combine(int op, int32_t nn, int64_t n, char order, const double* h, double h0,
                              const double* x, const double* k, const double* z, double* out,
                              double* err, cudaStream_t st);

static int lu_plan_of(pjg_mech* m, void** plan)
{
    std::lock_guard<std::mutex> g(m->lock);
    if (!m->lu_plan) {
        int rc = pjg_internal_lu_plan_create(m->nn, m->crs_ptr.data(), m->crs_ind.data(), &m->lu_plan);
        if (rc) return rc;
    }
    *plan = m->lu_plan;
    return 0;
}

int pjg_lu_plan_info(pjg_mech* m, int32_t* perm, int32_t* nnz_lu, int64_t* fma)
{
    if (!m) return fail(PJG_ERR_ARG, "null mechanism");
    void* pl = nullptr;
    if (int rc = lu_plan_of(m, &pl)) return rc;
    pjg_internal_lu_plan_info(pl, perm, nnz_lu, fma);
    return 0;
}

int pjg_lu_factor_sparse(pjg_mech* m, int64_t n, char order, double s, const double* h, double h0,
                         const double* jac, double* lu, int32_t* info, void* stream)
{
    if (!m) return fail(PJG_ERR_ARG, "null mechanism");
    void* pl = nullptr;
    if (int rc = lu_plan_of(m, &pl)) return rc;
    return pjg_internal_lu_factor_sparse(pl, n, order, s, h, h0, jac, lu, info, (cudaStream_t)stream);
}

int pjg_lu_solve_sparse(pjg_mech* m, int64_t n, char order, const double* lu, double* b, void* stream)
{
    if (!m) return fail(PJG_ERR_ARG, "null mechanism");
    void* pl = nullptr;
    if (int rc = lu_plan_of(m, &pl)) return rc;
    return pjg_internal_lu_solve_sparse(pl, n, order, lu, b, (cudaStream_t)stream);
}

// One step of ROS2 (Verwer, Spee, Blom and Hundsdorfer, SIAM J. Sci. Comput.
// 20(4), 1999), gamma = 1 + 1/sqrt(2):
//   (I - gamma h J) k1 = f(y),  (I - gamma h J) k2 = f(y + h k1) - 2 k1,
//   y_new = y + 1.5 h k1 + 0.5 h k2,  err = y_new - (y + h k1) = 0.5 h (k1 + k2),
// with J the analytical Jacobian at y and f the species rates (f(y) from the
// Jacobian's own pass, so one rates evaluation per step).  lu_kind 0
// factors with partial pivoting, 1 with the mechanism's static-pivot sparse
// plan (piv_work unused).
int pjg_ros2_step(pjg_mech* m, int64_t n, char order, int conp, const double* param,
                  const double* phi, const double* h, double h0, int lu_kind, double* phi_new,
                  double* err, double* jac_work, int32_t* piv_work, double* vec_work, int32_t* info,
                  void* stream)
{
    if (!m) return fail(PJG_ERR_ARG, "null mechanism");
    if (n < 0) return fail(PJG_ERR_ARG, "negative problem size");
    if (lu_kind != 0 && lu_kind != 1) return fail(PJG_ERR_ARG, "lu_kind must be 0 or 1");
    if (n == 0) return 0;
    if (!phi || !param || !phi_new || !jac_work || !vec_work || (lu_kind == 0 && !piv_work))
        return fail(PJG_ERR_ARG, "null array");
    if (phi_new == phi) return fail(PJG_ERR_ARG, "phi_new must not alias phi");
    const cudaStream_t st = (cudaStream_t)stream;
    const int nn = m->nn;
    const double gamma = 1.7071067811865475;  // 1 + 1/sqrt(2)
    void* plan = nullptr;
    if (lu_kind == 1)
        if (int rc = lu_plan_of(m, &plan)) return rc;
    auto factor = [&]() {
        return lu_kind == 0
                   ? pjg_internal_lu_factor(nn, n, order, gamma, h, h0, jac_work, jac_work, piv_work, info, st)
                   : pjg_internal_lu_factor_sparse(plan, n, order, gamma, h, h0, jac_work, jac_work, info, st);
    };
    auto solve = [&](double* b) {
        return lu_kind == 0 ? pjg_internal_lu_solve(nn, n, order, jac_work, piv_work, b, st)
                            : pjg_internal_lu_solve_sparse(plan, n, order, jac_work, b, st);
    };
    double* k1 = vec_work;
    double* k2 = vec_work + (size_t)n * nn;
    // f(y) comes out of the Jacobian's pass
    int rc = run_eval(m, PJG_JACOBIAN, n, order, conp, PJG_JAC_FULL, param, phi, jac_work, st, nullptr,
                      nullptr, 0, k1);
    if (!rc) rc = factor();
    if (!rc) rc = solve(k1);
    if (!rc) rc = pjg_internal_ros2_combine(0, nn, n, order, h, h0, phi, k1, nullptr, phi_new, nullptr, st);
    if (!rc) rc = run_eval(m, PJG_SPECIES_RATES, n, order, conp, 0, param, phi_new, k2, st);
    if (!rc) rc = pjg_internal_ros2_combine(1, nn, n, order, h, h0, k2, k1, nullptr, k2, nullptr, st);
    if (!rc) rc = solve(k2);
    if (!rc) rc = pjg_internal_ros2_combine(2, nn, n, order, h, h0, phi, k1, k2, phi_new, err, st);
    return rc;
}

int pjg_kernel_create(pjg_mech* m, int kind, size_t problem_size, size_t work_size, char order,
                      int conp, int jac_format, pjg_kernel** out)
{
    if (!m || !out) return fail(PJG_ERR_ARG, "null argument");
    if (kind != PJG_SPECIES_RATES && kind != PJG_JACOBIAN) return fail(PJG_ERR_ARG, "bad kind");
    if (order != 'C' && order != 'F') return fail(PJG_ERR_ARG, "order must be 'C' or 'F'");
    if (jac_format != PJG_JAC_FULL && jac_format != PJG_JAC_SPARSE)
        return fail(PJG_ERR_ARG, "bad jac_format");
    pjg_kernel* k = new pjg_kernel();
    k->mech = m;
    k->kind = kind;
    k->order = order;
    k->conp = conp;
    k->jac_format = jac_format;
    k->out_per_state = kind == PJG_SPECIES_RATES ? m->nn
                       : (jac_format == PJG_JAC_SPARSE ? (size_t)m->nnz : (size_t)m->nn * m->nn);
    bool ok = cudaStreamCreateWithFlags(&k->s_in, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&k->s_comp, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&k->s_out, cudaStreamNonBlocking) == cudaSuccess;
    for (int b = 0; ok && b < kRing; ++b)
        ok = cudaEventCreateWithFlags(&k->ev_in[b], cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&k->ev_k[b], cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&k->ev_out[b], cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
        pjg_kernel_destroy(k);
        return fail(PJG_ERR_CUDA, "stream or event creation failed");
    }
    int rc = pjg_kernel_resize(k, problem_size, work_size);
    if (rc) {
        pjg_kernel_destroy(k);
        return rc;
    }
    *out = k;
    return 0;
}

namespace {

void free_buffers(pjg_kernel* k)
{
    for (int b = 0; b < kRing; ++b) {
        cudaFree(k->d_param[b]);
        cudaFree(k->d_phi[b]);
        cudaFree(k->d_out[b]);
        k->d_param[b] = k->d_phi[b] = k->d_out[b] = nullptr;
    }
    cudaFree(k->work);
    k->work = nullptr;
    k->work_bytes = 0;
    k->chunk = 0;
}

}  // namespace

int pjg_kernel_resize(pjg_kernel* k, size_t problem_size, size_t work_size)
{
    if (!k) return fail(PJG_ERR_ARG, "null kernel");
    k->work_size = work_size;
    pjg_mech* m = k->mech;
    SlotTables* t = nullptr;
    if (k->kind == PJG_JACOBIAN && problem_size) {
        int rc = build_slots(m, k->order == 'F', k->jac_format == PJG_JAC_SPARSE, &t);
        if (rc) return rc;
    }
    const size_t nn = m->nn;
    const size_t per_state = eval_state_bytes(m, k->kind, k->order == 'F', t);
    // two waves per chunk; where the ring and working arrays of two waves
    // would pass the kernel object's budget (large mechanisms), as many whole
    // waves as the budget holds, and at least one wave if half the free
    // device memory holds it: a launch of part of a wave takes as long as a
    // whole one (synthetic 500-species sparse C-order Jacobian, 1.37 MB per
    // state: a third-of-a-wave chunk ran end to end at 48 % of the copy floor)
    const size_t ring_state = kRing * (1 + nn + k->out_per_state) * sizeof(double) + per_state;
    const int64_t wave = wave_states(m, PJG_JACOBIAN);
    int64_t chunk = std::min<int64_t>((int64_t)problem_size, PJG_CHUNK_WAVES * wave);
    if ((size_t)chunk * ring_state > kKernelBudget) {
        int64_t c = (int64_t)(kKernelBudget / ring_state);
        if (c >= wave) {
            c = c / wave * wave;
        } else {
            size_t free_b = 0, total_b = 0;
            if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) free_b = 0;
            c = std::max<int64_t>(c, std::min<int64_t>((int64_t)(free_b / 2 / ring_state), wave));
        }
        chunk = std::min<int64_t>((int64_t)problem_size,
                                  std::max<int64_t>(PJG_BLOCK, c / PJG_BLOCK * PJG_BLOCK));
    }
    if (chunk == k->chunk && k->d_phi[0]) {
        k->problem_size = problem_size;
        return 0;
    }
    free_buffers(k);
    k->problem_size = problem_size;
    if (problem_size == 0) return 0;
    for (int b = 0; b < kRing; ++b) {
        CUDA_TRY(cudaMalloc((void**)&k->d_param[b], chunk * sizeof(double)));
        CUDA_TRY(cudaMalloc((void**)&k->d_phi[b], chunk * nn * sizeof(double)));
        CUDA_TRY(cudaMalloc((void**)&k->d_out[b], chunk * k->out_per_state * sizeof(double)));
    }
    const int64_t padded = (chunk + PJG_BLOCK - 1) / PJG_BLOCK * PJG_BLOCK;
    k->work_bytes = per_state * (size_t)padded;
    if (k->work_bytes) CUDA_TRY(cudaMalloc((void**)&k->work, k->work_bytes));
    k->chunk = chunk;
    return 0;
}

}  // extern "C"

namespace {

// The copy-evaluate-copy pipeline of one pjg_kernel_call.  An error may return
// with copies still queued on the kernel object's streams; the caller
// synchronises them.
int kernel_stream(pjg_kernel* k, const double* param, const double* phi, double* out)
{
    const int64_t n = (int64_t)k->problem_size, nn = k->mech->nn, no = (int64_t)k->out_per_state;
    const bool F = k->order == 'F';
    const int64_t C = k->chunk;
    for (int64_t c = 0, s0 = 0; s0 < n; ++c, s0 += C) {
        const int b = (int)(c % kRing);
        const int64_t cnt = std::min<int64_t>(C, n - s0);
        if (c >= kRing) CUDA_TRY(cudaStreamWaitEvent(k->s_in, k->ev_k[b], 0));
        CUDA_TRY(cudaMemcpyAsync(k->d_param[b], param + s0, cnt * sizeof(double),
                                 cudaMemcpyHostToDevice, k->s_in));
        if (F)  // field j of the chunk: cnt contiguous doubles at phi[s0 + n * j]
            CUDA_TRY(cudaMemcpy2DAsync(k->d_phi[b], cnt * sizeof(double), phi + s0, n * sizeof(double),
                                       cnt * sizeof(double), nn, cudaMemcpyHostToDevice, k->s_in));
        else
            CUDA_TRY(cudaMemcpyAsync(k->d_phi[b], phi + s0 * nn, cnt * nn * sizeof(double),
                                     cudaMemcpyHostToDevice, k->s_in));
        CUDA_TRY(cudaEventRecord(k->ev_in[b], k->s_in));
        CUDA_TRY(cudaStreamWaitEvent(k->s_comp, k->ev_in[b], 0));
        if (c >= kRing) CUDA_TRY(cudaStreamWaitEvent(k->s_comp, k->ev_out[b], 0));
        int rc = run_eval(k->mech, k->kind, cnt, k->order, k->conp, k->jac_format, k->d_param[b],
                          k->d_phi[b], k->d_out[b], k->s_comp, nullptr, k->work, k->work_bytes);
        if (rc) return rc;
        CUDA_TRY(cudaEventRecord(k->ev_k[b], k->s_comp));
        CUDA_TRY(cudaStreamWaitEvent(k->s_out, k->ev_k[b], 0));
        if (F)
            CUDA_TRY(cudaMemcpy2DAsync(out + s0, n * sizeof(double), k->d_out[b], cnt * sizeof(double),
                                       cnt * sizeof(double), no, cudaMemcpyDeviceToHost, k->s_out));
        else
            CUDA_TRY(cudaMemcpyAsync(out + s0 * no, k->d_out[b], cnt * no * sizeof(double),
                                     cudaMemcpyDeviceToHost, k->s_out));
        CUDA_TRY(cudaEventRecord(k->ev_out[b], k->s_out));
    }
    CUDA_TRY(cudaStreamSynchronize(k->s_out));
    CUDA_TRY(cudaStreamSynchronize(k->s_comp));
    return 0;
}

}  // namespace

extern "C" {

int pjg_kernel_call(pjg_kernel* k, const double* param, const double* phi, double* out)
{
    if (!k) return fail(PJG_ERR_ARG, "null kernel");
    if (k->problem_size == 0) return 0;
    if (!param || !phi || !out) return fail(PJG_ERR_ARG, "null array");
    const int rc = kernel_stream(k, param, phi, out);
    if (rc) {
        // copies from and to the caller's host arrays may still be queued: let
        // them finish before the caller may free or reuse those arrays
        cudaStreamSynchronize(k->s_in);
        cudaStreamSynchronize(k->s_comp);
        cudaStreamSynchronize(k->s_out);
    }
    return rc;
}

int pjg_kernel_required_memory(const pjg_kernel* k, size_t* bytes)
{
    if (!k || !bytes) return fail(PJG_ERR_ARG, "null argument");
    *bytes = (size_t)kRing * k->chunk * (1 + k->mech->nn + k->out_per_state) * sizeof(double) +
             k->work_bytes;
    return 0;
}

int pjg_kernel_destroy(pjg_kernel* k)
{
    if (!k) return 0;
    if (k->s_out) cudaStreamSynchronize(k->s_out);
    if (k->s_comp) cudaStreamSynchronize(k->s_comp);
    free_buffers(k);
    for (int b = 0; b < kRing; ++b) {
        if (k->ev_in[b]) cudaEventDestroy(k->ev_in[b]);
        if (k->ev_k[b]) cudaEventDestroy(k->ev_k[b]);
        if (k->ev_out[b]) cudaEventDestroy(k->ev_out[b]);
    }
    if (k->s_in) cudaStreamDestroy(k->s_in);
    if (k->s_comp) cudaStreamDestroy(k->s_comp);
    if (k->s_out) cudaStreamDestroy(k->s_out);
    delete k;
    return 0;
}

}  // extern "C"
