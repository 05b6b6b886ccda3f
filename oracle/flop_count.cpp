/*
 * FP64 operation counter of the oracle (test and measurement infrastructure,
 * like pyjac_oracle.c itself; the product never links it).
 *
 * The oracle restates the reference's arithmetic for species rates and the
 * analytical Jacobian (pyjac/core/rate_subs.py:597-3278,
 * pyjac/core/create_jacobian.py:285-4522).  This translation unit compiles
 * the same source as C++ with every `double` replaced by orc_cd, a double
 * that counts the operations applied to it: additions and subtractions,
 * multiplications, divisions and fused multiply-adds, min/max guards, and
 * each transcendental function (exp, log, log10, pow) by name.  The counts
 * of one evaluation are the algorithmic FP64 work per state of the
 * reference's formulation, the denominator-free numerator of the FP64
 * roofline: flops = add + mul + div + 2 fma, transcendentals reported
 * separately.  The test-metric sums of the oracle (cancellation scales) are
 * compiled out (ORC_COUNTING).
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

namespace {

struct Counts {
    long long add, mul, div, fma, minmax, exp, log, log10, pow, sqrt;
};
thread_local Counts g_c;

}  // namespace

struct orc_cd {
    double v;
    orc_cd() = default;
    orc_cd(double x) : v(x) {}
    explicit operator double() const { return v; }
    explicit operator int() const { return (int)v; }
    explicit operator long() const { return (long)v; }
    orc_cd operator-() const { return orc_cd(-v); }
    orc_cd operator+() const { return *this; }
    orc_cd& operator+=(orc_cd o) { ++g_c.add; v += o.v; return *this; }
    orc_cd& operator-=(orc_cd o) { ++g_c.add; v -= o.v; return *this; }
    orc_cd& operator*=(orc_cd o) { ++g_c.mul; v *= o.v; return *this; }
    orc_cd& operator/=(orc_cd o) { ++g_c.div; v /= o.v; return *this; }
};
static_assert(sizeof(orc_cd) == sizeof(double), "orc_cd must lay out like double");

#define ORC_BINOP(op, field)                                                                   \
    static inline orc_cd operator op(orc_cd a, orc_cd b) { ++g_c.field; return orc_cd(a.v op b.v); } \
    static inline orc_cd operator op(orc_cd a, double b) { ++g_c.field; return orc_cd(a.v op b); }   \
    static inline orc_cd operator op(double a, orc_cd b) { ++g_c.field; return orc_cd(a op b.v); }
ORC_BINOP(+, add)
ORC_BINOP(-, add)
ORC_BINOP(*, mul)
ORC_BINOP(/, div)
#undef ORC_BINOP
#define ORC_CMP(op)                                                                            \
    static inline bool operator op(orc_cd a, orc_cd b) { return a.v op b.v; }                    \
    static inline bool operator op(orc_cd a, double b) { return a.v op b; }                      \
    static inline bool operator op(double a, orc_cd b) { return a op b.v; }
ORC_CMP(<)
ORC_CMP(>)
ORC_CMP(<=)
ORC_CMP(>=)
ORC_CMP(==)
ORC_CMP(!=)
#undef ORC_CMP

static inline orc_cd fmin(orc_cd a, orc_cd b) { ++g_c.minmax; return orc_cd(::fmin(a.v, b.v)); }
static inline orc_cd fmax(orc_cd a, orc_cd b) { ++g_c.minmax; return orc_cd(::fmax(a.v, b.v)); }
static inline orc_cd fabs(orc_cd a) { return orc_cd(::fabs(a.v)); }
static inline bool isfinite(orc_cd a) { return std::isfinite(a.v); }
static inline orc_cd fma(orc_cd a, orc_cd b, orc_cd c) { ++g_c.fma; return orc_cd(::fma(a.v, b.v, c.v)); }
static inline orc_cd exp(orc_cd a) { ++g_c.exp; return orc_cd(::exp(a.v)); }
static inline orc_cd log(orc_cd a) { ++g_c.log; return orc_cd(::log(a.v)); }
static inline orc_cd log10(orc_cd a) { ++g_c.log10; return orc_cd(::log10(a.v)); }
static inline orc_cd pow(orc_cd a, orc_cd b) { ++g_c.pow; return orc_cd(::pow(a.v, b.v)); }
static inline orc_cd sqrt(orc_cd a) { ++g_c.sqrt; return orc_cd(::sqrt(a.v)); }

#define ORC_COUNTING 1
#define double orc_cd
#include "pyjac_oracle.c"
#undef double

extern "C" {

/* Operation counts of `n` evaluations (kind 0: species rates, 1: dense
 * Jacobian) of the states (param, phi) in C order, summed; counts[10] =
 * (add, mul, div, fma, minmax, exp, log, log10, pow, sqrt).  Single thread. */
int orc_count_ops(const orc_mech* m, int kind, long n, int conp, const double* param,
                  const double* phi, long long* counts)
{
    if (!m || n <= 0 || !param || !phi || !counts) return -1;
    const int NN = m->ns + 1;
    ws w;
    if (ws_alloc(m, &w)) return -2;
    orc_cd* jac = kind == 1 ? (orc_cd*)malloc(sizeof(orc_cd) * (size_t)NN * NN) : nullptr;
    if (kind == 1 && !jac) {
        free(w.conc);
        return -2;
    }
    g_c = Counts{};
    for (long s = 0; s < n; ++s) {
        const orc_cd* ph = reinterpret_cast<const orc_cd*>(phi) + (size_t)s * NN;
        if (kind == 1)
            eval_jacobian(m, conp, orc_cd(param[s]), ph, &w, jac);
        else
            eval_rates(m, conp, orc_cd(param[s]), ph, &w);
    }
    const Counts c = g_c;
    const long long out[10] = {c.add, c.mul, c.div, c.fma, c.minmax, c.exp, c.log, c.log10, c.pow, c.sqrt};
    memcpy(counts, out, sizeof(out));
    free(jac);
    free(w.conc);
    return 0;
}

}  // extern "C"
