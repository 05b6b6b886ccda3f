/*
 * pyjac-v2_gb300 internal entry points: instrumentation and test hooks.
 *
 * These are exported by the same library as include/pyjac_gb300.h but are not
 * part of the drop-in boundary: the benchmark driver (bench.py) and the tests
 * use them to count launches, time the evaluation kernels and measure the
 * FP64 roofline and the exponential's error.  None has a reference
 * counterpart; the reference prints wall-clock timings from its generated
 * main (pyjac/kernel_utils/common/kernel.cpp.in:645-712).
 */
#ifndef PYJAC_GB300_INTERNAL_H
#define PYJAC_GB300_INTERNAL_H
#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* pjg_launch_count: GPU kernel launches this library has issued so far.
 * pjg_profile_begin / pjg_profile_end: record CUDA events around every launch
 * of the evaluation kernels between the two calls; end synchronises those
 * events and returns their number and summed duration in milliseconds. */
int pjg_launch_count(int64_t* count);
/* Measured dense FP64 FMA throughput of the current device in TFLOP/s (the
 * denominator of the FP64 roofline; runs a ~10 ms probe kernel). */
int pjg_fp64_peak(double* tflops);
int pjg_profile_begin(void);
int pjg_profile_end(int64_t* launches, double* total_ms);
/* y = exp(x) through the table-driven exponential the evaluation kernels use
 * for rate constants, equilibrium constants and fall-off blending (device
 * pointers, asynchronous on `stream`); exposed so that its error against the
 * CUDA library exp can be measured.  No reference counterpart. */
int pjg_math_exp(const double* x, double* y, int64_t n, void* stream);
/* States per launch of the device-pointer entry points for n states (kind 0
 * species rates, 1 Jacobian, 2 J^T v; order and jac_format as for
 * pjg_jacobian): larger problems run as several launches of this size, the
 * last one shorter.  Lets a checker sample the states at launch boundaries. */
struct pjg_mech;
struct pjg_tables;
/* The reaction order of the device tables, computed on the host without a
 * device: for packed position p, orig[p] is the mechanism's reaction index
 * and cls[p] the code that evaluates it (0 the elementary class
 * A + B <=> C + D, 1..10 the mass-action patterns, 11..13 the third-body and
 * fall-off patterns, -1 the general code); flags[p] (if flags is not NULL)
 * the packed record's flag word, with the packing's marks 1 << 20 ([M]
 * equals the previous record's) and 1 << 21 (ln [M] formed earlier in that
 * run).  Each array holds tables->nr entries. */
int pjg_reaction_order(const struct pjg_tables* tables, int32_t* orig, int32_t* cls,
                       int32_t* flags);
int pjg_eval_chunk(struct pjg_mech* mech, int kind, int64_t n, char order, int jac_format,
                   int64_t* states);

#ifdef __cplusplus
}
#endif
#endif
