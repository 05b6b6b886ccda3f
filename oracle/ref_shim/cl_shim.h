/*
 * OpenCL-C -> host C++ shim for the reference's shipped generated kernels.
 *
 * Test infrastructure only: this header lets the generated OpenCL files under
 * pyJac-v2's examples/opencl/<mech>/ (species_rates.ocl, chem_utils.ocl,
 * jacobian.ocl) compile as one host C++ translation unit so that the
 * reference's own arithmetic can serve as the numeric oracle.
 *
 * The generated kernels are "wide" vectorised (reqd_work_group_size 128) and
 * contain no barriers, local memory or atomics: every work item evaluates its
 * own state end to end, addressing its working buffer as
 * rwk[128 * gid + lid + work_size * 128 * i]
 * (examples/opencl/h2o2/species_rates.ocl:15-32).  Work-item ids are therefore
 * thread-local variables that the driver sets before each call.
 */
#pragma once
#include <cmath>
#include <cstdlib>
#include <cstring>

#define __kernel
#define __global
#define __constant static
#define __OPENCL_C_VERSION__ 120

namespace clshim {
extern thread_local int lid;
extern thread_local int gid;
extern thread_local int ngroups;
}

static inline size_t get_local_id(int) { return (size_t)clshim::lid; }
static inline size_t get_group_id(int) { return (size_t)clshim::gid; }
static inline size_t get_num_groups(int) { return (size_t)clshim::ngroups; }
static inline size_t get_global_size(int) { return (size_t)clshim::ngroups * 128; }

using std::exp;
using std::log;
using std::log10;
using std::pow;
using std::fmin;
using std::fmax;
using std::fabs;
