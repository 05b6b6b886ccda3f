"""Build recipe: compile the reference's shipped generated kernels for the host.

Test infrastructure only.  For each mechanism shipped under the reference's
``examples/opencl/<mech>/`` (H2/O2 and GRI-Mech 3.0, generated with
``--lang opencl --width 128 --data_order F``), this compiles
``oracle/ref_shim/ref_driver.cpp`` with the example directory on the include
path, producing ``oracle/_ref/libref_<mech>.so``.  The reference sources are
read where they lie and are never copied; outputs go only to ``oracle/_ref/``.

Sizes the driver needs are read from the generated host code:
* ``REF_RWK``: doubles of working buffer per work group, from
  ``jacobian_main.ocl`` (``work_size*<RWK> * sizeof(double)``);
* ``REF_JAC_SIZE``: Jacobian entries per state, from the offset of
  ``jac_local`` in ``jacobian_driver.ocl`` (``(RWK - offset) / 128``).

Flags follow the reference's libgen C flags (pyjac/libgen/libgen.py:24-49:
``-O3 -fopenmp``), without ``-march=native`` so that the build is portable.

Usage: python oracle/build_ref.py [--reference DIR]
"""
import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
MECHS = ("h2o2", "ch4")


def _sizes(exdir):
    with open(os.path.join(exdir, "jacobian_main.ocl")) as f:
        main = f.read()
    rwk = int(re.search(r"work_size\s*\*\s*(\d+)\s*\*\s*sizeof\(double\)", main).group(1))
    with open(os.path.join(exdir, "jacobian_driver.ocl")) as f:
        drv = f.read()
    off = int(re.search(r"jac_local\s*=\s*\(rwk\s*\+\s*(\d+)\s*\*\s*work_size\)", drv).group(1))
    assert (rwk - off) % 128 == 0
    return rwk, (rwk - off) // 128


def build(reference="/root/reference", quiet=False):
    """Compile every shipped example; return {mech: path_to_so}."""
    os.makedirs(OUT, exist_ok=True)
    built = {}
    for mech in MECHS:
        exdir = os.path.join(reference, "examples", "opencl", mech)
        if not os.path.isdir(exdir):
            continue
        so = os.path.join(OUT, "libref_%s.so" % mech)
        src = os.path.join(HERE, "ref_shim", "ref_driver.cpp")
        deps = [src, os.path.join(HERE, "ref_shim", "cl_shim.h")] + [
            os.path.join(exdir, f) for f in ("species_rates.ocl", "jacobian.ocl", "chem_utils.ocl")]
        if os.path.exists(so) and all(os.path.getmtime(so) >= os.path.getmtime(d) for d in deps):
            built[mech] = so
            continue
        rwk, jac = _sizes(exdir)
        cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared",
               "-Wno-attributes", "-Wno-unknown-pragmas", "-w",
               "-I", os.path.join(HERE, "ref_shim"), "-I", exdir,
               "-DREF_RWK=%d" % rwk, "-DREF_JAC_SIZE=%d" % jac,
               src, "-o", so]
        if not quiet:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
        built[mech] = so
    return built


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    a = ap.parse_args()
    out = build(a.reference)
    print(out)
    sys.exit(0 if out else 1)
