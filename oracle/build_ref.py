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

The reference tree is taken from --reference, else from the PYJAC_REFERENCE
environment variable, else from this recipe's default location
(``DEFAULT_REFERENCE``, where the reference is mounted in the build
container).
"""
import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
MECHS = ("h2o2", "ch4")
DEFAULT_REFERENCE = "/root/reference"


def reference_dir(reference=None):
    """The reference tree this recipe reads: the argument, else
    $PYJAC_REFERENCE, else DEFAULT_REFERENCE."""
    return reference or os.environ.get("PYJAC_REFERENCE") or DEFAULT_REFERENCE


def _sizes(exdir):
    with open(os.path.join(exdir, "jacobian_main.ocl")) as f:
        main = f.read()
    rwk = int(re.search(r"work_size\s*\*\s*(\d+)\s*\*\s*sizeof\(double\)", main).group(1))
    with open(os.path.join(exdir, "jacobian_driver.ocl")) as f:
        drv = f.read()
    off = int(re.search(r"jac_local\s*=\s*\(rwk\s*\+\s*(\d+)\s*\*\s*work_size\)", drv).group(1))
    assert (rwk - off) % 128 == 0
    return rwk, (rwk - off) // 128


_QUOTED = re.compile(r'^\s*#\s*include\s*"([^"]+)"', re.M)


def _bundle(path, dirs, seen=None):
    """Text of `path` with every quoted #include inlined from `dirs` (each file
    once, as its include guard would have it); system (<...>) includes stay as
    they are, so that the result compiles against the headers of whichever
    host builds it."""
    seen = set() if seen is None else seen
    seen.add(os.path.realpath(path))
    with open(path) as f:
        text = f.read()

    def sub(m):
        for d in [os.path.dirname(path)] + dirs:
            q = os.path.join(d, m.group(1))
            if os.path.exists(q):
                if os.path.realpath(q) in seen:
                    return ""
                return _bundle(q, dirs, seen)
        raise FileNotFoundError(m.group(1))
    return _QUOTED.sub(sub, text)


def _compile_tu(tu, so, quiet):
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-w", "-x", "c++", tu,
           "-o", so]
    if not quiet:
        print(" ".join(cmd))
    subprocess.check_call(cmd)


def build_from_preprocessed(quiet=True):
    """Where the reference tree is absent (the aarch64 GPU host), compile the
    preprocessed translation units this recipe left in oracle/_ref/."""
    built = {}
    for mech in MECHS:
        tu = os.path.join(OUT, "ref_%s.ii" % mech)
        so = os.path.join(OUT, "libref_%s.so" % mech)
        if not os.path.exists(tu):
            continue
        if not (os.path.exists(so) and os.path.getmtime(so) >= os.path.getmtime(tu)):
            try:
                _compile_tu(tu, so, quiet)
            except (OSError, subprocess.CalledProcessError):
                continue
        built[mech] = so
    return built


def build(reference=None, quiet=False):
    """Compile every shipped example; return {mech: path_to_so}.

    Also writes oracle/_ref/ref_<mech>.ii, the shim with the example's
    generated code inlined (a build intermediate, not committed),
    so that hosts without the reference tree can build the same library with
    build_from_preprocessed()."""
    reference = reference_dir(reference)
    if not os.path.isdir(os.path.join(reference, "examples", "opencl")):
        return build_from_preprocessed(quiet)
    os.makedirs(OUT, exist_ok=True)
    built = {}
    for mech in MECHS:
        exdir = os.path.join(reference, "examples", "opencl", mech)
        if not os.path.isdir(exdir):
            continue
        tu = os.path.join(OUT, "ref_%s.ii" % mech)
        rwk, jac = _sizes(exdir)
        with open(tu, "w") as f:
            f.write("#define REF_RWK %d\n#define REF_JAC_SIZE %d\n" % (rwk, jac))
            f.write(_bundle(os.path.join(HERE, "ref_shim", "ref_driver.cpp"),
                            [os.path.join(HERE, "ref_shim"), exdir]))
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
    ap.add_argument("--reference", default=None)
    a = ap.parse_args()
    out = build(a.reference)
    print(out)
    sys.exit(0 if out else 1)
