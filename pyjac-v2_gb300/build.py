"""Build the CUDA library ``_build/libpyjac_gb300.so`` for sm_103a with nvcc.

Translation units are compiled in parallel and linked into one shared
library exporting the C ABI of include/pyjac_gb300.h.  The build is in-tree
(git-ignored) and rebuilt only when a source is newer than the library.
"""
import concurrent.futures
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libpyjac_gb300.so")
STAMP = os.path.join(BUILD, "flags.txt")  # extra nvcc flags the library was built with
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", CSRC, "-I", INCLUDE]


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    out = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h"))]
    out += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return out + [os.path.abspath(__file__)]


def up_to_date(extra=()):
    if not os.path.exists(LIB):
        return False
    try:
        with open(STAMP) as f:
            if f.read() != " ".join(extra):
                return False
    except OSError:
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force=False, verbose=False, nvcc="nvcc", extra_flags=None):
    """Compile every .cu under csrc/ and link libpyjac_gb300.so; return its path.

    ``extra_flags`` (or the PJG_NVCC_EXTRA environment variable) appends nvcc
    flags, e.g. ``-DPJG_JAC_MINB=2`` to change the Jacobian kernel's
    launch bounds.  The flags are recorded beside the library, so a build with
    different flags (or none) after a variant build rebuilds everything.
    """
    extra = list(extra_flags or []) + os.environ.get("PJG_NVCC_EXTRA", "").split()
    if not force and up_to_date(extra):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in srcs]

    def compile_one(pair):
        src, obj = pair
        cmd = [nvcc] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (src, r.stdout, r.stderr))
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        list(ex.map(compile_one, zip(srcs, objs)))
    tmp = LIB + ".tmp"
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
    if verbose:
        print(" ".join(cmd))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(" ".join(extra))
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
