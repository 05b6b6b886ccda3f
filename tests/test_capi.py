"""C ABI checks that need no GPU: the library builds, loads, exports every
function include/*.h declares (the boundary, pyjac_gb300.h, and the
instrumentation hooks, pyjac_gb300_internal.h), and rejects bad arguments
with an error status (never an abort) before touching the device."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, load_mech, pkg


def declared_functions(headers=("pyjac_gb300.h", "pyjac_gb300_internal.h")):
    text = ""
    for h in headers:
        with open(os.path.join(ROOT, "include", h)) as fh:
            text += fh.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\bint\s+(pjg_\w+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    pkg("build").build()
    return pkg("_lib").load()


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    bound = {s[0] for s in pkg("_lib").SIGNATURES}
    assert set(names) <= bound


def test_instrumentation_hooks_are_not_in_the_boundary_header():
    """Bench and test hooks live in the internal header only."""
    public = set(declared_functions(("pyjac_gb300.h",)))
    internal = set(declared_functions(("pyjac_gb300_internal.h",)))
    assert internal == {"pjg_launch_count", "pjg_fp64_peak", "pjg_profile_begin",
                        "pjg_profile_end", "pjg_math_exp", "pjg_eval_chunk", "pjg_reaction_order"}
    assert not public & internal


def test_bad_arguments_return_status(lib):
    L = pkg("_lib")
    assert lib.pjg_mech_create(None, None) == -1
    assert "null" in L.last_error()
    t = L.PjgTables()
    t.ns = 1
    h = ctypes.c_void_p()
    assert lib.pjg_mech_create(ctypes.byref(t), ctypes.byref(h)) == -3
    assert lib.pjg_species_rates(None, 10, b"C", 1, None, None, None, None) == -1
    assert lib.pjg_jacobian(None, 10, b"C", 1, 0, None, None, None, None) == -1
    assert lib.pjg_kernel_call(None, None, None, None) == -1
    assert lib.pjg_jacobian_indices(None, b"C", None, None, None) == -1
    buf = ctypes.create_string_buffer(4)
    assert lib.pjg_last_error(buf, 4) == 0 and len(buf.value) <= 3


def test_packed_tables_layout():
    pack = pkg("pack")
    mech = load_mech("gri30")
    pt = pack.PackedTables(mech)
    assert pt.rxn.dtype.itemsize == 192 and len(pt.rxn) == 325
    assert pt.species.shape == (53, 48)
    flags = pt.rxn["flags"]
    assert ((flags & 7) <= 2).all()                      # no PLOG / Chebyshev in GRI
    assert int(((flags >> 4) & 3 != 0).sum()) == 41      # third-body + fall-off reactions
    assert int(((flags >> 6) & 3 == 2).sum()) == 26      # Troe
    assert int((flags & pack.RX_REV != 0).sum()) == 309  # reversible
    assert pt.nnz == 1984
    mt = pkg("mech")
    tm = load_mech("testmech")
    ft = pack.PackedTables(tm).rxn["flags"]
    assert (ft & 7 == 3).sum() == tm.val["plog"]["num"]
    assert (ft & 7 == 4).sum() == tm.val["cheb"]["num"]
    assert mt is not None


def test_product_path_has_no_cpu_fallback(monkeypatch, tmp_path):
    """Without the CUDA library the API raises instead of computing on the CPU."""
    L = pkg("_lib")
    monkeypatch.setattr(L, "_lib", None)
    monkeypatch.setattr(L, "library_path", lambda: str(tmp_path / "missing.so"))
    with pytest.raises(RuntimeError):
        pkg("api").Evaluator(load_mech("h2o2"))


def test_header_is_plain_c(tmp_path):
    """include/pyjac_gb300.h (and the internal header) is usable from C (C99, pedantic, warnings as
    errors) and from C++: the boundary has no C++-only syntax."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    src = tmp_path / "use.c"
    src.write_text('#include "pyjac_gb300.h"\n#include "pyjac_gb300_internal.h"\n'
                   'int main(void) { pjg_mech* m = 0; int32_t ns = 0; int64_t c = 0;\n'
                   '  return pjg_mech_info(m, &ns, 0, 0) == PJG_OK && pjg_launch_count(&c) == 0; }\n')
    inc = os.path.join(ROOT, "include")
    for cmd in (["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror"],
                ["g++", "-std=c++11", "-Wall", "-Wextra", "-Werror", "-x", "c++"]):
        if shutil.which(cmd[0]) is None:
            continue
        r = subprocess.run(cmd + ["-I", inc, "-c", str(src), "-o", str(tmp_path / "use.o")],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_c_caller_links_and_runs(lib, tmp_path):
    """A plain C program links against the library and calls host-side entry
    points (the Markowitz analysis of an arrow pattern, which orders the
    dense node late and fills nothing; an initial-condition file round
    trip): the C ABI works without Python."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no gcc")
    data = tmp_path / "data.bin"
    src = tmp_path / "main.c"
    src.write_text(r'''
#include <stdio.h>
#include "pyjac_gb300.h"
int main(void) {
    int32_t row_ptr[5] = {0, 4, 6, 8, 10};
    int32_t col_ind[10] = {0, 1, 2, 3, 0, 1, 0, 2, 0, 3};
    int32_t perm[4], nnz = 0; int64_t fma = 0;
    int rc = pjg_lu_symbolic(4, row_ptr, col_ind, perm, &nnz, &fma);
    printf("%d %d %d %d %d %d %lld\n", rc, perm[0], perm[1], perm[2], perm[3], nnz, (long long)fma);
    double param[2] = {101325.0, 2e5}, phi[6] = {1000, 1, 0.1, 1500, 2, 0.2}, p2[2], phi2[6];
    rc = pjg_write_initial_conditions("%s", 2, 3, 'C', param, phi);
    rc |= pjg_read_initial_conditions("%s", 2, 3, 'C', p2, phi2);
    printf("%d %g %g %g\n", rc, p2[1], phi2[3], phi2[5]);
    return 0;
}
'''.replace('"%s"', '"' + str(data) + '"'))
    build_dir = os.path.dirname(pkg("_lib").library_path())
    exe = tmp_path / "a.out"
    r = subprocess.run(["gcc", "-std=c99", "-I", os.path.join(ROOT, "include"), str(src), "-L",
                        build_dir, "-lpyjac_gb300", "-Wl,-rpath," + build_dir, "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.split("\n")
    assert lines[0].split() == ["0", "1", "2", "0", "3", "10", "3"]
    assert lines[1].split() == ["0", "200000", "1500", "0.2"]
