"""Pin the CPU oracle (test infrastructure) before trusting it.

* against the reference's own shipped generated kernels: the golden outputs in
  tests/golden/ref_<mech>.npz (H2/O2 dense F, GRI-30 sparse CCS F, conp),
  produced by tests/golden/make_golden.py from the shim-compiled
  examples/opencl/{h2o2,ch4};
* against central finite differences of its own species rates for every
  reaction form (PLOG, Chebyshev, SRI, Troe, Lindemann, third bodies, single
  species third bodies, chemically activated) in conp and conv: those forms
  have no runnable reference artefact here ("parity unpinned" by reference
  values, pinned by the formulas and this consistency check);
* guard behaviour at out-of-range states.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, bath_rich_states, load_mech, oracle_mod, row_rel_err


def _dense_from_shipped(jac_F, mech, name):
    n = jac_F.shape[1]
    NN = mech.nn
    if jac_F.shape[0] == NN * NN:
        return jac_F.T.reshape(n, NN, NN).transpose(0, 2, 1)
    ptr, ind = mech.pattern("F")
    J = np.zeros((n, NN, NN))
    for c in range(NN):
        for p in range(ptr[c], ptr[c + 1]):
            J[:, ind[p], c] = jac_F[p]
    return J


@pytest.mark.parametrize("name", ["h2o2", "gri30"])
def test_oracle_matches_shipped_reference_kernels(name):
    g = np.load(os.path.join(GOLDEN, "ref_%s.npz" % name))
    mech = load_mech(name)
    o = oracle_mod().Oracle(mech)
    d = o.species_rates(g["P"], g["phi"])
    ref = g["dphi_F"].T
    assert np.array_equal(d, ref) or np.max(np.abs(d - ref) / np.maximum(np.abs(ref), 1e-300)) < 1e-13
    J = o.jacobian(g["P"], g["phi"])
    Jr = _dense_from_shipped(g["jac_F"], mech, name)
    assert row_rel_err(J, Jr) < 1e-12
    big = np.abs(Jr) > 1e-6 * np.abs(Jr).max(axis=2, keepdims=True)
    assert (np.abs(J - Jr)[big] / np.abs(Jr)[big]).max() < 1e-9


def fd_jacobian(o, P, phi, conp, rel=1e-5):
    """4th-order central differences of the oracle's species rates."""
    n, NN = phi.shape
    Jfd = np.zeros((n, NN, NN))
    ntot = phi[:, 2:].sum(axis=1)
    for c in range(NN):
        h = rel * (np.maximum(np.abs(phi[:, c]), 1e-2 * ntot) if c >= 2 else np.abs(phi[:, c]))
        f = []
        for k in (2, 1, -1, -2):
            pp = phi.copy()
            pp[:, c] += k * h
            f.append(o.species_rates(P, pp, conp=conp))
        Jfd[:, :, c] = (-f[0] + 8 * f[1] - 8 * f[2] + f[3]) / (12 * h)[:, None]
    return Jfd


@pytest.mark.parametrize("name", ["h2o2", "gri30", "testmech", "synthetic_small"])
@pytest.mark.parametrize("conp", [True, False])
def test_oracle_jacobian_matches_finite_differences(name, conp):
    mech = load_mech(name)
    o = oracle_mod().Oracle(mech)
    P, phi = bath_rich_states(mech, 6, 3, conp)
    J = o.jacobian(P, phi, conp=conp)
    assert row_rel_err(J, fd_jacobian(o, P, phi, conp)) < 2e-8


def test_oracle_guards_out_of_range_states():
    mech = load_mech("gri30")
    o = oracle_mod().Oracle(mech)
    P, phi = bath_rich_states(mech, 4, 9, True)
    phi[0, 0] = 50.0        # below the 100 K clamp
    phi[1, 0] = 2.0e4       # above the 10000 K clamp
    phi[2, 2:10] = 0.0      # zero moles (guarded at 1e-300)
    phi[3, 1] = 0.0         # zero volume (guarded at 1e-30)
    d = o.species_rates(P, phi)
    assert np.isfinite(d[:3]).all()
    J = o.jacobian(P, phi[:3])
    assert np.isfinite(J).all()


@pytest.mark.parametrize("name", ["h2o2", "gri30"])
def test_oracle_chem_utils_matches_shipped_reference(name):
    """Species thermo (the chem_utils kernel type: cp, h, b at the guarded T)
    against the shipped chem_utils kernel over a 50 K - 12,000 K sweep."""
    g = np.load(os.path.join(GOLDEN, "ref_%s.npz" % name))
    o = oracle_mod().Oracle(load_mech(name))
    for got, ref in zip(o.chem_utils(g["cu_phi"]), (g["cu_cp_F"], g["cu_h_F"], g["cu_b_F"])):
        ref = ref.T
        assert np.max(np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)) < 1e-13


@pytest.mark.parametrize("name", ["h2o2", "gri30", "testmech", "synthetic_small"])
def test_oracle_approximate_jacobian_drops_only_bath_gas_terms(name):
    """The 'approximate' type omits d n_Ns / d n_j in the reaction-rate
    derivatives (create_jacobian.py:3578-3582, :4187-4191): in every species
    row the exact and approximate Jacobians differ by the same amount in all
    species columns, and not at all in the T and E columns."""
    exact, approx = load_mech(name), load_mech(name, jac_type="approximate")
    P, phi = bath_rich_states(exact, 32, 5)
    Je = oracle_mod().Oracle(exact).jacobian(P, phi)
    Ja = oracle_mod().Oracle(approx).jacobian(P, phi)
    d = Je[:, 2:, :] - Ja[:, 2:, :]
    scale = np.abs(Je[:, 2:, :]).max(axis=2, keepdims=True) + 1e-300
    assert (np.abs(d[:, :, :2]) / scale).max() < 1e-13
    spread = d[:, :, 2:].max(axis=2) - d[:, :, 2:].min(axis=2)
    assert (spread / scale[:, :, 0]).max() < 1e-11
    # the approximate pattern holds every non-zero of the approximate Jacobian
    ptr, ind = approx.pattern("C")
    mask = np.zeros((approx.nn, approx.nn), dtype=bool)
    for r in range(approx.nn):
        mask[r, ind[ptr[r]:ptr[r + 1]]] = True
    assert (Ja[:, ~mask] == 0).all()
    if name in ("h2o2", "gri30"):  # mechanisms with bath-gas reactions
        assert np.abs(d[:, :, 2:]).max() > 0


def test_op_counter_is_pinned_and_stored():
    """The FP64 operation counter (oracle/flop_count.cpp, the oracle's source
    compiled with a counting double) reproduces the committed per-state
    counts of data/fp64_op_counts.json, which bench.py uses for the FP64
    roofline; a rebuilt count of H2/O2 and GRI-Mech 3.0 equals them."""
    import importlib
    import json
    import sys
    from conftest import ROOT
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    cf = importlib.import_module("count_flops")
    with open(os.path.join(ROOT, "data", "fp64_op_counts.json")) as fh:
        stored = json.load(fh)["mechanisms"]
    for name in ("h2o2", "gri30"):
        fresh = cf.count(name)
        for kind in ("rates", "jacobian", "vjp"):
            assert fresh[kind] == stored[name][kind], (name, kind)
    g = stored["gri30"]
    # the Jacobian carries the rates' work plus its derivative blocks
    assert g["jacobian"]["flops"] > 5 * g["rates"]["flops"]
    assert g["rates"]["exp"] >= 325  # at least one exponential per reaction


def test_op_counter_leaves_the_arithmetic_unchanged():
    """The counting build evaluates the same IEEE operations as the plain
    oracle: the counts are of the arithmetic the oracle's results come from."""
    import ctypes
    mech = load_mech("h2o2")
    orc = oracle_mod()
    o = orc.Oracle(mech)
    states = __import__("conftest").pkg("states")
    P, phi = states.draw_states(mech.n_species, 16, seed=5, x_floor=1e-12)
    ref = o.jacobian(P, phi)
    o.op_counts(P, phi, "jacobian")  # loads the counting library
    lib = o._count_lib
    # the counting library exports the plain entry points of the same source
    fn = lib.orc_jacobian
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.POINTER(orc._OrcMech), ctypes.c_long, ctypes.c_int] + [orc._D] * 3 + [ctypes.c_int]
    out = np.empty_like(ref)
    P = np.ascontiguousarray(P)
    phi = np.ascontiguousarray(phi)
    assert fn(ctypes.byref(o._m), 16, 1, P.ctypes.data_as(orc._D), phi.ctypes.data_as(orc._D),
              out.ctypes.data_as(orc._D), 1) == 0
    assert np.array_equal(out, ref)


def test_oracle_matches_reference_kernel_text_forms():
    """The forms no shipped kernel runs (PLOG, Chebyshev, SRI and Troe
    blending, dT/dt and the extra-variable rate at constant pressure and
    constant volume) against the reference's own generated kernel text,
    executed on the same states (tests/golden/ref_forms_testmech.npz, made by
    tests/golden/make_ref_forms.py): the oracle's intermediates agree to
    1e-13, with the kernels' inputs equal to the stored ones."""
    g = np.load(os.path.join(GOLDEN, "ref_forms_testmech.npz"))
    mech = load_mech("testmech")
    o = oracle_mod().Oracle(mech)

    def rel(a, b):
        return float((np.abs(a - b) / np.maximum(np.abs(b), 1e-300)).max())

    for tag, conp in (("conp", True), ("conv", False)):
        P, phi = g[tag + "/P"], g[tag + "/phi"]
        # the fixture reaches the guards and the tables' ends
        assert phi[:, 0].min() < 100.0 and phi[:, 0].max() > 10000.0
        d = o.rates_detail(P, phi, conp=conp)
        assert np.array_equal(d["Pr"], g[tag + "/in_Pr"])
        assert np.array_equal(d["wdot"], g[tag + "/in_wdot"])
        assert rel(d["kf"][:, g["plog_map"]], g[tag + "/ref_plog"]) <= 1e-13
        assert rel(d["kf"][:, g["cheb_map"]], g[tag + "/ref_cheb"]) <= 1e-13
        for form in ("sri", "troe"):
            m = g[form + "_map"]
            assert m.size and rel(d["Fi"][:, m], g[tag + "/ref_" + form][:, m]) <= 1e-13, form
        assert rel(d["dphi"][:, 0], g[tag + "/ref_temperature"][:, 0]) <= 1e-13
        assert rel(d["dphi"][:, 1], g[tag + "/ref_extra_var"][:, 1]) <= 1e-13
    texts = "\n".join(str(t) for t in g["conv/texts"])
    assert "pow(" in texts and "cheb_params" in texts and "plog_params" in texts


@pytest.mark.skipif(not os.environ.get("PYJAC_REFERENCE"), reason="PYJAC_REFERENCE not set")
def test_reference_form_fixture_regenerates():
    """With the reference tree at hand, its generators' text executed again
    gives the stored golden values bit for bit."""
    import importlib
    import sys
    from conftest import ROOT
    for p in (os.path.join(ROOT, "tests", "golden"), os.path.join(ROOT, "oracle")):
        sys.path.insert(0, p)
    mk = importlib.import_module("make_ref_forms")
    rf = importlib.import_module("ref_frontend")
    g = np.load(os.path.join(GOLDEN, "ref_forms_testmech.npz"))
    mech = load_mech("testmech")
    o = oracle_mod().Oracle(mech)
    for tag, conp in (("conp", True), ("conv", False)):
        knls, info, _ = rf.reference_rate_kernels(mk.MECH, conp=conp)
        res = mk.run_forms(knls, info, mech, o, conp)
        for k, v in res.items():
            assert np.array_equal(v, g[tag + "/" + k]), (tag, k)
