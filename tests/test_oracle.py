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
