"""GPU against the reference's own outputs, directly (not through the oracle).

* tests/golden/ref_<mech>.npz: outputs of the reference's shipped generated
  kernels (examples/opencl/{h2o2,ch4}), shim-compiled and run by
  tests/golden/make_golden.py: H2/O2 dense F Jacobian (256 states) and
  GRI-Mech 3.0 sparse CCS F Jacobian (1,024 states), F order, conp.  The GPU
  evaluates the same states in the same layout; the spec bars are
  asserted in two forms: relative to each row's largest entry, and element
  by element on every entry of at least 1e-6 of its row's largest.
* tests/golden/ref_forms_testmech.npz: states of the reference's all-forms
  test mechanism (PLOG, Chebyshev, SRI, Troe, Lindemann) at constant
  pressure and constant volume, temperatures beyond the 100 K / 10,000 K
  guards and pressures outside the PLOG and Chebyshev tables; the GPU's rates
  and Jacobians there against the oracle, whose forms on those states are
  pinned to the reference's own kernel text (tests/test_oracle.py).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_mech, oracle_mod, pkg

pytestmark = pytest.mark.gpu


def _dense_ref(jac_F, mech):
    """The reference's F-order output (dense or sparse CCS) as dense (n, NN, NN)
    plus the mask of its stored entries."""
    n, NN = jac_F.shape[1], mech.nn
    if jac_F.shape[0] == NN * NN:
        return jac_F.T.reshape(n, NN, NN).transpose(0, 2, 1), np.ones((NN, NN), dtype=bool)
    ptr, ind = mech.pattern("F")
    J = np.zeros((n, NN, NN))
    mask = np.zeros((NN, NN), dtype=bool)
    for c in range(NN):
        for p in range(ptr[c], ptr[c + 1]):
            J[:, ind[p], c] = jac_F[p]
            mask[ind[p], c] = True
    return J, mask


@pytest.mark.parametrize("name", ["h2o2", "gri30"])
def test_gpu_matches_shipped_reference_outputs(cuda_device, name):
    import torch
    g = np.load(os.path.join(GOLDEN, "ref_%s.npz" % name))
    mech = load_mech(name)
    ev = pkg("api").Evaluator(mech)
    P, phi = g["P"], g["phi"]
    n, NN = P.shape[0], mech.nn
    sparse = g["jac_F"].shape[0] != NN * NN
    tP = torch.from_numpy(P).to(cuda_device)
    tphi = torch.from_numpy(np.ascontiguousarray(phi.T)).to(cuda_device)
    # the shipped layout itself: F order, sparse CCS for GRI-Mech 3.0
    jac = ev.jacobian(tP, tphi, order="F", jac_format="sparse" if sparse else "full").cpu().numpy()
    dphi = ev.species_rates(tP, tphi, order="F").cpu().numpy()
    jr = g["jac_F"]
    # both layouts index entry (row, col) of state s at (col * NN + row, s)
    got = jac.reshape(jr.shape) if sparse else jac.reshape(NN * NN, n)
    Jg, _ = _dense_ref(got, mech)
    Jr, mask = _dense_ref(jr, mech)
    rowmax = np.abs(Jr).max(axis=2, keepdims=True)
    rowmax[rowmax == 0] = 1.0
    err = np.abs(Jg - Jr) * mask
    assert float((err / rowmax).max()) <= 1e-8
    well = (np.abs(Jr) >= 1e-6 * rowmax) & mask
    rel = err[well] / np.abs(Jr[well])
    assert well.sum() > 0.3 * n * mask.sum()
    assert float(rel.max()) <= 1e-8, float(rel.max())
    # rates, in two forms.  scale: the same sums in absolute values (the
    # cancellation scale); an entry k times smaller than its scale carries
    # about k * (number of terms) ulps of rounding in any FP64 evaluation, so
    # a plain relative bar is asserted where k <= 1e3 and every entry is
    # measured against |value| + scale
    scale = oracle_mod().Oracle(mech).rates_scale(P, phi).T
    dr = g["dphi_F"]
    diff = np.abs(dphi - dr)
    rs = diff / np.maximum(np.abs(dr) + scale, 1e-300)
    assert float(rs.max()) <= 1e-10, float(rs.max())
    wellr = (np.abs(dr) >= 1e-3 * scale) & (dr != 0)
    assert wellr.mean() > 0.5
    rw = diff[wellr] / np.abs(dr[wellr])
    assert float(rw.max()) <= 1e-10, float(rw.max())


@pytest.mark.parametrize("conp", [True, False])
def test_gpu_on_reference_form_states(cuda_device, conp):
    """PLOG, Chebyshev, SRI and Troe reactions at guard temperatures and
    out-of-table pressures, both state formulations, both orders."""
    import torch
    g = np.load(os.path.join(GOLDEN, "ref_forms_testmech.npz"))
    tag = "conp" if conp else "conv"
    P, phi = g[tag + "/P"], g[tag + "/phi"]
    mech = load_mech("testmech")
    o = oracle_mod().Oracle(mech)
    ref = o.species_rates(P, phi, conp=conp)
    scale = o.rates_scale(P, phi, conp=conp)
    Jref = o.jacobian(P, phi, conp=conp)
    ev = pkg("api").Evaluator(mech)
    tP = torch.from_numpy(P).to(cuda_device)
    for order in ("C", "F"):
        x = phi if order == "C" else np.ascontiguousarray(phi.T)
        tphi = torch.from_numpy(np.ascontiguousarray(x)).to(cuda_device)
        d = ev.species_rates(tP, tphi, order=order, conp=conp).cpu().numpy()
        J = ev.jacobian(tP, tphi, order=order, conp=conp).cpu().numpy()
        if order == "F":
            d = d.T
            J = J.transpose(2, 1, 0)
        rr = np.abs(d - ref) / np.maximum(np.abs(ref) + scale, 1e-300)
        assert float(rr.max()) <= 1e-10, (order, float(rr.max()))
        rowmax = np.abs(Jref).max(axis=2, keepdims=True)
        rowmax[rowmax == 0] = 1.0
        assert float((np.abs(J - Jref) / rowmax).max()) <= 1e-8, order
