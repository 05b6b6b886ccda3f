"""J^T v kernel and the torch autograd path (GPU).

* against the oracle's dense analytical Jacobian: |vjp - J^T v| <= 1e-9 * s,
  s = sum_r |J_rc v_r| (the product's cancellation scale), every mechanism,
  conp/conv, C/F order;
* the autograd backward against central finite differences of the forward
  (relative step 1e-6) along random directions: <v, J u>.
"""
import numpy as np
import pytest

from conftest import bath_rich_states, load_mech, oracle_mod, pkg

pytestmark = pytest.mark.gpu

MECHS = ["h2o2", "gri30", "testmech", "synthetic_small"]
_ev = {}


def evaluator(name):
    if name not in _ev:
        _ev[name] = pkg("api").Evaluator(load_mech(name))
    return _ev[name]


def dev(a, device):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


@pytest.mark.parametrize("name", MECHS)
@pytest.mark.parametrize("conp", [True, False])
@pytest.mark.parametrize("order", ["C", "F"])
def test_vjp_matches_dense_jacobian(cuda_device, name, conp, order):
    mech = load_mech(name)
    n = 150
    P, phi = bath_rich_states(mech, n, 21, conp)
    rng = np.random.default_rng(5)
    v = rng.standard_normal(phi.shape)
    J = oracle_mod().Oracle(mech).jacobian(P, phi, conp=conp)
    ref = np.einsum("nrc,nr->nc", J, v)
    scale = np.einsum("nrc,nr->nc", np.abs(J), np.abs(v))
    ev = evaluator(name)
    x, vv = (phi, v) if order == "C" else (phi.T, v.T)
    out = ev.vjp(dev(P, cuda_device), dev(x, cuda_device), dev(vv, cuda_device), order=order,
                 conp=conp).cpu().numpy()
    if order == "F":
        out = out.T
    assert np.isfinite(out).all()
    err = np.abs(out - ref) / np.where(scale > 0, scale, 1.0)
    assert err.max() < 1e-9


def test_wdot_autograd_backward_vs_finite_differences(cuda_device):
    import torch
    mech = load_mech("gri30")
    ev = evaluator("gri30")
    ops = pkg("torch_ops")
    n = 256
    P, phi = bath_rich_states(mech, n, 31, True)
    tP = dev(P, cuda_device)
    x = dev(phi, cuda_device).requires_grad_(True)
    out = ops.wdot(ev, tP, x)
    rng = np.random.default_rng(7)
    v = dev(rng.standard_normal(phi.shape), cuda_device)
    (g,) = torch.autograd.grad(out, x, grad_outputs=v)
    # directional derivative <v, J u> with u scaled per component
    u = rng.standard_normal(phi.shape) * np.abs(phi)
    u[:, 2:] += 1e-3 * phi[:, 2:].sum(axis=1, keepdims=True) * rng.standard_normal(phi[:, 2:].shape)
    h = 1e-6
    with torch.no_grad():
        fp = ev.species_rates(tP, dev(phi + h * u, cuda_device))
        fm = ev.species_rates(tP, dev(phi - h * u, cuda_device))
        fd = ((fp - fm) / (2 * h) * v).sum(dim=1).cpu().numpy()
    ad = (g.cpu().numpy() * u).sum(axis=1)
    scale = np.abs(g.cpu().numpy() * u).sum(axis=1)
    assert (np.abs(ad - fd) / scale).max() < 1e-6


def test_wdot_backward_equals_dense_jacobian_transpose(cuda_device):
    import torch
    mech = load_mech("gri30")
    ev = evaluator("gri30")
    ops = pkg("torch_ops")
    P, phi = pkg("states").draw_states(mech.n_species, 64, seed=3, x_floor=1e-12)
    tP = dev(P, cuda_device)
    x = dev(phi, cuda_device).requires_grad_(True)
    out = ops.wdot(ev, tP, x)
    v = torch.randn_like(out)
    (g,) = torch.autograd.grad(out, x, grad_outputs=v)
    J = ev.jacobian(tP, x.detach())
    ref = torch.einsum("nrc,nr->nc", J, v)
    scale = torch.einsum("nrc,nr->nc", J.abs(), v.abs())
    assert float(((g - ref).abs() / scale.clamp_min(1e-300)).max()) < 1e-9
