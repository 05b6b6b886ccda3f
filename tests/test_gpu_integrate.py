"""GPU Newton-matrix LU, solves and ROS2 steps against the oracle.

The factorisation and the solves perform the oracle's IEEE operations in the
same order (fma entries, first-largest pivot, reciprocal scaling, rank-1 FMA
updates; row-oriented FMA substitution), so their results must be identical
bit for bit.  A ROS2 step also involves the rates and the Jacobian, which
agree with the oracle to 1e-10 / 1e-8; the step is compared at 1e-9 of each
component's scale.
"""
import numpy as np
import pytest

from conftest import load_mech, oracle_mod, pkg

pytestmark = pytest.mark.gpu


def _to_dev_mat(J, order, device):
    import torch
    a = J if order == "C" else J.transpose(2, 1, 0)  # F: [col, row, state]
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def _from_dev_mat(t, order):
    a = t.cpu().numpy()
    return a if order == "C" else a.transpose(2, 1, 0)


def _to_dev_vec(x, order, device):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x if order == "C" else x.T)).to(device)


def _from_dev_vec(t, order):
    a = t.cpu().numpy()
    return a if order == "C" else a.T


def _newton_inputs(name, n, seed):
    mech = load_mech(name)
    P, phi = pkg("states").draw_states(mech.n_species, n, seed=seed, x_floor=1e-12)
    return mech, P, phi, oracle_mod().Oracle(mech).jacobian(P, phi)


@pytest.mark.parametrize("order", ["C", "F"])
@pytest.mark.parametrize("name", ["h2o2", "gri30"])
@pytest.mark.parametrize("per_state_h", [False, True])
def test_lu_factor_bitwise(cuda_device, order, name, per_state_h):
    import torch
    orc = oracle_mod()
    integ = pkg("integrate")
    mech, P, phi, J = _newton_inputs(name, 1000, 41)
    rng = np.random.default_rng(3)
    h = 10.0 ** rng.uniform(-9, -2, J.shape[0]) if per_state_h else 3e-6
    lu_ref, piv_ref, info_ref = orc.lu_factor(J, integ.ROS2_GAMMA, h)
    hd = torch.from_numpy(h).to(cuda_device) if per_state_h else h
    lu, piv, info = integ.lu_factor(_to_dev_mat(J, order, cuda_device), hd, s=integ.ROS2_GAMMA,
                                    order=order)
    assert np.array_equal(_from_dev_mat(lu, order), lu_ref)
    assert np.array_equal(_from_dev_vec(piv, order), piv_ref)
    assert np.array_equal(info.cpu().numpy(), info_ref)


@pytest.mark.parametrize("order", ["C", "F"])
@pytest.mark.parametrize("nn", [1, 2, 5, 31, 32, 33, 64, 100, 169])
def test_lu_factor_random_matrices_bitwise(cuda_device, order, nn):
    """General matrices (heavy pivoting) at sizes around the warp width and up
    to the 169 limit of one state per block of shared memory."""
    orc = oracle_mod()
    integ = pkg("integrate")
    rng = np.random.default_rng(nn)
    n = 97 if nn <= 64 else 9
    J = rng.standard_normal((n, nn, nn))
    lu_ref, piv_ref, info_ref = orc.lu_factor(J, 1.0, 1.0)
    lu, piv, info = integ.lu_factor(_to_dev_mat(J, order, cuda_device), 1.0, order=order)
    assert np.array_equal(_from_dev_mat(lu, order), lu_ref)
    assert np.array_equal(_from_dev_vec(piv, order), piv_ref)
    assert np.array_equal(info.cpu().numpy(), info_ref)


def test_lu_factor_in_place_and_zero_pivots(cuda_device):
    orc = oracle_mod()
    integ = pkg("integrate")
    rng = np.random.default_rng(8)
    M = rng.standard_normal((5, 12, 12))
    M[0, :, 4] = 0.0
    M[1, :, 0] = 0.0
    M[2, :, 11] = 0.0
    M[3] = 0.0
    J = np.eye(12)[None] - M
    lu_ref, piv_ref, info_ref = orc.lu_factor(J, 1.0, 1.0)
    assert list(info_ref) == [5, 1, 12, 1, 0]
    t = _to_dev_mat(J, "C", cuda_device)
    lu, piv, info = integ.lu_factor(t, 1.0, out=t)
    assert lu.data_ptr() == t.data_ptr()
    assert np.array_equal(lu.cpu().numpy(), lu_ref)
    assert np.array_equal(piv.cpu().numpy(), piv_ref)
    assert np.array_equal(info.cpu().numpy(), info_ref)


@pytest.mark.parametrize("order", ["C", "F"])
@pytest.mark.parametrize("name", ["h2o2", "gri30"])
def test_lu_solve_bitwise(cuda_device, order, name):
    orc = oracle_mod()
    integ = pkg("integrate")
    mech, P, phi, J = _newton_inputs(name, 777, 5)
    lu_ref, piv_ref, _ = orc.lu_factor(J, integ.ROS2_GAMMA, 1e-5)
    b = np.random.default_rng(6).standard_normal((777, mech.nn))
    x_ref = orc.lu_solve(lu_ref, piv_ref, b)
    lu = _to_dev_mat(lu_ref, order, cuda_device)
    piv = _to_dev_vec(piv_ref, order, cuda_device)
    x = integ.lu_solve(lu, piv, _to_dev_vec(b, order, cuda_device), order=order)
    assert np.array_equal(_from_dev_vec(x, order), x_ref)


def test_empty_and_unsupported_sizes(cuda_device):
    import torch
    integ = pkg("integrate")
    z = torch.zeros((0, 10, 10), dtype=torch.float64, device=cuda_device)
    lu, piv, info = integ.lu_factor(z, 1e-6)
    assert lu.numel() == 0 and piv.numel() == 0 and info.numel() == 0
    big = torch.zeros((1, 170, 170), dtype=torch.float64, device=cuda_device)
    with pytest.raises(RuntimeError, match="nn must be in"):
        integ.lu_factor(big, 1e-6)


@pytest.mark.parametrize("order", ["C", "F"])
@pytest.mark.parametrize("name", ["h2o2", "gri30"])
def test_ros2_step_matches_oracle(cuda_device, order, name):
    """Radical-rich random states with steps of 1e-10 to 1e-7 s.

    (1) Bit for bit: the step equals the oracle's LU, solves and stage
    arithmetic applied to this library's own rates and Jacobian (each pinned
    to the oracle by the parity tests).  (2) Against the step computed
    entirely by the oracle: the Newton matrices of these states are ill
    conditioned, and perturbing the oracle's Jacobian by 1e-13 and its rates
    by 1e-12 (relative, random) moves the H2/O2 step by 2e-7 of a component's
    scale, so the bound here is 1e-5."""
    import torch
    orc = oracle_mod()
    integ = pkg("integrate")
    mech = load_mech(name)
    n = 513
    P, phi = pkg("states").draw_states(mech.n_species, n, seed=12, x_floor=1e-12)
    h = 10.0 ** np.random.default_rng(1).uniform(-10, -7, n)
    ev = pkg("api").Evaluator(mech)
    Pd, hd = torch.from_numpy(P).to(cuda_device), torch.from_numpy(h).to(cuda_device)
    phid = _to_dev_vec(phi, order, cuda_device)

    def rates(y):
        return _from_dev_vec(ev.species_rates(Pd, _to_dev_vec(y, order, cuda_device), order=order),
                             order)

    J = _from_dev_mat(ev.jacobian(Pd, phid, order=order), order)
    lu, piv, info_ref = orc.lu_factor(J, integ.ROS2_GAMMA, h)
    k1 = orc.lu_solve(lu, piv, rates(phi))
    k2 = orc.lu_solve(lu, piv, orc.ros2_combine(1, h, rates(orc.ros2_combine(0, h, phi, k1)), k1))
    ref, err_ref = orc.ros2_combine(2, h, phi, k1, k2)

    st = integ.Ros2Stepper(ev, n, order=order)
    out, err, info = st.step(Pd, phid, hd)
    out, err = _from_dev_vec(out, order), _from_dev_vec(err, order)
    assert np.array_equal(info.cpu().numpy(), info_ref)
    assert np.array_equal(out, ref)
    assert np.array_equal(err, err_ref)
    assert np.array_equal(_from_dev_mat(st.lu, order), lu)

    full, _, _ = orc.ros2_step(orc.Oracle(mech), P, phi, h)
    scale = np.abs(phi) + np.abs(full - phi) + 1e-300
    assert (np.abs(out - full) / scale).max() < 1e-5


def test_ros2_trajectory_premix(cuda_device):
    """64 ROS2 steps of an H2/O2/Ar premix on the GPU follow the oracle's
    trajectory (the same method with the oracle's rates and Jacobian)."""
    import torch
    from test_integrate_oracle import premix_h2o2
    orc = oracle_mod()
    integ = pkg("integrate")
    mech, P, phi = premix_h2o2()
    o = orc.Oracle(mech)
    ev = pkg("api").Evaluator(mech)
    st = integ.Ros2Stepper(ev, 1)
    h = 2e-5 / 64
    y_ref = phi.copy()
    y = torch.from_numpy(phi).to(cuda_device)
    Pd = torch.from_numpy(P).to(cuda_device)
    for _ in range(64):
        y_ref, _, _ = orc.ros2_step(o, P, y_ref, h)
        y, _, _ = st.step(Pd, y, h, out=torch.empty_like(y))
    y = y.cpu().numpy()
    scale = np.abs(y_ref) + 1e-8 * np.abs(y_ref).max()
    assert (np.abs(y - y_ref) / scale).max() < 1e-8
