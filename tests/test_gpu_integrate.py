"""GPU Newton-matrix LU (partial pivoting and static-pivot sparse), solves
and ROS2 steps against the oracle.

The factorisations and the solves perform the oracle's IEEE operations in the
same order (fma entries, first-largest pivot or the static Markowitz order,
reciprocal scaling, rank-1 FMA updates; row-oriented FMA substitution), so
their results must be identical bit for bit.  A ROS2 step also involves the
rates and the Jacobian: it is compared bit for bit with the oracle's
factorisation, solves and stage arithmetic applied to this library's own
rates and Jacobian, and within a conditioning-aware bound with the step
computed entirely by the oracle.
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
    big = torch.zeros((1, 4097, 4097), dtype=torch.float64, device=cuda_device)
    with pytest.raises(RuntimeError, match="nn must be in"):
        integ.lu_factor(big, 1e-6)


@pytest.mark.parametrize("order", ["C", "F"])
@pytest.mark.parametrize("nn", [170, 177, 257, 501])
def test_lu_factor_global_memory_sizes_bitwise(cuda_device, order, nn):
    """Matrices beyond shared memory (nn > 169): the blocked global-memory
    factorisation performs the oracle's operations in the same order, so the
    factors, pivots and solves are identical; 501 is the synthetic
    500-species mechanism's size.  Also in place, with a zero column, and
    with the vector solve beyond the local-array solve (nn > 176)."""
    import torch
    orc = oracle_mod()
    integ = pkg("integrate")
    rng = np.random.default_rng(nn)
    n = 6
    J = rng.standard_normal((n, nn, nn)) * 10.0 ** rng.uniform(-3, 3, (n, 1, nn))
    h = 10.0 ** rng.uniform(-1, 0, n)
    # state 1: an exactly zero column of M = I - h J (h = 1, J's column the
    # unit vector), so info reports the first zero pivot
    J[1, :, nn // 3] = 0.0
    J[1, nn // 3, nn // 3] = 1.0
    h[1] = 1.0
    lu_ref, piv_ref, info_ref = orc.lu_factor(J, 1.0, h)
    assert info_ref[1] != 0
    t = _to_dev_mat(J, order, cuda_device)
    hd = torch.from_numpy(h).to(cuda_device)
    lu, piv, info = integ.lu_factor(t, hd, order=order)
    assert np.array_equal(_from_dev_mat(lu, order), lu_ref)
    assert np.array_equal(_from_dev_vec(piv, order), piv_ref)
    assert np.array_equal(info.cpu().numpy(), info_ref)
    lu2, _, _ = integ.lu_factor(t, hd, order=order, out=t)  # in place
    assert lu2.data_ptr() == t.data_ptr()
    assert np.array_equal(_from_dev_mat(lu2, order), lu_ref)
    b = rng.standard_normal((n, nn))
    keep = [0, 2, 3, 4, 5]  # solves with a nonsingular factor
    x_ref = orc.lu_solve(lu_ref[keep], piv_ref[keep], b[keep])
    x = integ.lu_solve(_to_dev_mat(lu_ref[keep], order, cuda_device),
                       _to_dev_vec(piv_ref[keep], order, cuda_device),
                       _to_dev_vec(b[keep], order, cuda_device), order=order)
    assert np.array_equal(_from_dev_vec(x, order), x_ref)


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


def _plan(mech):
    pk = pkg("pack").PackedTables(mech)
    return oracle_mod().lu_plan(pk.crs_row_ptr, pk.crs_col_ind)


@pytest.mark.parametrize("order", ["C", "F"])
@pytest.mark.parametrize("name", ["h2o2", "gri30", "testmech"])
@pytest.mark.parametrize("per_state_h", [False, True])
def test_lu_factor_sparse_bitwise(cuda_device, order, name, per_state_h):
    import torch
    orc = oracle_mod()
    integ = pkg("integrate")
    mech, P, phi, J = _newton_inputs(name, 700, 23)
    plan = _plan(mech)
    h = 10.0 ** np.random.default_rng(4).uniform(-9, -3, J.shape[0]) if per_state_h else 2e-6
    lu_ref, info_ref = orc.lu_factor_sparse(J, integ.ROS2_GAMMA, h, plan)
    ev = pkg("api").Evaluator(mech)
    assert np.array_equal(integ.lu_plan_info(ev)[0], plan["perm"])
    hd = torch.from_numpy(h).to(cuda_device) if per_state_h else h
    lu, info = integ.lu_factor_sparse(ev, _to_dev_mat(J, order, cuda_device), hd,
                                      s=integ.ROS2_GAMMA, order=order)
    assert np.array_equal(_from_dev_mat(lu, order), lu_ref)
    assert np.array_equal(info.cpu().numpy(), info_ref)
    b = np.random.default_rng(9).standard_normal((700, mech.nn))
    x_ref = orc.lu_solve_sparse(lu_ref, b, plan)
    x = integ.lu_solve_sparse(ev, lu, _to_dev_vec(b, order, cuda_device), order=order)
    assert np.array_equal(_from_dev_vec(x, order), x_ref)


def test_lu_factor_sparse_zero_pivot_info(cuda_device):
    """A state whose Newton matrix is exactly zero (s h = 1, J = I) reports
    info = 1, and one whose second pivot overflows reports -2, as the oracle
    does."""
    import torch
    orc = oracle_mod()
    integ = pkg("integrate")
    mech = load_mech("h2o2")
    plan = _plan(mech)
    J = np.zeros((4, mech.nn, mech.nn))
    J[1] = np.eye(mech.nn)
    # state 3: the first elimination step overflows the second pivot
    p0, p1 = plan["perm"][0], plan["perm"][1]
    J[3][p1, p0] = J[3][p0, p1] = -1e200
    lu_ref, info_ref = orc.lu_factor_sparse(J, 1.0, 1.0, plan)
    ev = pkg("api").Evaluator(mech)
    lu, info = integ.lu_factor_sparse(ev, _to_dev_mat(J, "C", cuda_device), 1.0)
    assert list(info.cpu().numpy()) == list(info_ref) == [0, 1, 0, -2]
    bits = lambda a: np.ascontiguousarray(a).view(np.int64)
    assert np.array_equal(bits(lu.cpu().numpy()), bits(lu_ref))


@pytest.mark.parametrize("order", ["C", "F"])
@pytest.mark.parametrize("name", ["h2o2", "gri30"])
def test_ros2_step_sparse_lu_bitwise(cuda_device, order, name):
    """ROS2 with the static-pivot factorisation equals the oracle's sparse LU,
    solves and stage arithmetic applied to this library's rates and Jacobian,
    bit for bit."""
    import torch
    orc = oracle_mod()
    integ = pkg("integrate")
    mech = load_mech(name)
    plan = _plan(mech)
    n = 257
    P, phi = pkg("states").draw_states(mech.n_species, n, seed=19, x_floor=1e-12)
    h = 10.0 ** np.random.default_rng(2).uniform(-10, -7, n)
    ev = pkg("api").Evaluator(mech)
    Pd, hd = torch.from_numpy(P).to(cuda_device), torch.from_numpy(h).to(cuda_device)
    phid = _to_dev_vec(phi, order, cuda_device)

    def rates(y):
        return _from_dev_vec(ev.species_rates(Pd, _to_dev_vec(y, order, cuda_device), order=order),
                             order)

    J = _from_dev_mat(ev.jacobian(Pd, phid, order=order), order)
    lu, info_ref = orc.lu_factor_sparse(J, integ.ROS2_GAMMA, h, plan)
    k1 = orc.lu_solve_sparse(lu, rates(phi), plan)
    k2 = orc.lu_solve_sparse(lu, orc.ros2_combine(1, h, rates(orc.ros2_combine(0, h, phi, k1)), k1),
                             plan)
    ref, err_ref = orc.ros2_combine(2, h, phi, k1, k2)
    st = integ.Ros2Stepper(ev, n, order=order, lu_kind="sparse")
    out, err, info = st.step(Pd, phid, hd)
    assert np.array_equal(info.cpu().numpy(), info_ref)
    assert np.array_equal(_from_dev_vec(out, order), ref)
    assert np.array_equal(_from_dev_vec(err, order), err_ref)


@pytest.mark.parametrize("n_species,states_per_block", [(119, 2), (168, 1)])
def test_lu_factor_sparse_large_mechanisms(cuda_device, tmp_path, n_species, states_per_block):
    """Seeded synthetic mechanisms whose Newton matrices (NN = 120, 169) fit two
    or one per block of shared memory: the sparse and the pivoting
    factorisations stay bit for bit the oracle's.  The random mechanisms'
    Jacobians reach 1e168 at these states, where elimination without
    interchanges overflows, so each state's Jacobian is divided by its largest
    entry first (M = I - 0.0171 J / max|J|); results are compared as bit
    patterns."""
    import torch
    orc = oracle_mod()
    integ = pkg("integrate")
    path = str(tmp_path / "syn.inp")
    pkg("mech.synthetic").write(path, n_species=n_species, n_reactions=3 * n_species, seed=5)
    mech = pkg().load_mechanism(path)
    assert mech.nn == n_species + 1
    assert 4 * mech.nn * (mech.nn | 1) * 8 > 227 * 1024  # not the four-state path
    n = 37
    P, phi = pkg("states").draw_states(mech.n_species, n, seed=6, x_floor=1e-12)
    J = orc.Oracle(mech).jacobian(P, phi)
    J = J / np.abs(J).max(axis=(1, 2), keepdims=True)
    bits = lambda a: np.ascontiguousarray(a).view(np.int64)
    plan = _plan(mech)
    lu_ref, info_ref = orc.lu_factor_sparse(J, integ.ROS2_GAMMA, 1e-2, plan)
    assert np.isfinite(lu_ref).all() and (info_ref == 0).all()
    ev = pkg("api").Evaluator(mech)
    for order in ("C", "F"):
        lu, info = integ.lu_factor_sparse(ev, _to_dev_mat(J, order, cuda_device), 1e-2,
                                          s=integ.ROS2_GAMMA, order=order)
        assert np.array_equal(bits(_from_dev_mat(lu, order)), bits(lu_ref))
        assert np.array_equal(info.cpu().numpy(), info_ref)
    lu_d, piv_d, _ = integ.lu_factor(_to_dev_mat(J, "C", cuda_device), 1e-2, s=integ.ROS2_GAMMA)
    lu_p, piv_p, _ = orc.lu_factor(J, integ.ROS2_GAMMA, 1e-2)
    assert np.array_equal(bits(lu_d.cpu().numpy()), bits(lu_p))
    assert np.array_equal(piv_d.cpu().numpy(), piv_p)


@pytest.mark.parametrize("order", ["C", "F"])
@pytest.mark.parametrize("fmt", ["full", "sparse"])
@pytest.mark.parametrize("name", ["h2o2", "gri30"])
def test_jacobian_rates_one_pass_bitwise(cuda_device, order, fmt, name):
    """pjg_jacobian_rates: the Jacobian equals pjg_jacobian's and the rates
    equal pjg_species_rates', bit for bit, from one pass."""
    import torch
    mech = load_mech(name)
    n = 1000
    P, phi = pkg("states").draw_states(mech.n_species, n, seed=27, x_floor=1e-12)
    ev = pkg("api").Evaluator(mech)
    Pd, phid = torch.from_numpy(P).to(cuda_device), _to_dev_vec(phi, order, cuda_device)
    dphi = torch.empty_like(phid)
    J1 = ev.jacobian(Pd, phid, order=order, jac_format=fmt, dphi=dphi)
    J0 = ev.jacobian(Pd, phid, order=order, jac_format=fmt)
    r0 = ev.species_rates(Pd, phid, order=order)
    assert torch.equal(J1, J0)
    assert torch.equal(dphi, r0)


@pytest.mark.parametrize("lu_kind", ["pivoting", "sparse"])
@pytest.mark.parametrize("name", ["h2o2", "gri30"])
def test_ros2_step_constant_volume_bitwise(cuda_device, lu_kind, name):
    """Constant volume (param = V, phi_1 = P): the step equals the oracle's
    factorisation, solves and stage arithmetic applied to this library's own
    constant-volume rates and Jacobian, bit for bit."""
    import torch
    orc = oracle_mod()
    integ = pkg("integrate")
    mech = load_mech(name)
    n = 300
    V, phi = pkg("states").draw_states(mech.n_species, n, seed=33, x_floor=1e-12, conp=False)
    h = 10.0 ** np.random.default_rng(8).uniform(-10, -7, n)
    ev = pkg("api").Evaluator(mech)
    Vd, hd = torch.from_numpy(V).to(cuda_device), torch.from_numpy(h).to(cuda_device)
    phid = _to_dev_vec(phi, "F", cuda_device)

    def rates(y):
        return _from_dev_vec(ev.species_rates(Vd, _to_dev_vec(y, "F", cuda_device), order="F",
                                              conp=False), "F")

    J = _from_dev_mat(ev.jacobian(Vd, phid, order="F", conp=False), "F")
    if lu_kind == "pivoting":
        lu, piv, info_ref = orc.lu_factor(J, integ.ROS2_GAMMA, h)
        solve = lambda b: orc.lu_solve(lu, piv, b)
    else:
        plan = _plan(mech)
        lu, info_ref = orc.lu_factor_sparse(J, integ.ROS2_GAMMA, h, plan)
        solve = lambda b: orc.lu_solve_sparse(lu, b, plan)
    k1 = solve(rates(phi))
    k2 = solve(orc.ros2_combine(1, h, rates(orc.ros2_combine(0, h, phi, k1)), k1))
    ref, err_ref = orc.ros2_combine(2, h, phi, k1, k2)
    st = integ.Ros2Stepper(ev, n, order="F", lu_kind=lu_kind)
    out, err, info = st.step(Vd, phid, hd, conp=False)
    assert np.array_equal(info.cpu().numpy(), info_ref)
    assert np.array_equal(_from_dev_vec(out, "F"), ref)
    assert np.array_equal(_from_dev_vec(err, "F"), err_ref)


_PREMIX_T = (1000.0, 1100.0, 1200.0, 1300.0)
_PREMIX_T_END = 2e-5
_premix_refs = {}


def _premix_reference(T):
    """Radau (rtol 1e-13) end state of the oracle's ODE for the premix at T."""
    if T not in _premix_refs:
        from scipy.integrate import solve_ivp
        from test_integrate_oracle import premix_h2o2
        mech, P, phi = premix_h2o2(T=T)
        o = oracle_mod().Oracle(mech)
        _premix_refs[T] = solve_ivp(lambda t, v: o.species_rates(P, v[None])[0],
                                    (0, _PREMIX_T_END), phi[0], method="Radau",
                                    jac=lambda t, v: o.jacobian(P, v[None])[0], rtol=1e-13,
                                    atol=1e-22).y[:, -1]
    return _premix_refs[T]


@pytest.mark.parametrize("order,lu_kind", [("C", "pivoting"), ("F", "sparse")])
def test_integrate_ros2_adaptive_premix(cuda_device, order, lu_kind):
    """Adaptive ROS2 (rtol 1e-5) over 20 us on H2/O2/Ar premixes at four
    temperatures, each state with its own step sizes: the end states agree
    with Radau solutions of the oracle's ODE at rtol 1e-13 to 2e-3 of each
    component's scale."""
    import torch
    from test_integrate_oracle import premix_h2o2
    integ = pkg("integrate")
    rows = [premix_h2o2(T=T) for T in _PREMIX_T]
    mech = rows[0][0]
    P = np.concatenate([r[1] for r in rows])
    phi = np.concatenate([r[2] for r in rows])
    ev = pkg("api").Evaluator(mech)
    y, stats = integ.integrate_ros2(ev, torch.from_numpy(P).to(cuda_device),
                                    _to_dev_vec(phi, order, cuda_device), _PREMIX_T_END, h0=1e-9,
                                    rtol=1e-5, atol=1e-16, order=order, lu_kind=lu_kind)
    y = _from_dev_vec(y, order)
    assert (stats["steps"] > 0).all()
    for i, T in enumerate(_PREMIX_T):
        ref = _premix_reference(T)
        scale = np.abs(ref) + 1e-8 * np.abs(ref).max()
        assert (np.abs(y[i] - ref) / scale).max() < 2e-3, (T, stats)


def test_integrate_ros2_radical_rich_states(cuda_device):
    """Radical-rich random GRI states over 10 ns from a first step of 100 ns,
    so that steps are rejected: every state reaches t_end with finite
    values."""
    import torch
    integ = pkg("integrate")
    mech = load_mech("gri30")
    n = 64
    P, phi = pkg("states").draw_states(mech.n_species, n, seed=71, x_floor=1e-12)
    ev = pkg("api").Evaluator(mech)
    y, stats = integ.integrate_ros2(ev, torch.from_numpy(P).to(cuda_device),
                                    torch.from_numpy(phi).to(cuda_device), 1e-8, h0=1e-7,
                                    rtol=1e-4, atol=1e-14)
    assert np.isfinite(y.cpu().numpy()).all()
    assert (stats["steps"] > 0).all() and stats["rejected"].sum() > 0
