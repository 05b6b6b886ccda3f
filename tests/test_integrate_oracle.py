"""The oracle of the implicit-step row (Newton-matrix LU, solves, ROS2),
pinned on the CPU: the factorisation against LAPACK's dgetrf (through
scipy.linalg.lu_factor: identical pivots, factors to rounding), the solves
against numpy.linalg.solve, and the ROS2 step against a tightly converged
Radau solution of the same ODE (second-order convergence)."""
import numpy as np
import pytest

from conftest import load_mech, oracle_mod, pkg

sl = pytest.importorskip("scipy.linalg")


def _newton(J, s, h):
    n, nn = J.shape[:2]
    hs = np.broadcast_to(np.asarray(h, dtype=np.float64), (n,))
    return np.eye(nn)[None] - (s * hs)[:, None, None] * J


@pytest.mark.parametrize("name,h", [("h2o2", 1e-6), ("h2o2", 1e-3), ("gri30", 1e-7), ("gri30", 1e-4)])
def test_lu_factor_matches_lapack_on_newton_matrices(name, h):
    mech = load_mech(name)
    P, phi = pkg("states").draw_states(mech.n_species, 64, seed=3, x_floor=1e-12)
    J = oracle_mod().Oracle(mech).jacobian(P, phi)
    orc = oracle_mod()
    lu, piv, info = orc.lu_factor(J, orc.ROS2_GAMMA, h)
    M = _newton(J, orc.ROS2_GAMMA, h)
    assert (info == 0).all()
    for i in range(J.shape[0]):
        LU, p = sl.lu_factor(M[i])
        assert np.array_equal(p + 1, piv[i])
        scale = np.abs(M[i]).max()
        assert np.abs(LU - lu[i]).max() <= 1e-12 * scale


def test_lu_factor_random_matrices_pivot_like_lapack():
    orc = oracle_mod()
    rng = np.random.default_rng(11)
    J = rng.standard_normal((200, 17, 17))
    h = rng.uniform(0.5, 2.0, 200)
    lu, piv, info = orc.lu_factor(J, 1.0, h)
    M = _newton(J, 1.0, h)
    swaps = 0
    for i in range(200):
        LU, p = sl.lu_factor(M[i])
        assert np.array_equal(p + 1, piv[i])
        assert np.abs(LU - lu[i]).max() <= 1e-12 * np.abs(M[i]).max() * 17
        swaps += int((p != np.arange(17)).sum())
    assert swaps > 1000  # partial pivoting is exercised


def test_lu_factor_zero_pivot_info():
    """A zero column gives LAPACK's info (1-based index of the first zero
    pivot) and leaves the factorisation finite."""
    orc = oracle_mod()
    rng = np.random.default_rng(2)
    M = rng.standard_normal((3, 6, 6))
    M[0, :, 2] = 0.0            # zero column 2 -> info 3
    M[1, :, 0] = 0.0            # zero column 0 -> info 1
    J = np.eye(6)[None] - M    # so that I - 1 * 1 * J = M
    lu, piv, info = orc.lu_factor(J, 1.0, 1.0)
    assert list(info) == [3, 1, 0]
    assert np.isfinite(lu).all()
    for i in range(3):
        LU, p = sl.lu_factor(M[i], check_finite=False) if i == 2 else (None, None)
        if i == 2:
            assert np.array_equal(p + 1, piv[i])


def test_lu_solve_matches_numpy():
    orc = oracle_mod()
    mech = load_mech("gri30")
    P, phi = pkg("states").draw_states(mech.n_species, 32, seed=4, x_floor=1e-12)
    J = oracle_mod().Oracle(mech).jacobian(P, phi)
    lu, piv, _ = orc.lu_factor(J, orc.ROS2_GAMMA, 1e-6)
    b = np.random.default_rng(5).standard_normal((32, mech.nn))
    x = orc.lu_solve(lu, piv, b)
    M = _newton(J, orc.ROS2_GAMMA, 1e-6)
    ref = np.linalg.solve(M, b[..., None])[..., 0]
    err = np.abs(x - ref).max(axis=1) / np.abs(ref).max(axis=1)
    assert err.max() < 1e-10


def premix_h2o2(T=1200.0, P=101325.0):
    """H2 : O2 : AR = 0.2 : 0.1 : 0.7 (other species 1e-10) at T, P, V = 1 m^3."""
    mech = load_mech("h2o2")
    names = mech.species_names()
    X = np.full(mech.n_species, 1e-10)
    for sp, x in (("H2", 0.2), ("O2", 0.1), ("AR", 0.7)):
        X[names.index(sp)] = x
    X /= X.sum()
    n = X * P / (8314.4621 * T)
    return mech, np.array([P]), np.concatenate([[T, 1.0], n[:-1]])[None]


def test_ros2_converges_at_second_order():
    """ROS2 with the oracle's rates and Jacobian on an H2/O2/Ar premix in its
    induction period (1200 K, 20 us): the error against a Radau solution at
    rtol 1e-13 falls by about 4x per halving of the step."""
    from scipy.integrate import solve_ivp
    orc = oracle_mod()
    mech, P, phi = premix_h2o2()
    o = orc.Oracle(mech)
    t_end = 2e-5

    def f(t, y):
        return o.species_rates(P, y[None])[0]

    def jac(t, y):
        return o.jacobian(P, y[None])[0]

    ref = solve_ivp(f, (0, t_end), phi[0], method="Radau", jac=jac, rtol=1e-13,
                    atol=1e-22).y[:, -1]
    scale = np.abs(ref) + 1e-8 * np.abs(ref).max()
    errs = []
    for steps in (16, 32, 64):
        y = phi.copy()
        h = t_end / steps
        for _ in range(steps):
            y, err, info = orc.ros2_step(o, P, y, h)
            assert (info == 0).all()
        errs.append((np.abs(y[0] - ref) / scale).max())
    rates = [errs[i] / errs[i + 1] for i in range(2)]
    assert all(3.0 < r < 5.5 for r in rates), (errs, rates)


@pytest.mark.parametrize("name", ["h2o2", "gri30", "testmech"])
def test_lu_symbolic_matches_oracle_plan(name):
    """The library's host Markowitz order (pjg_lu_symbolic, no GPU) equals the
    oracle's independent restatement, with the same fill and FMA counts."""
    orc = oracle_mod()
    mech = load_mech(name)
    pk = pkg("pack").PackedTables(mech)
    plan = orc.lu_plan(pk.crs_row_ptr, pk.crs_col_ind)
    perm, nnz, fma = pkg("integrate").lu_symbolic(pk.crs_row_ptr, pk.crs_col_ind)
    assert np.array_equal(perm, plan["perm"])
    assert (nnz, fma) == (plan["nnz_lu"], plan["fma"])
    if name == "gri30":
        assert (nnz, fma) == (2043, 19752)  # against 2,916 entries and 51,039 FMAs dense


def test_lu_symbolic_random_patterns():
    orc = oracle_mod()
    rng = np.random.default_rng(4)
    for nn in (1, 3, 17, 40):
        A = rng.random((nn, nn)) < 0.2
        rp = np.concatenate([[0], np.cumsum(A.sum(1))]).astype(np.int32)
        ci = np.nonzero(A)[1].astype(np.int32)
        plan = orc.lu_plan(rp, ci)
        perm, nnz, fma = pkg("integrate").lu_symbolic(rp, ci)
        assert np.array_equal(perm, plan["perm"]) and (nnz, fma) == (plan["nnz_lu"], plan["fma"])


@pytest.mark.parametrize("h", [1e-8, 1e-6, 1e-4])
def test_sparse_lu_solves_match_numpy(h):
    orc = oracle_mod()
    mech = load_mech("gri30")
    pk = pkg("pack").PackedTables(mech)
    plan = orc.lu_plan(pk.crs_row_ptr, pk.crs_col_ind)
    P, phi = pkg("states").draw_states(mech.n_species, 64, seed=3, x_floor=1e-12)
    J = orc.Oracle(mech).jacobian(P, phi)
    lu, info = orc.lu_factor_sparse(J, orc.ROS2_GAMMA, h, plan)
    assert (info == 0).all()
    b = np.random.default_rng(1).standard_normal((64, mech.nn))
    x = orc.lu_solve_sparse(lu, b, plan)
    ref = np.linalg.solve(_newton(J, orc.ROS2_GAMMA, h), b[..., None])[..., 0]
    assert (np.abs(x - ref).max(axis=1) / np.abs(ref).max(axis=1)).max() < 1e-7


def test_ros2_sparse_lu_converges_at_second_order():
    from scipy.integrate import solve_ivp
    orc = oracle_mod()
    mech, P, phi = premix_h2o2()
    o = orc.Oracle(mech)
    pk = pkg("pack").PackedTables(mech)
    plan = orc.lu_plan(pk.crs_row_ptr, pk.crs_col_ind)
    t_end = 2e-5
    ref = solve_ivp(lambda t, y: o.species_rates(P, y[None])[0], (0, t_end), phi[0],
                    method="Radau", jac=lambda t, y: o.jacobian(P, y[None])[0], rtol=1e-13,
                    atol=1e-22).y[:, -1]
    scale = np.abs(ref) + 1e-8 * np.abs(ref).max()
    errs = []
    for steps in (16, 32, 64):
        y = phi.copy()
        for _ in range(steps):
            y, _, info = orc.ros2_step(o, P, y, t_end / steps, plan=plan)
        errs.append((np.abs(y[0] - ref) / scale).max())
    rates = [errs[i] / errs[i + 1] for i in range(2)]
    assert all(3.0 < r < 5.5 for r in rates), (errs, rates)


def test_lu_symbolic_large_mechanism():
    """The host symbolic analysis sizes mechanisms beyond the factorisation
    kernels' NN <= 169: the 500-species benchmark mechanism fills to 205,216
    L + U entries and 28.9M FMAs per state, as the oracle's restatement
    finds."""
    orc = oracle_mod()
    mech = load_mech("synthetic500")
    pk = pkg("pack").PackedTables(mech)
    perm, nnz, fma = pkg("integrate").lu_symbolic(pk.crs_row_ptr, pk.crs_col_ind)
    plan = orc.lu_plan(pk.crs_row_ptr, pk.crs_col_ind)
    assert np.array_equal(perm, plan["perm"])
    assert (nnz, fma) == (plan["nnz_lu"], plan["fma"]) == (205216, 28893626)


def test_ros2_constant_volume_converges_at_second_order():
    """The same premix at constant volume (param = V = 1 m^3, phi_1 = P): the
    oracle's ROS2 converges at second order against Radau on the conv ODE."""
    from scipy.integrate import solve_ivp
    orc = oracle_mod()
    mech, P, phi = premix_h2o2()
    o = orc.Oracle(mech)
    V = np.array([1.0])
    phi = phi.copy()
    phi[0, 1] = P[0]  # phi_1 is the pressure at constant volume
    t_end = 2e-5
    ref = solve_ivp(lambda t, v: o.species_rates(V, v[None], conp=False)[0], (0, t_end), phi[0],
                    method="Radau", jac=lambda t, v: o.jacobian(V, v[None], conp=False)[0],
                    rtol=1e-13, atol=1e-22).y[:, -1]
    scale = np.abs(ref) + 1e-8 * np.abs(ref).max()
    errs = []
    for steps in (16, 32, 64):
        y = phi.copy()
        for _ in range(steps):
            y, _, info = orc.ros2_step(o, V, y, t_end / steps, conp=False)
        errs.append((np.abs(y[0] - ref) / scale).max())
    rates = [errs[i] / errs[i + 1] for i in range(2)]
    assert all(3.0 < r < 5.5 for r in rates), (errs, rates)


def test_sparse_lu_reports_overflowing_pivots():
    """Without interchanges a pivot can overflow: info is then minus the
    1-based step of the first non-finite pivot, and a zero pivot that comes
    first keeps its positive step."""
    orc = oracle_mod()
    mech = load_mech("h2o2")
    pk = pkg("pack").PackedTables(mech)
    plan = orc.lu_plan(pk.crs_row_ptr, pk.crs_col_ind)
    p0, p1, p2 = plan["perm"][:3]
    J = np.zeros((3, mech.nn, mech.nn))
    J[0][p1, p0] = J[0][p0, p1] = -1e200      # a_11 = 1 - 1e400: -inf at step 2
    J[1][p2, p2] = 1.0                          # exactly zero pivot at step 3
    J[2][p2, p2] = 1.0
    J[2][p1, p0] = J[2][p0, p1] = -1e200      # the overflow (step 2) comes first
    lu, info = orc.lu_factor_sparse(J, 1.0, 1.0, plan)
    assert list(info) == [-2, 3, -2]
