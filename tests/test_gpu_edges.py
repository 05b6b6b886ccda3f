"""GPU edge cases against the oracle: empty and single-state batches, states at
and beyond the guards' limits, exact-zero moles, and problems that span more
than one launch chunk of the working buffer.

The guards are pyJac's (pyjac/core/instruction_creator.py:370-478): rates use
T clamped to [100, 10000] K, moles floored at 1e-300 in the concentration
products, exp arguments clamped at 690.775527898; the explicit T, V, P factors
of the Jacobian use the unclamped state.
"""
import numpy as np
import pytest

from conftest import load_mech, oracle_mod, pkg, row_rel_err

pytestmark = pytest.mark.gpu

RTOL_RATES = 1e-10
RTOL_JAC = 1e-8


def _dev(a, device):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def _rates_err(d, ref, scale):
    den = np.abs(ref) + scale
    diff = np.abs(d - ref)
    return float(np.where(den > 0, diff / np.where(den > 0, den, 1.0),
                          np.where(diff > 0, np.inf, 0.0)).max())


def _check(ev, mech, P, phi, order, conp, device):
    o = oracle_mod().Oracle(mech)
    ref = o.species_rates(P, phi, conp=conp)
    scale = o.rates_scale(P, phi, conp=conp)
    x = phi if order == "C" else phi.T
    d = ev.species_rates(_dev(P, device), _dev(x, device), order=order, conp=conp).cpu().numpy()
    d = d if order == "C" else d.T
    assert np.isfinite(d).all()
    assert _rates_err(d, ref, scale) < RTOL_RATES
    n, NN = phi.shape
    out = ev.jacobian(_dev(P, device), _dev(x, device), order=order, conp=conp).cpu().numpy()
    J = out.reshape(n, NN, NN) if order == "C" else out.reshape(NN, NN, n).transpose(2, 1, 0)
    assert np.isfinite(J).all()
    assert row_rel_err(J, o.jacobian(P, phi, conp=conp)) < RTOL_JAC


@pytest.mark.parametrize("order", ["C", "F"])
def test_empty_batch_writes_nothing(cuda_device, order):
    import torch
    mech = load_mech("gri30")
    ev = pkg("api").Evaluator(mech)
    P = torch.zeros(0, dtype=torch.float64, device=cuda_device)
    phi = torch.zeros((0, mech.nn) if order == "C" else (mech.nn, 0), dtype=torch.float64,
                      device=cuda_device)
    assert ev.species_rates(P, phi, order=order).numel() == 0
    assert ev.jacobian(P, phi, order=order).numel() == 0
    assert ev.vjp(P, phi, phi, order=order).numel() == 0


@pytest.mark.parametrize("order", ["C", "F"])
@pytest.mark.parametrize("conp", [True, False])
def test_single_state(cuda_device, order, conp):
    mech = load_mech("gri30")
    P, phi = pkg("states").draw_states(mech.n_species, 1, seed=5, x_floor=1e-12, conp=conp)
    _check(pkg("api").Evaluator(mech), mech, P, phi, order, conp, cuda_device)


@pytest.mark.parametrize("name", ["h2o2", "gri30"])
@pytest.mark.parametrize("order", ["C", "F"])
def test_temperatures_at_and_beyond_the_limits(cuda_device, name, order):
    """T below the 100 K clamp, across the NASA-7 switch at T_mid, up to and
    beyond the 10,000 K clamp."""
    mech = load_mech(name)
    temps = np.array([80.0, 100.0, 100.5, 300.0, 999.999999, 1000.0, 1000.000001, 2500.0,
                      3500.0, 6000.0, 9999.0, 10000.0, 12000.0])
    P, phi = pkg("states").draw_states(mech.n_species, temps.size, seed=21, x_floor=1e-12)
    # keep the composition and pressure, move T (moles follow the ideal gas law)
    phi = phi.copy()
    phi[:, 2:] *= (phi[:, 0] / temps)[:, None]
    phi[:, 0] = temps
    _check(pkg("api").Evaluator(mech), mech, P, phi, order, True, cuda_device)


def _gibbs_b(mech, T):
    """b_k = S_k/R - H_k/(R T) - ln T of every species at each T (NASA-7), the
    exponent of the equilibrium constants' per-species factors"""
    out = np.empty((T.size, mech.n_species))
    lnT = np.log(T)
    for k, sp in enumerate(mech.species):
        lo, hi = np.asarray(sp.lo, float), np.asarray(sp.hi, float)
        a = np.where((T < sp.Trange[1])[:, None], lo[None, :], hi[None, :])
        h = (a[:, 0] + T * (a[:, 1] / 2 + T * (a[:, 2] / 3 + T * (a[:, 3] / 4 + T * a[:, 4] / 5)))
             + a[:, 5] / T)
        s = a[:, 0] * lnT + T * (a[:, 1] + T * (a[:, 2] / 2 + T * (a[:, 3] / 3 + T * a[:, 4] / 4))) + a[:, 6]
        out[:, k] = s - h - lnT
    return out


@pytest.mark.parametrize("order", ["C", "F"])
def test_equilibrium_constants_on_both_sides_of_the_split(cuda_device, order):
    """1 / Kc is the product of per-species factors exp(+-b_k) in states whose
    |b_k| are all at most 138, and exp(-sum nu b) per reaction in the others
    (GRI below about 500 K): states of both kinds interleaved within every
    warp, rates, Jacobian and J^T v against the oracle."""
    mech = load_mech("gri30")
    n = 256
    rng = np.random.default_rng(41)
    temps = np.where(np.arange(n) % 3 == 0, rng.uniform(250.0, 700.0, n), rng.uniform(700.0, 3000.0, n))
    big = np.abs(_gibbs_b(mech, temps)).max(axis=1) > 138.0
    assert 0.1 < big.mean() < 0.5
    P, phi = pkg("states").draw_states(mech.n_species, n, seed=41, x_floor=1e-12)
    phi = phi.copy()
    phi[:, 2:] *= (phi[:, 0] / temps)[:, None]
    phi[:, 0] = temps
    ev = pkg("api").Evaluator(mech)
    _check(ev, mech, P, phi, order, True, cuda_device)
    v = rng.standard_normal(phi.shape)
    J = oracle_mod().Oracle(mech).jacobian(P, phi)
    ref = np.einsum("nrc,nr->nc", J, v)
    scale = np.einsum("nrc,nr->nc", np.abs(J), np.abs(v))
    x, vv = (phi, v) if order == "C" else (phi.T, v.T)
    out = ev.vjp(_dev(P, cuda_device), _dev(x, cuda_device), _dev(vv, cuda_device),
                 order=order).cpu().numpy()
    out = out if order == "C" else out.T
    assert np.isfinite(out).all()
    assert (np.abs(out - ref) / np.where(scale > 0, scale, 1.0)).max() < 1e-9


@pytest.mark.parametrize("order", ["C", "F"])
def test_exact_zero_moles(cuda_device, order):
    """Species with exactly zero moles exercise the 1e-300 floors."""
    mech = load_mech("gri30")
    P, phi = pkg("states").draw_states(mech.n_species, 257, seed=8, x_floor=1e-12)
    phi = phi.copy()
    rng = np.random.default_rng(8)
    zero = rng.random(phi[:, 2:].shape) < 0.5
    phi[:, 2:][zero] = 0.0
    phi[0, 2:] = 0.0  # bath gas only
    _check(pkg("api").Evaluator(mech), mech, P, phi, order, True, cuda_device)


def test_problem_spanning_several_launches(cuda_device):
    """The per-state working arrays are capped (8 GiB), so large batches run as
    several launches of whole waves of resident blocks: for the dense GRI
    Jacobian in order 'C' (27 KB of scratch per state) four waves, 311,296
    states on a 152-SM GB300.  States on both sides of every multiple of one
    wave (77,824 states there) up to 320,000 must match the oracle."""
    import torch
    mech = load_mech("gri30")
    NN = mech.nn
    n = 320000
    P, phi = pkg("states").draw_states(mech.n_species, n, seed=31, x_floor=1e-12)
    ev = pkg("api").Evaluator(mech)
    out = ev.jacobian(_dev(P, cuda_device), _dev(phi, cuda_device), order="C")
    wave = 77824
    pick = np.unique(np.concatenate([np.r_[0:32, n - 32:n]] +
                                    [np.r_[m - 32:m + 32] for m in range(wave, n, wave)]))
    idx = torch.from_numpy(pick).to(cuda_device)
    J = out.view(n, NN, NN).index_select(0, idx).cpu().numpy()
    del out
    torch.cuda.empty_cache()
    Jref = oracle_mod().Oracle(mech).jacobian(P[pick], phi[pick])
    assert np.isfinite(J).all()
    assert row_rel_err(J, Jref) < RTOL_JAC


def test_table_driven_exp_against_cuda_exp(cuda_device):
    """The kernels' exponential (Tang's table-driven method) against the CUDA
    library exp (each within about 1 ulp of the true value): at most 3 ulp
    apart over the range the kinetics use, identical beyond |x| = 708 where the
    library takes over, and the same IEEE special values."""
    import torch
    lib = pkg("_lib")
    rng = np.random.default_rng(17)
    x = np.concatenate([rng.uniform(-745.0, 709.7, 2_000_000), rng.uniform(-1, 1, 500_000),
                        rng.uniform(-1e-8, 1e-8, 100_000),
                        np.array([0.0, -0.0, 1.0, -1.0, 707.999, -707.999, 708.0, -708.0, 709.7,
                                  -745.0, 690.775527898, -690.775527898, 800.0, -800.0,
                                  np.inf, -np.inf, np.nan])])
    tx = torch.from_numpy(x).to(cuda_device)
    y = torch.empty_like(tx)
    st = torch.cuda.current_stream(cuda_device).cuda_stream
    assert lib.load().pjg_math_exp(tx.data_ptr(), y.data_ptr(), tx.numel(), st) == 0
    ref = torch.exp(tx)  # the CUDA library exp
    torch.cuda.synchronize()
    y, ref = y.cpu().numpy(), ref.cpu().numpy()
    same_class = (np.isnan(y) == np.isnan(ref)) & (np.isinf(y) == np.isinf(ref))
    assert same_class.all()
    fin = np.isfinite(ref) & (ref > 0)
    ulp = np.abs(y[fin] - ref[fin]) / np.spacing(ref[fin])
    assert ulp.max() <= 3.0, ulp.max()
    assert (y[~fin & ~np.isnan(ref)] == ref[~fin & ~np.isnan(ref)]).all()
