"""GPU parity: the CUDA kernels through the C ABI against the CPU oracle.

Tolerances (the spec bars):
* species rates: |gpu - ref| <= 1e-10 * (|ref| + s), s = cancellation scale of
  the entry (the same rate sums with absolute values, oracle.rates_scale);
* Jacobian: |gpu - ref| <= 1e-8 * max_col |ref[row]| (row-relative);
* sparse values equal the dense values at the pattern's (row, col).
"""
import numpy as np
import pytest

from conftest import (bath_rich_states, load_mech, oracle_mod, pkg, rel_err, row_rel_err)

pytestmark = pytest.mark.gpu

RTOL_RATES = 1e-10
RTOL_JAC = 1e-8
MECHS = ["h2o2", "gri30", "testmech", "synthetic_small"]

_ev = {}


def evaluator(name):
    if name not in _ev:
        _ev[name] = pkg("api").Evaluator(load_mech(name))
    return _ev[name]


def states(name, n, seed, conp):
    mech = load_mech(name)
    if name == "gri30":
        return pkg("states").draw_states(mech.n_species, n, seed=seed, x_floor=1e-12, conp=conp)
    if name == "h2o2":
        return pkg("states").draw_states(mech.n_species, n, seed=seed, conp=conp)
    return bath_rich_states(mech, n, seed, conp)


def to_dev(a, device):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def rates_ok(d, ref, scale):
    den = np.abs(ref) + scale
    diff = np.abs(d - ref)
    err = np.where(den > 0, diff / np.where(den > 0, den, 1.0), np.where(diff > 0, np.inf, 0.0))
    return float(err.max())


@pytest.mark.parametrize("name", MECHS)
@pytest.mark.parametrize("conp", [True, False])
@pytest.mark.parametrize("order", ["C", "F"])
def test_species_rates(cuda_device, name, conp, order):
    mech = load_mech(name)
    n = 300  # not a multiple of the block size: exercises the ragged tail
    P, phi = states(name, n, 11, conp)
    o = oracle_mod().Oracle(mech)
    ref = o.species_rates(P, phi, conp=conp)
    scale = o.rates_scale(P, phi, conp=conp)
    ev = evaluator(name)
    x = phi if order == "C" else phi.T
    d = ev.species_rates(to_dev(P, cuda_device), to_dev(x, cuda_device), order=order,
                         conp=conp).cpu().numpy()
    if order == "F":
        d = d.T
    assert np.isfinite(d).all()
    assert rates_ok(d, ref, scale) < RTOL_RATES


def _dense_from(out, order, fmt, mech, dm, n):
    NN = mech.nn
    if fmt == "full":
        if order == "C":
            return out.reshape(n, NN, NN)
        # F: jac[i + N*row + N*NN*col]
        return out.reshape(NN, NN, n).transpose(2, 1, 0)
    ptr, ind = dm.jacobian_indices(order)
    J = np.zeros((n, NN, NN))
    vals = out.reshape(n, -1) if order == "C" else out.reshape(-1, n).T
    for a in range(NN):
        for p in range(ptr[a], ptr[a + 1]):
            if order == "C":
                J[:, a, ind[p]] = vals[:, p]
            else:
                J[:, ind[p], a] = vals[:, p]
    return J


@pytest.mark.parametrize("name", MECHS)
@pytest.mark.parametrize("conp", [True, False])
@pytest.mark.parametrize("order", ["C", "F"])
@pytest.mark.parametrize("fmt", ["full", "sparse"])
def test_jacobian(cuda_device, name, conp, order, fmt):
    mech = load_mech(name)
    n = 200
    P, phi = states(name, n, 12, conp)
    o = oracle_mod().Oracle(mech)
    Jref = o.jacobian(P, phi, conp=conp)
    ev = evaluator(name)
    x = phi if order == "C" else phi.T
    out = ev.jacobian(to_dev(P, cuda_device), to_dev(x, cuda_device), order=order, conp=conp,
                      jac_format=fmt).cpu().numpy()
    assert np.isfinite(out).all()
    J = _dense_from(out, order, fmt, mech, ev, n)
    if fmt == "sparse":
        # entries outside the pattern are not stored; compare on the pattern
        mask = np.zeros((mech.nn, mech.nn), dtype=bool)
        ptr, ind = ev.jacobian_indices("C")
        for r in range(mech.nn):
            mask[r, ind[ptr[r]:ptr[r + 1]]] = True
        Jref = np.where(mask[None], Jref, 0.0)
    assert row_rel_err(J, Jref) < RTOL_JAC


@pytest.mark.parametrize("order", ["C", "F"])
def test_jacobian_repeats_bitwise(cuda_device, order):
    """Each state's entries are summed by one thread in a fixed order (global
    reductions included), so repeated calls are bitwise equal."""
    n = 1000
    P, phi = states("gri30", n, 14, True)
    ev = evaluator("gri30")
    x = phi if order == "C" else phi.T
    tP, tx = to_dev(P, cuda_device), to_dev(x, cuda_device)
    a = ev.jacobian(tP, tx, order=order).cpu().numpy()
    for _ in range(3):
        assert np.array_equal(a, ev.jacobian(tP, tx, order=order).cpu().numpy())


def test_pywrap_kernels_match_device_api(cuda_device):
    """PyJacobianKernel / PySpecies_RatesKernel (host arrays) equal the device path."""
    mech = load_mech("gri30")
    api = pkg("api")
    n = 129
    P, phi = states("gri30", n, 13, True)
    for order in ("C", "F"):
        mod = api.pywrap(mech, order=order, conp=True, jac_format="sparse")
        x = np.ascontiguousarray(phi if order == "C" else phi.T)
        rk = mod.PySpecies_RatesKernel(n, 4)
        dphi = np.zeros_like(x)
        rk(P, x, dphi)
        jk = mod.PyJacobianKernel(n, 4)
        jac = np.zeros(n * mech.jac_nnz())
        jk(P, x, jac)
        ev = evaluator("gri30")
        d2 = ev.species_rates(to_dev(P, cuda_device), to_dev(x, cuda_device), order=order).cpu().numpy()
        j2 = ev.jacobian(to_dev(P, cuda_device), to_dev(x, cuda_device), order=order,
                         jac_format="sparse").cpu().numpy()
        assert np.array_equal(dphi, d2)
        assert np.array_equal(jac, j2.ravel())
        assert rk.num_species() == 53 and rk.num_reactions() == 325
        assert jk.required_working_memory() > 0


def test_indices_bit_exact_device(cuda_device):
    """The index arrays the C ABI returns equal the front end's (bit-exact)."""
    for name in MECHS:
        mech = load_mech(name)
        ev = evaluator(name)
        for order in ("C", "F"):
            ptr, ind = ev.jacobian_indices(order)
            eptr, eind = mech.pattern(order)
            assert np.array_equal(ptr, eptr) and np.array_equal(ind, eind)


@pytest.mark.parametrize("name,n,combos", [
    ("h2o2", 700001, [("C", "full"), ("C", "sparse"), ("F", "full"), ("F", "sparse")]),
    ("gri30", 160000, [("F", "sparse")]),
])
def test_pywrap_kernel_streams_many_chunks(cuda_device, name, n, combos):
    """The host-pointer kernel objects stream large problems through a ring of
    three device buffers of two waves of blocks (155,648 states on 152 SMs;
    strided copies for order F): h2o2 at 700,001 states wraps the ring.  The
    result equals the device-pointer evaluation of the whole problem."""
    mech = load_mech(name)
    api = pkg("api")
    P, phi = states(name, n, 16, True)
    ev = evaluator(name)
    for order, fmt in combos:
        mod = api.pywrap(mech, order=order, conp=True, jac_format=fmt)
        x = np.ascontiguousarray(phi if order == "C" else phi.T)
        per = mech.nn * mech.nn if fmt == "full" else mech.jac_nnz()
        jk = mod.PyJacobianKernel(n, 1)
        jac = np.full(n * per, np.nan)
        jk(P, x, jac)
        ref = ev.jacobian(to_dev(P, cuda_device), to_dev(x, cuda_device), order=order,
                          jac_format=fmt).cpu().numpy().ravel()
        assert np.array_equal(jac, ref), (order, fmt)
        rk = mod.PySpecies_RatesKernel(n, 1)
        dphi = np.full_like(x, np.nan)
        rk(P, x, dphi)
        assert np.array_equal(dphi, ev.species_rates(to_dev(P, cuda_device), to_dev(x, cuda_device),
                                                     order=order).cpu().numpy()), order
        jk.close()
        rk.close()


@pytest.mark.parametrize("name,n,combos", [
    ("h2o2", 400001, [("C", "full"), ("F", "sparse")]),
    ("gri30", 3000, [("F", "full"), ("C", "full"), ("C", "sparse")]),
])
def test_pywrap_kernel_pinned_arrays(cuda_device, name, n, combos):
    """Pinned host arrays (the copies then run asynchronously beside the
    kernels) give the same result as the device-pointer evaluation."""
    import torch
    mech = load_mech(name)
    api = pkg("api")
    P, phi = states(name, n, 17, True)
    ev = evaluator(name)
    hP = torch.from_numpy(P).pin_memory().numpy()
    for order, fmt in combos:
        mod = api.pywrap(mech, order=order, conp=True, jac_format=fmt)
        x = torch.from_numpy(np.ascontiguousarray(phi if order == "C" else phi.T)).pin_memory().numpy()
        per = mech.nn * mech.nn if fmt == "full" else mech.jac_nnz()
        jac = torch.full((n * per,), float("nan"), dtype=torch.float64, pin_memory=True).numpy()
        jk = mod.PyJacobianKernel(n, 1)
        jk(hP, x, jac)
        ref = ev.jacobian(to_dev(hP, cuda_device), to_dev(x, cuda_device), order=order,
                          jac_format=fmt).cpu().numpy().ravel()
        assert np.array_equal(jac, ref), (order, fmt)
        dphi = torch.full(x.shape, float("nan"), dtype=torch.float64, pin_memory=True).numpy()
        rk = mod.PySpecies_RatesKernel(n, 1)
        rk(hP, x, dphi)
        assert np.array_equal(dphi, ev.species_rates(to_dev(hP, cuda_device), to_dev(x, cuda_device),
                                                     order=order).cpu().numpy()), order
        jk.close()
        rk.close()


@pytest.mark.parametrize("order", ["C", "F"])
def test_synthetic500_rates_and_sparse_jacobian(cuda_device, order):
    """The large benchmark mechanism (500 species, 2,500 reactions with
    third-body, Troe, SRI, PLOG and Chebyshev forms; 41k Jacobian non-zeros):
    species rates and the sparse Jacobian (CRS for 'C', CCS for 'F') against
    the oracle on 192 states."""
    mech = load_mech("synthetic500")
    n = 192
    P, phi = pkg("states").draw_states(mech.n_species, n, seed=18)
    o = oracle_mod().Oracle(mech)
    ev = evaluator("synthetic500")
    x = phi if order == "C" else phi.T
    d = ev.species_rates(to_dev(P, cuda_device), to_dev(x, cuda_device), order=order).cpu().numpy()
    d = d if order == "C" else d.T
    assert rates_ok(d, o.species_rates(P, phi), o.rates_scale(P, phi)) < RTOL_RATES
    out = ev.jacobian(to_dev(P, cuda_device), to_dev(x, cuda_device), order=order,
                      jac_format="sparse").cpu().numpy()
    J = _dense_from(out, order, "sparse", mech, ev, n)
    Jref = o.jacobian(P, phi)
    mask = np.zeros((mech.nn, mech.nn), dtype=bool)
    ptr, ind = ev.jacobian_indices("C")
    for r in range(mech.nn):
        mask[r, ind[ptr[r]:ptr[r + 1]]] = True
    assert row_rel_err(J, np.where(mask[None], Jref, 0.0)) < RTOL_JAC
    # the pattern holds every non-zero of the analytical Jacobian
    assert (np.abs(np.where(mask[None], 0.0, Jref)) <= 1e-12 * np.abs(Jref).max()).all()


@pytest.mark.parametrize("name", MECHS)
@pytest.mark.parametrize("conp", [True, False])
@pytest.mark.parametrize("order", ["C", "F"])
def test_chem_utils(cuda_device, name, conp, order):
    """Species thermo (the chem_utils kernel type) against the oracle, over
    temperatures through both NASA ranges and beyond the guards.  h and b
    cross zero along the sweep, so the error is measured against each
    species' largest magnitude (the kernels use precomputed polynomial
    quotients, the oracle divides: last-ulp differences)."""
    mech = load_mech(name)
    n = 300
    P, phi = states(name, n, 19, conp)
    phi = phi.copy()
    phi[:, 0] = np.linspace(50.0, 12000.0, n)
    ref = oracle_mod().Oracle(mech).chem_utils(phi, conp=conp)
    x = phi if order == "C" else phi.T
    got = evaluator(name).chem_utils(to_dev(x, cuda_device), order=order, conp=conp)
    for g, r in zip(got, ref):
        g = g.cpu().numpy()
        g = g if order == "C" else g.T
        scale = np.abs(r).max(axis=0, keepdims=True)
        assert np.max(np.abs(g - r) / scale) < 1e-13


def test_pywrap_chem_utils_kernel(cuda_device):
    mech = load_mech("gri30")
    n = 129
    P, phi = states("gri30", n, 20, True)
    mod = pkg("api").pywrap(mech, order="F", conp=True)
    ck = mod.PyChem_UtilsKernel(n, 1)
    x = np.ascontiguousarray(phi.T)
    cp, h, b = (np.zeros(n * mech.n_species) for _ in range(3))
    ck(x, cp, h, b)
    ref = oracle_mod().Oracle(mech).chem_utils(phi)
    for got, r in zip((cp, h, b), ref):
        scale = np.abs(r).max(axis=0, keepdims=True)
        assert np.max(np.abs(got.reshape(mech.n_species, n).T - r) / scale) < 1e-13


@pytest.mark.parametrize("name", ["h2o2", "gri30", "testmech", "synthetic_small"])
@pytest.mark.parametrize("order", ["C", "F"])
@pytest.mark.parametrize("fmt", ["full", "sparse"])
def test_approximate_jacobian(cuda_device, name, order, fmt):
    """The 'approximate' Jacobian type (tables flag bit 1): its own pattern,
    bit-exact index arrays, and values equal to the oracle's approximate
    Jacobian."""
    mech = load_mech(name, jac_type="approximate")
    n = 200
    P, phi = states(name, n, 21, True)
    Jref = oracle_mod().Oracle(mech).jacobian(P, phi)
    ev = pkg("api").Evaluator(mech)
    ptr, ind = ev.jacobian_indices(order)
    eptr, eind = mech.pattern(order)
    assert np.array_equal(ptr, eptr) and np.array_equal(ind, eind)
    x = phi if order == "C" else phi.T
    out = ev.jacobian(to_dev(P, cuda_device), to_dev(x, cuda_device), order=order,
                      jac_format=fmt).cpu().numpy()
    assert np.isfinite(out).all()
    assert row_rel_err(_dense_from(out, order, fmt, mech, ev, n), Jref) < RTOL_JAC


def test_pywrap_kernel_registered_host_arrays(cuda_device):
    """The kernel object into host arrays page-locked in place
    (hostmem.empty -> pjg_host_register) gives the same Jacobian as into
    pageable arrays; the registration is released with the array."""
    import gc
    mech = load_mech("gri30")
    n = 20000
    P, phi = pkg("states").draw_states(mech.n_species, n, seed=44, x_floor=1e-12)
    x = np.ascontiguousarray(phi.T)
    hm = pkg("hostmem")
    mod = pkg("api").pywrap(mech, order="F")
    k = mod.PyJacobianKernel(n, 1)
    ref = np.empty(n * mech.nn * mech.nn)
    k(P, x, ref)
    hP = hm.empty(P.shape)
    hx = hm.empty(x.shape)
    hout = hm.empty(ref.shape)
    hP[:] = P
    hx[:] = x
    k(hP, hx, hout)
    assert np.array_equal(hout, ref)
    k.close()
    del hP, hx, hout
    gc.collect()
    assert not pkg("hostmem")._keep


def test_pywrap_kernel_large_mechanism_whole_wave_chunks(cuda_device):
    """The kernel object for the 500-species mechanism's sparse C-order
    Jacobian: 1.37 MB of ring and working arrays per state put two waves past
    its 32 GiB budget, so it takes one whole wave per chunk when half the free
    device memory holds it (else what the budget holds).  90,000 states span
    more than one wave; states on both sides of every possible chunk boundary
    must match the oracle."""
    import torch
    torch.cuda.empty_cache()
    mech = load_mech("synthetic500")
    n = 90000
    P, phi = pkg("states").draw_states(mech.n_species, n, seed=51)
    mod = pkg("api").pywrap(mech, order="C", jac_format="sparse")
    k = mod.PyJacobianKernel(n, 1)
    ev = evaluator("synthetic500")
    nnz = ev.nnz
    out = np.empty(n * nnz)
    k(P, phi, out)
    k.close()
    bounds = set()
    for c in (77824, 25344, 25088, 24576):
        bounds.update(range(c, n, c))
    pick = np.unique(np.concatenate([np.r_[0:8, n - 8:n]] +
                                    [np.r_[b - 4:b + 4] for b in sorted(bounds)]))
    pick = pick[(pick >= 0) & (pick < n)]
    J = out.reshape(n, nnz)[pick]
    Jref = oracle_mod().Oracle(mech).jacobian(P[pick], phi[pick])
    ptr, ind = ev.jacobian_indices("C")
    rows = np.repeat(np.arange(mech.nn), np.diff(ptr))
    ref = Jref[:, rows, ind]
    scale = np.abs(Jref).max(axis=2)[:, rows]
    scale[scale == 0] = 1.0
    assert np.isfinite(J).all()
    assert (np.abs(J - ref) / scale).max() < RTOL_JAC
