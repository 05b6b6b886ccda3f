"""pjg_vjp_noalloc: the allocation-free J^T v entry point (GPU).

Callers that cannot allocate device memory at call time (solvers calling the
chemistry from a hot loop, hosts whose pool owns all device memory) use this
entry point; its scratch is a fixed array inside the library.  It must give
the same result as pjg_vjp, on consecutive calls, including problems larger
than one scratch-sized chunk, and it must not take device memory: on a fresh
mechanism whose working buffer was never allocated, a call leaves the free
device memory unchanged.  Collected last so that a failure here comes after
every other test has run.
"""
import numpy as np
import pytest

from conftest import bath_rich_states, load_mech, pkg

pytestmark = pytest.mark.gpu


def _call(lib, fn, dm, n, order, P, phi, v, out):
    import torch
    st = torch.cuda.current_stream(P.device).cuda_stream
    return getattr(lib, fn)(dm.handle, n, order.encode(), 1, P.data_ptr(), phi.data_ptr(),
                            v.data_ptr(), out.data_ptr(), st)


def _inputs(mech, n, order, device, seed):
    import torch
    P, phi = bath_rich_states(mech, n, seed, True)
    x = phi if order == "C" else np.ascontiguousarray(phi.T)
    return (torch.from_numpy(P).to(device), torch.from_numpy(np.ascontiguousarray(x)).to(device))


def test_noalloc_takes_no_device_memory(cuda_device):
    """A call on a fresh mechanism (no working buffer yet) after a warm-up
    call (which loads the module that holds the fixed array) changes the
    free device memory by nothing; the mechanism tables are uploaded before
    the measurement."""
    import torch
    L = pkg("_lib")
    lib = L.load()
    mech = load_mech("gri30")
    n = 10000
    tP, tphi = _inputs(mech, n, "F", cuda_device, 7)
    v = torch.randn(tphi.shape, dtype=torch.float64, device=cuda_device)
    out = torch.empty_like(tphi)
    warm = pkg("api").DeviceMechanism(mech)
    assert _call(lib, "pjg_vjp_noalloc", warm, n, "F", tP, tphi, v, out) == 0, L.last_error()
    torch.cuda.synchronize()
    fresh = pkg("api").DeviceMechanism(mech)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    assert _call(lib, "pjg_vjp_noalloc", fresh, n, "F", tP, tphi, v, out) == 0, L.last_error()
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, (free0, free1)
    # pjg_vjp on the same fresh mechanism grows its working buffer: the
    # measurement above would have seen an allocation
    ref = torch.empty_like(tphi)
    assert _call(lib, "pjg_vjp", fresh, n, "F", tP, tphi, v, ref) == 0, L.last_error()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] < free1
    assert float((out - ref).abs().max() / ref.abs().max()) <= 1e-12


@pytest.mark.parametrize("order", ["C", "F"])
def test_noalloc_vjp_matches_pjg_vjp_on_consecutive_calls(cuda_device, order):
    import torch
    L = pkg("_lib")
    lib = L.load()
    mech = load_mech("gri30")
    dm = pkg("api").DeviceMechanism(mech)
    n = 10000  # more than one 3,840-state chunk of the 16 MiB scratch for GRI-Mech 3.0
    tP, tphi = _inputs(mech, n, order, cuda_device, 41)
    rng = np.random.default_rng(3)
    for call in range(2):
        v = torch.from_numpy(rng.standard_normal(tuple(tphi.shape))).to(cuda_device)
        ref = torch.empty_like(tphi)
        got = torch.full_like(tphi, float("nan"))
        assert _call(lib, "pjg_vjp_noalloc", dm, n, order, tP, tphi, v, got) == 0, L.last_error()
        assert _call(lib, "pjg_vjp", dm, n, order, tP, tphi, v, ref) == 0, L.last_error()
        torch.cuda.synchronize()
        assert torch.isfinite(got).all()
        err = float((got - ref).abs().max() / ref.abs().max())
        assert err <= 1e-12, (call, err)


def test_noalloc_rejects_bad_arguments(cuda_device):
    L = pkg("_lib")
    lib = L.load()
    assert lib.pjg_vjp_noalloc(None, 10, b"C", 1, None, None, None, None, None) == -1
    dm = pkg("api").DeviceMechanism(load_mech("h2o2"))
    assert lib.pjg_vjp_noalloc(dm.handle, 10, b"X", 1, None, None, None, None, None) == -1
    assert "order" in L.last_error()
    assert lib.pjg_vjp_noalloc(dm.handle, 0, b"C", 1, None, None, None, None, None) == 0
