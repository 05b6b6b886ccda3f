"""Host-side control of the adaptive ROS2 driver (integrate.integrate_ros2),
on the CPU with a stand-in stepper: the exact solution of y' = -k y per state,
reporting an error estimate proportional to h^2 like ROS2's embedded one."""
import numpy as np
import pytest

from conftest import pkg

torch = pytest.importorskip("torch")


class ExactDecay(object):
    """step(): y_new = y exp(-k h), err = c (k h)^2 y, per state (order 'C')."""

    def __init__(self, k, c=1.0):
        self.k = torch.as_tensor(k, dtype=torch.float64)
        self.c = c
        self.calls = 0
        self.zero_steps_changed = False

    def step(self, param, y, h, conp=True, out=None, err=None):
        self.calls += 1
        kh = (self.k * h)[:, None]
        out.copy_(y * torch.exp(-kh))
        err.copy_(self.c * kh * kh * y)
        zero = h == 0
        if zero.any() and not torch.equal(out[zero], y[zero]):
            self.zero_steps_changed = True
        return out, err, None


def _run(k, t_end, **kw):
    integ = pkg("integrate")
    n = len(k)
    y0 = torch.ones((n, 3), dtype=torch.float64)
    st = ExactDecay(k)
    y, stats = integ.integrate_ros2(None, torch.zeros(n, dtype=torch.float64), y0, t_end,
                                    stepper=st, **kw)
    return y0, y, stats, st


def test_reaches_t_end_with_per_state_steps():
    k = [1.0, 1e2, 1e4]
    y0, y, stats, st = _run(k, 1e-3, h0=1e-8, rtol=1e-4, atol=1e-30)
    # the stand-in stepper is exact: every state ends at exp(-k t_end) iff its
    # accepted steps sum to t_end exactly
    ref = torch.exp(-torch.tensor(k, dtype=torch.float64) * 1e-3)[:, None] * y0
    assert torch.allclose(y, ref, rtol=1e-9, atol=0)
    assert (stats["steps"] > 0).all()
    # stiffer states need more steps
    assert stats["steps"][0] < stats["steps"][1] < stats["steps"][2]
    assert not st.zero_steps_changed


def test_rejects_and_recovers():
    # a first step far too large for k = 1e6 is rejected, then shrunk
    y0, y, stats, st = _run([1.0, 1e5], 1e-4, h0=1e-4, rtol=1e-3, atol=1e-30)
    assert stats["rejected"][1] > 0
    ref = torch.exp(-torch.tensor([1e-4, 10.0], dtype=torch.float64))[:, None]
    assert torch.allclose(y, ref, rtol=1e-9, atol=0)


def test_finished_states_take_zero_steps():
    y0, y, stats, st = _run([1.0, 1e5], 1e-3, h0=1e-3, rtol=1e-3, atol=1e-30)
    # the slow state finishes in one step; the loop keeps stepping the other
    assert stats["steps"][0] == 1 and st.calls > 1
    assert not st.zero_steps_changed


def test_max_steps_raises():
    with pytest.raises(RuntimeError, match="max_steps"):
        _run([1e9], 1.0, h0=1e-12, rtol=1e-8, atol=1e-30, max_steps=5)


def test_exactly_max_steps_is_not_a_failure():
    # the slow state reaches t_end in one accepted step (h0 = t_end), so a
    # step cap of exactly one is enough and must not raise
    y0, y, stats, st = _run([1.0], 1e-3, h0=1e-3, rtol=1e-3, atol=1e-30, max_steps=1)
    assert stats["steps"][0] == 1 and st.calls == 1
    assert torch.allclose(y, torch.exp(torch.tensor(-1e-3, dtype=torch.float64)) * y0,
                          rtol=1e-12, atol=0)


def test_entry_points_validate_before_the_library():
    """Host tensors, wrong dtypes and non-square matrices are refused in
    Python, before any library call."""
    integ = pkg("integrate")
    cpu = torch.zeros((2, 3, 3), dtype=torch.float64)
    with pytest.raises(TypeError):
        integ.lu_factor(cpu, 1e-6)
    with pytest.raises(TypeError):
        integ.lu_solve(cpu, torch.zeros((2, 3), dtype=torch.int32), torch.zeros((2, 3)))
    with pytest.raises(ValueError, match="square"):
        integ._n_of(torch.zeros((2, 3, 4)), "C")
    with pytest.raises(ValueError, match="dense"):
        integ._n_of(torch.zeros((2, 3)), "C")
    with pytest.raises(ValueError):
        integ.Ros2Stepper.__init__(object.__new__(integ.Ros2Stepper), None, 4, lu_kind="qr")
