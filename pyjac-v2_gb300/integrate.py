"""Linearly implicit integration on this library's Jacobians (device arrays).

The consumer of the Jacobian in real use: an implicit ODE solver factors the
Newton matrix M = I - s h J of every state and solves with it once per stage.
No reference counterpart (the reference lists coupling to Rosenbrock solvers
as future work).  Everything runs in the CUDA library (include/pyjac_gb300.h:
pjg_lu_factor, pjg_lu_solve, pjg_lu_factor_sparse, pjg_lu_solve_sparse,
pjg_ros2_step) on the current torch stream.

Two factorisations: partial pivoting (LAPACK dgetf2's algorithm, any dense
matrix up to 4096 x 4096: in shared memory up to 169, above that blocked in
global memory with the same operations), and the static-pivot sparse LU of
implicit chemistry
solvers (KPP): rows and columns ordered once by the Markowitz rule on the
mechanism's Jacobian pattern, no interchanges, only the filled pattern
updated (GRI-Mech 3.0: 19,752 FMAs per state instead of 51,039).

On top of the step, integrate_ros2 advances every state to a common end time
with its own adaptive step sizes (the control runs as a few element-wise
tensor operations per step; the step itself is the library's).

Layouts are the dense Jacobian's: order 'C' — jac and lu (N, NN, NN)
[state, row, col]; order 'F' — (NN, NN, N) [col, row, state].  Vectors and
pivots are laid out like phi: (N, NN) for 'C', (NN, N) for 'F'.  Step sizes
are a Python float (the same for every state) or a CUDA float64 tensor of N
per-state values.
"""
import torch

from . import _lib
from .api import _order

ROS2_GAMMA = 1.7071067811865475  # 1 + 1/sqrt(2)


def _stream(t):
    return torch.cuda.current_stream(t.device).cuda_stream


def _h_args(h, n):
    if isinstance(h, torch.Tensor):
        if not (h.is_cuda and h.dtype == torch.float64 and h.is_contiguous() and h.numel() == n):
            raise ValueError("h must be a contiguous CUDA float64 tensor of %d values" % n)
        return h.data_ptr(), 0.0
    return None, float(h)


def _check_f64(*ts):
    for t in ts:
        if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float64
                and t.is_contiguous()):
            raise TypeError("expected contiguous CUDA float64 tensors")


def _n_of(jac, order):
    if jac.dim() != 3:
        raise ValueError("jac must be a dense (N, NN, NN) or (NN, NN, N) tensor")
    nn = jac.shape[1]
    n = jac.shape[0] if order == "C" else jac.shape[2]
    if (order == "C" and jac.shape[2] != nn) or (order == "F" and jac.shape[0] != nn):
        raise ValueError("jac must be square per state")
    return n, nn


def lu_factor(jac, h, s=1.0, order="C", out=None, info=True):
    """Factor M_i = I - s h_i J_i with partial pivoting (LAPACK dgetf2's
    algorithm).  Returns (lu, piv, info): lu like jac (``out=jac`` factors in
    place), piv int32 1-based row interchanges laid out like phi, info int32
    (N,) = 0 or the 1-based index of the first exactly zero pivot."""
    _check_f64(jac)
    n, nn = _n_of(jac, order)
    lu = torch.empty_like(jac) if out is None else out
    _check_f64(lu)
    if lu.shape != jac.shape:
        raise ValueError("out must match jac")
    piv = torch.empty((n, nn) if order == "C" else (nn, n), dtype=torch.int32, device=jac.device)
    inf = torch.empty(n, dtype=torch.int32, device=jac.device) if info else None
    hp, h0 = _h_args(h, n)
    _lib.check("pjg_lu_factor", _lib.load().pjg_lu_factor(
        nn, n, _order(order), float(s), hp, h0, jac.data_ptr(), lu.data_ptr(), piv.data_ptr(),
        None if inf is None else inf.data_ptr(), _stream(jac)))
    return lu, piv, inf


def lu_solve(lu, piv, b, order="C"):
    """b <- M^-1 b in place from lu_factor's output; returns b."""
    _check_f64(lu, b)
    n, nn = _n_of(lu, order)
    if b.numel() != n * nn or piv.numel() != n * nn or piv.dtype != torch.int32:
        raise ValueError("b and piv must hold N x NN values")
    _lib.check("pjg_lu_solve", _lib.load().pjg_lu_solve(
        nn, n, _order(order), lu.data_ptr(), piv.data_ptr(), b.data_ptr(), _stream(lu)))
    return b


def lu_symbolic(row_ptr, col_ind):
    """Markowitz order of a CRS pattern (plus the diagonal) and its counts,
    computed on the host: (perm, nnz of L + U, FMAs per state), with
    perm[position] = variable."""
    import ctypes
    import numpy as np
    rp = np.ascontiguousarray(row_ptr, dtype=np.int32)
    ci = np.ascontiguousarray(col_ind, dtype=np.int32)
    nn = rp.size - 1
    perm = np.empty(nn, dtype=np.int32)
    nnz = ctypes.c_int32()
    fma = ctypes.c_int64()
    _lib.check("pjg_lu_symbolic", _lib.load().pjg_lu_symbolic(
        nn, rp.ctypes.data, ci.ctypes.data, perm.ctypes.data, ctypes.addressof(nnz),
        ctypes.byref(fma)))
    return perm, nnz.value, fma.value


def lu_plan_info(evaluator):
    """The mechanism's static-pivot plan: (perm, nnz of L + U, FMAs per state)."""
    import ctypes
    import numpy as np
    perm = np.empty(evaluator.nn, dtype=np.int32)
    nnz = ctypes.c_int32()
    fma = ctypes.c_int64()
    _lib.check("pjg_lu_plan_info", evaluator._lib.pjg_lu_plan_info(
        evaluator.handle, perm.ctypes.data, ctypes.addressof(nnz), ctypes.byref(fma)))
    return perm, nnz.value, fma.value


def lu_factor_sparse(evaluator, jac, h, s=1.0, order="C", out=None):
    """Static-pivot factorisation of M_i = I - s h_i J_i on the evaluator's
    mechanism plan.  Returns (lu, info): lu like jac, holding the factors of
    the permuted matrix M[perm][:, perm]; info int32 (N,) = 0, the 1-based
    step k of the first exactly zero pivot, or -k where a pivot that is not
    finite comes first (overflow without interchanges: factor those states
    with lu_factor instead)."""
    _check_f64(jac)
    n, nn = _n_of(jac, order)
    if nn != evaluator.nn:
        raise ValueError("jac does not match the mechanism")
    lu = torch.empty_like(jac) if out is None else out
    _check_f64(lu)
    inf = torch.empty(n, dtype=torch.int32, device=jac.device)
    hp, h0 = _h_args(h, n)
    _lib.check("pjg_lu_factor_sparse", evaluator._lib.pjg_lu_factor_sparse(
        evaluator.handle, n, _order(order), float(s), hp, h0, jac.data_ptr(), lu.data_ptr(),
        inf.data_ptr(), _stream(jac)))
    return lu, inf


def lu_solve_sparse(evaluator, lu, b, order="C"):
    """b <- M^-1 b in place from lu_factor_sparse's output; returns b."""
    _check_f64(lu, b)
    n, nn = _n_of(lu, order)
    if b.numel() != n * nn:
        raise ValueError("b must hold N x NN values")
    _lib.check("pjg_lu_solve_sparse", evaluator._lib.pjg_lu_solve_sparse(
        evaluator.handle, n, _order(order), lu.data_ptr(), b.data_ptr(), _stream(lu)))
    return b


class Ros2Stepper(object):
    """Steps of the L-stable two-stage Rosenbrock method ROS2 (Verwer, Spee,
    Blom and Hundsdorfer, SIAM J. Sci. Comput. 20(4), 1999) for up to
    ``capacity`` states of one mechanism:

        (I - gamma h J) k1 = f(y),  (I - gamma h J) k2 = f(y + h k1) - 2 k1,
        y_new = y + 1.5 h k1 + 0.5 h k2,  err = 0.5 h (k1 + k2)

    with f the species rates and J the analytical Jacobian at y
    (gamma = 1 + 1/sqrt 2).  ``lu_kind`` "pivoting" factors the Newton matrix
    with partial pivoting, "sparse" with the mechanism's static-pivot plan.
    The work arrays (a dense Jacobian per state) are allocated once; after a
    step ``lu`` (and ``piv`` for "pivoting") hold the factors of the step's
    Newton matrix."""

    def __init__(self, evaluator, capacity, order="C", device=None, lu_kind="pivoting"):
        if lu_kind not in ("pivoting", "sparse"):
            raise ValueError("lu_kind must be 'pivoting' or 'sparse'")
        self.ev = evaluator
        self.order = order
        self.lu_kind = lu_kind
        self.capacity = int(capacity)
        nn = evaluator.nn
        dev = device or torch.device("cuda", torch.cuda.current_device())
        n = max(self.capacity, 1)
        self.lu = torch.empty((n, nn, nn) if order == "C" else (nn, nn, n), dtype=torch.float64,
                              device=dev)
        self.piv = (torch.empty((n, nn) if order == "C" else (nn, n), dtype=torch.int32, device=dev)
                    if lu_kind == "pivoting" else None)
        self.vec = torch.empty(2 * n * nn, dtype=torch.float64, device=dev)
        self.info = torch.empty(n, dtype=torch.int32, device=dev)

    def step(self, param, phi, h, conp=True, out=None, err=None):
        """One step from phi; returns (phi_new, err, info)."""
        n, st = self.ev._prep(param, phi, self.order)
        if n != self.capacity:
            raise ValueError("the stepper was sized for %d states" % self.capacity)
        if out is None:
            out = torch.empty_like(phi)
        if err is None:
            err = torch.empty_like(phi)
        hp, h0 = _h_args(h, n)
        _lib.check("pjg_ros2_step", self.ev._lib.pjg_ros2_step(
            self.ev.handle, n, _order(self.order), int(bool(conp)), param.data_ptr(), phi.data_ptr(),
            hp, h0, 0 if self.lu_kind == "pivoting" else 1, out.data_ptr(), err.data_ptr(),
            self.lu.data_ptr(), None if self.piv is None else self.piv.data_ptr(),
            self.vec.data_ptr(), self.info.data_ptr(), st))
        return out, err, self.info[:n]


def integrate_ros2(evaluator, param, phi, t_end, h0=1e-8, rtol=1e-6, atol=1e-12, order="C",
                   conp=True, lu_kind="pivoting", max_steps=100000, stepper=None):
    """Integrate every state from t = 0 to t_end with ROS2 steps of its own
    size, controlled by the embedded first-order error estimate.

    A state's step is accepted when max_j |err_j| / (atol + rtol max(|y_j|,
    |y_new_j|)) <= 1; its next step is h * min(5, max(0.2, 0.9 / sqrt(e))) (the
    estimate is O(h^2)), cut to reach t_end exactly.  States that have reached
    t_end take steps of size 0, which leave them unchanged.  Returns
    (phi at t_end, stats) with stats = dict(steps=..., rejected=...) per state
    (CPU int64 arrays).  param and phi as for Evaluator; phi is not modified."""
    n = param.numel()
    st = stepper or Ros2Stepper(evaluator, n, order=order, lu_kind=lu_kind)
    dev = phi.device
    y = phi.clone()
    t = torch.zeros(n, dtype=torch.float64, device=dev)
    h = torch.full((n,), float(h0), dtype=torch.float64, device=dev)
    steps = torch.zeros(n, dtype=torch.int64, device=dev)
    rejected = torch.zeros(n, dtype=torch.int64, device=dev)
    y_new = torch.empty_like(y)
    err = torch.empty_like(y)
    state_dim = 1 if order == "C" else 0  # the axis that holds one state's variables
    for _ in range(int(max_steps)):
        live = t < t_end
        if not bool(live.any()):
            break
        hs = torch.where(live, torch.minimum(h, t_end - t), torch.zeros_like(h))
        st.step(param, y, hs.contiguous(), conp=conp, out=y_new, err=err)
        scale = atol + rtol * torch.maximum(y.abs(), y_new.abs())
        e = (err.abs() / scale).amax(dim=state_dim)
        e = torch.where(torch.isfinite(e), e, torch.full_like(e, float("inf")))
        ok = live & (e <= 1.0)
        acc = ok.unsqueeze(state_dim) if order == "C" else ok.unsqueeze(0)
        y = torch.where(acc, y_new, y)
        t = torch.where(ok, t + hs, t)
        steps += ok.to(torch.int64)
        rejected += (live & ~ok).to(torch.int64)
        fac = torch.clamp(0.9 / torch.sqrt(torch.clamp(e, min=1e-10)), 0.2, 5.0)
        h = torch.where(live, hs * fac, h)
    if bool((t < t_end).any()):
        # a run that needs exactly max_steps steps ends here with every state
        # at t_end, and is not a failure
        raise RuntimeError("integrate_ros2: max_steps reached before t_end")
    return y, {"steps": steps.cpu().numpy(), "rejected": rejected.cpu().numpy()}
