"""torch entry points: the species rates as a differentiable function.

``wdot(evaluator, param, phi)`` returns dphi/dt (T, extra variable and molar
rates) for CUDA float64 tensors.  Its backward is the hand-written
vector-Jacobian product kernel (``pjg_vjp``): ``J^T v`` is assembled on the fly
from the same per-reaction quantities as the Jacobian, without materialising
the (NN x NN) Jacobian.  No reference counterpart: pyJac exposes the Jacobian
only, this is its adjoint for gradient-based use.  ``param`` (P or V) is not
differentiated.
"""
import torch


class _Wdot(torch.autograd.Function):
    @staticmethod
    def forward(ctx, param, phi, ev, order, conp):
        param = param.contiguous()
        phi = phi.contiguous()
        out = ev.species_rates(param, phi, order=order, conp=conp)
        ctx.save_for_backward(param, phi)
        ctx.ev, ctx.order, ctx.conp = ev, order, conp
        return out

    @staticmethod
    def backward(ctx, grad):
        param, phi = ctx.saved_tensors
        g = None
        if ctx.needs_input_grad[1]:
            g = ctx.ev.vjp(param, phi, grad.contiguous(), order=ctx.order, conp=ctx.conp)
        return None, g, None, None, None


def wdot(ev, param, phi, order="C", conp=True):
    """Differentiable species rates; ``ev`` is an api.Evaluator."""
    return _Wdot.apply(param, phi, ev, order, conp)


def jacobian_vector_product(ev, param, phi, u, order="C", conp=True):
    """J u through the dense Jacobian kernel (reference path for tests and tools)."""
    J = ev.jacobian(param, phi, order=order, conp=conp, jac_format="full")
    if order == "C":
        return torch.einsum("nrc,nc->nr", J, u)
    # F layout: J[col, row, state]
    return torch.einsum("crn,cn->rn", J, u)
