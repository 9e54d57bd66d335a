"""torch.autograd binding of the solve.

``omni_solve(solver, ax, ay, az)`` returns p as a differentiable function of the three
acceleration components.  The backward pass calls the library's hand-written adjoint
(omni3d_adjoint): the transpose of the solve's affine map, computed by scattering back
along the lines and through the iterations without stored iterates.  Every method is
differentiable with the curl field held fixed: the methods other than the plain one weight
and split their lines by the curl, and the gradient does not flow through it (the curl
given in ``curl``, or the one the solve computes from the field and ``mask``, is treated as
a constant).
"""
from __future__ import annotations

import torch


class _OmniSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, ax, ay, az, solver, p_init, curl, mask):
        args = [t.detach().reshape(-1).to(torch.float32).contiguous() for t in (ax, ay, az)]
        flat = lambda t: None if t is None else t.detach().reshape(-1).to(torch.float32).contiguous()
        r = solver.solve(*args, p_init=flat(p_init), curl=flat(curl), mask=flat(mask))
        ctx.solver = solver
        ctx.token = solver.solve_count
        ctx.shape = ax.shape
        return r.p.reshape(ax.shape)

    @staticmethod
    def backward(ctx, grad_p):
        s = ctx.solver
        if s.solve_count != ctx.token:
            raise RuntimeError("omni_solve: the solver context ran another solve before this backward pass; "
                               "use one context per differentiated solve")
        gx, gy, gz = s.adjoint(grad_p.contiguous())
        return gx.reshape(ctx.shape), gy.reshape(ctx.shape), gz.reshape(ctx.shape), None, None, None, None


def omni_solve(solver, ax, ay, az, p_init=None, curl=None, mask=None):
    """p = P(ax, ay, az) through `solver` (an omni3d.Omni3D), differentiable with respect
    to ax, ay, az; the curl (given, or computed from the field and mask) is held fixed."""
    return _OmniSolve.apply(ax, ay, az, solver, p_init, curl, mask)
