"""torch.autograd binding of the plain-method solve.

``omni_solve(solver, ax, ay, az)`` returns p as a differentiable function of the three
acceleration components.  The backward pass calls the library's hand-written adjoint
(omni3d_adjoint): the transpose of the solve's affine map, computed by scattering back
along the lines and through the iterations without stored iterates.  Only the plain method
is differentiable (the selected method's weights depend on the field through the curl).
"""
from __future__ import annotations

import torch


class _OmniSolve(torch.autograd.Function):
    @staticmethod
    def forward(ctx, ax, ay, az, solver, p_init):
        args = [t.detach().reshape(-1).to(torch.float32).contiguous() for t in (ax, ay, az)]
        p0 = None if p_init is None else p_init.detach().reshape(-1).to(torch.float32).contiguous()
        r = solver.solve(*args, p_init=p0)
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
        return gx.reshape(ctx.shape), gy.reshape(ctx.shape), gz.reshape(ctx.shape), None, None


def omni_solve(solver, ax, ay, az, p_init=None):
    """p = P(ax, ay, az) through `solver` (an omni3d.Omni3D with method="plain"),
    differentiable with respect to ax, ay, az."""
    if solver.method != "plain":
        raise ValueError("only the plain method is differentiable")
    return _OmniSolve.apply(ax, ay, az, solver, p_init)
