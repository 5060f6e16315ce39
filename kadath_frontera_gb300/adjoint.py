"""dQ/dp of a converged observable as a torch.autograd.Function.

forward(p) sets the double constant `cst` of the system to p, runs Newton
steps (System_of_eqs.do_newton) until |F| < precision, and returns Q: the
value of the unknown `var` at `point` (ConvergedObservable), or an integral
observable (ConvergedIntegral: the integral at infinity of an expression,
as FUKA's ADM mass -integ(dn(P)) / (2 pi), or a sum of volume integrals).
backward() uses the adjoint of the converged system (J^T lambda = dQ/dy,
dQ/dp = -lambda . dF/dp) instead of finite differences of re-solves: one
FP64 factorisation and one transposed solve, or, with reuse_factors and a
mixed-precision Newton solve, GMRES on J^T preconditioned by that solve's
last factors (no new factorisation).
"""
from __future__ import annotations

import numpy as np
import torch


def _converge(syst, precision, max_steps, lu_mode):
    for _ in range(max_steps):
        done, err = syst.do_newton(precision, lu_mode=lu_mode)
        if done:
            return
    raise RuntimeError(f"Newton did not converge (|F| = {err:.3e})")


class ConvergedObservable(torch.autograd.Function):
    @staticmethod
    def forward(ctx, p, syst, field, var, cst, point, precision=1e-12, max_steps=30):
        syst.set_cst(cst, float(p.item()))
        _converge(syst, precision, max_steps, None)
        q = field.val_point(point)
        g = syst.val_point_gradient(var, point)
        dqdp, _ = syst.adjoint(g, cst)
        ctx.save_for_backward(torch.tensor(dqdp, dtype=p.dtype))
        return torch.tensor(q, dtype=p.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        (dqdp,) = ctx.saved_tensors
        return grad_out * dqdp, None, None, None, None, None, None, None


class ConvergedIntegral(torch.autograd.Function):
    @staticmethod
    def forward(ctx, p, syst, expr, kind, domains, scale, cst, precision, max_steps, lu_mode, reuse_factors):
        syst.set_cst(cst, float(p.item()))
        _converge(syst, precision, max_steps, lu_mode)
        q, g = syst.integral_gradient(expr, kind, domains)
        dqdp, _ = syst.adjoint(scale * g, cst, reuse_factors=reuse_factors)
        ctx.save_for_backward(torch.tensor(dqdp, dtype=p.dtype))
        return torch.tensor(scale * q, dtype=p.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        (dqdp,) = ctx.saved_tensors
        return (grad_out * dqdp,) + (None,) * 10


def converged_observable(p, syst, field, var, cst, point, precision=1e-12):
    """Q(p) with dQ/dp by the adjoint: differentiable in p (a 0-d tensor)."""
    return ConvergedObservable.apply(p, syst, field, var, cst, np.asarray(point, dtype=float), precision)


def converged_integral(p, syst, expr, cst, kind="inf", domains=None, scale=1.0, precision=1e-12, max_steps=30,
                       lu_mode=None, reuse_factors=False):
    """Q(p) = scale * (integral observable expr) at the converged fields, with
    dQ/dp by the adjoint: differentiable in p (a 0-d tensor).  For the ADM
    mass of a conformal factor P: expr = "integ(dn(P))", scale = -1 / (2 pi)."""
    return ConvergedIntegral.apply(p, syst, expr, kind, domains, scale, cst, precision, max_steps, lu_mode,
                                   reuse_factors)
