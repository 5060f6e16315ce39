"""dQ/dp of a converged observable as a torch.autograd.Function.

forward(p) sets the double constant `cst` of the system to p, runs Newton
steps (System_of_eqs.do_newton) until |F| < precision, and returns Q = the
value of the unknown `var` at `point`.  backward() uses the adjoint of the
converged system (J^T lambda = dQ/dy, dQ/dp = -lambda . dF/dp), one FP64
factorisation and one transposed solve, instead of finite differences of
re-solves.
"""
from __future__ import annotations

import numpy as np
import torch


class ConvergedObservable(torch.autograd.Function):
    @staticmethod
    def forward(ctx, p, syst, field, var, cst, point, precision=1e-12, max_steps=30):
        syst.set_cst(cst, float(p.item()))
        for _ in range(max_steps):
            done, err = syst.do_newton(precision)
            if done:
                break
        else:
            raise RuntimeError(f"Newton did not converge (|F| = {err:.3e})")
        q = field.val_point(point)
        g = syst.val_point_gradient(var, point)
        dqdp, _ = syst.adjoint(g, cst)
        ctx.save_for_backward(torch.tensor(dqdp, dtype=p.dtype))
        return torch.tensor(q, dtype=p.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        (dqdp,) = ctx.saved_tensors
        return grad_out * dqdp, None, None, None, None, None, None, None


def converged_observable(p, syst, field, var, cst, point, precision=1e-12):
    """Q(p) with dQ/dp by the adjoint: differentiable in p (a 0-d tensor)."""
    return ConvergedObservable.apply(p, syst, field, var, cst, np.asarray(point, dtype=float), precision)
