"""The κ-Poisson residual as a differentiable torch function.

R(u, m) = K(exp(m)) u - F, with K the kappa-weighted P1 stiffness and
kappa = exp(m) per element. With a BoundaryMap, constrained rows are replaced
by R_bc = u_bc - g (femx's replaceRes, BoundaryMap.cpp:172-189), which is the
residual femx's constrained residuals hand to the state and adjoint solvers.

backward() is the transpose action the adjoint drivers need
(femx/state/Residual.hpp:55-59, femx/inverse/ReducedFunctional.hpp:94-117),
computed element by element by gbfem_vjp_p1_kappa without forming the
Jacobian or its transpose:
    lam~      = lam with constrained rows zeroed          (zeroBoundary)
    dL/du     = K^T lam~ + lam on the constrained rows
    dL/dm_e   = kappa_e lam~_e^T Khat_e u_e
"""
from __future__ import annotations

import torch

from . import assembly as A

__all__ = ["P1KappaResidual", "p1_kappa_residual"]


class P1KappaResidual(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u, m, amap, coords, f, bc, bc_vals, precision):
        kappa = torch.exp(m)
        res = torch.empty(amap.numRes(), dtype=torch.float64, device=u.device)
        A.assembleP1Kappa(amap, coords, kappa, f, u, res, None, precision=precision)
        if bc is not None:
            A.replaceRes(bc, u, bc_vals, res)
        ctx.save_for_backward(u, kappa)
        ctx.amap, ctx.coords, ctx.bc, ctx.precision = amap, coords, bc, precision
        return res

    @staticmethod
    def backward(ctx, lam):
        u, kappa = ctx.saved_tensors
        lam = lam.contiguous()
        lam_t = lam
        if ctx.bc is not None:
            lam_t = lam.clone()
            A.zeroBoundary(ctx.bc, lam_t)
        g_u = torch.empty_like(u) if ctx.needs_input_grad[0] else None
        g_m = torch.empty_like(kappa) if ctx.needs_input_grad[1] else None
        if g_u is not None or g_m is not None:
            A.vjpP1Kappa(ctx.amap, ctx.coords, kappa, u, lam_t, g_u, g_m,
                         precision=ctx.precision)
        if g_u is not None and ctx.bc is not None:
            rows = ctx.bc.view()["bc_rows"].long()
            g_u.index_add_(0, rows, lam.index_select(0, rows))
        return g_u, g_m, None, None, None, None, None, None


def p1_kappa_residual(u, m, amap, coords, f=None, bc=None, bc_vals=None,
                      precision: str = "fp64"):
    """R(u, m) as a differentiable function of the state u and the control m."""
    return P1KappaResidual.apply(u, m, amap, coords, f, bc, bc_vals, precision)
