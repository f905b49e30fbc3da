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

__all__ = ["P1KappaResidual", "p1_kappa_residual", "TaylorHoodResidual",
           "taylor_hood_residual"]


class P1KappaResidual(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u, m, amap, coords, f, bc, bc_vals, precision, tiled=False):
        kappa = torch.exp(m)
        res = torch.empty(amap.numRes(), dtype=torch.float64, device=u.device)
        A.assembleP1Kappa(amap, coords, kappa, f, u, res, None, precision=precision,
                          tiled=tiled)
        if bc is not None:
            A.replaceRes(bc, u, bc_vals, res)
        ctx.save_for_backward(u, kappa)
        ctx.amap, ctx.coords, ctx.bc, ctx.precision = amap, coords, bc, precision
        ctx.tiled = tiled
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
                         precision=ctx.precision, tiled=ctx.tiled)
        if g_u is not None and ctx.bc is not None:
            rows = ctx.bc.view()["bc_rows"].long()
            g_u.index_add_(0, rows, lam.index_select(0, rows))
        return g_u, g_m, None, None, None, None, None, None, None


def p1_kappa_residual(u, m, amap, coords, f=None, bc=None, bc_vals=None,
                      precision: str = "fp64", tiled: bool = False):
    """R(u, m) as a differentiable function of the state u and the control m.
    tiled=True (amap.enableTiles(coords) first; precision "fp64" or
    "double_float"): the owner-computes tiled residual and VJPs, no atomics,
    bitwise reproducible forward and backward."""
    return P1KappaResidual.apply(u, m, amap, coords, f, bc, bc_vals, precision, tiled)


class TaylorHoodResidual(torch.autograd.Function):
    """The Taylor-Hood P2/P1 steady Navier-Stokes residual R(state, nu), with
    constrained rows replaced by state - g when a BoundaryMap is given.

    backward() gives the state VJP J(state)^T lam element by element through
    gbfem_vjp_th_ns without forming J (the transpose action of
    TimeResidual::applyJacT / the adjoint solves, femx/state/TimeResidual.hpp:
    223-227, ConstrainedTimeResidual.cpp:379-405, which zeroes the constrained
    adjoint entries first), plus lam on the constrained rows; and the
    viscosity derivative: R is affine in nu, so (dR/dnu)^T lam =
    lam~ . (R(nu = 1) - R(nu = 0)), two residual assemblies.
    """

    @staticmethod
    def forward(ctx, state, nu, amap, coords, conn6, bc, bc_vals, precision):
        res = torch.empty(amap.numRes(), dtype=torch.float64, device=state.device)
        A.assembleTaylorHood(amap, coords, conn6, float(nu), state, res, None,
                             precision=precision)
        if bc is not None:
            A.replaceRes(bc, state, bc_vals, res)
        ctx.save_for_backward(state)
        ctx.nu, ctx.amap, ctx.coords, ctx.conn6, ctx.bc = float(nu), amap, coords, conn6, bc
        ctx.precision = precision
        return res

    @staticmethod
    def backward(ctx, lam):
        (state,) = ctx.saved_tensors
        lam = lam.contiguous()
        lam_t = lam
        if ctx.bc is not None:
            lam_t = lam.clone()
            A.zeroBoundary(ctx.bc, lam_t)
        g_state = g_nu = None
        if ctx.needs_input_grad[0]:
            g_state = torch.empty_like(state)
            A.vjpTaylorHood(ctx.amap, ctx.coords, ctx.conn6, ctx.nu, state, lam_t, g_state,
                            precision=ctx.precision)
            if ctx.bc is not None:
                rows = ctx.bc.view()["bc_rows"].long()
                g_state.index_add_(0, rows, lam.index_select(0, rows))
        if ctx.needs_input_grad[1]:
            r1 = torch.empty(ctx.amap.numRes(), dtype=torch.float64, device=state.device)
            r0 = torch.empty_like(r1)
            A.assembleTaylorHood(ctx.amap, ctx.coords, ctx.conn6, 1.0, state, r1, None,
                                 precision=ctx.precision)
            A.assembleTaylorHood(ctx.amap, ctx.coords, ctx.conn6, 0.0, state, r0, None,
                                 precision=ctx.precision)
            g_nu = torch.dot(lam_t, r1 - r0).reshape(())
        return g_state, g_nu, None, None, None, None, None, None


def taylor_hood_residual(state, nu, amap, coords, conn6, bc=None, bc_vals=None,
                         precision: str = "fp64"):
    """R(state, nu) as a differentiable function of the state and of nu (a
    float, or a 0-dim float64 tensor to differentiate with respect to it)."""
    if not torch.is_tensor(nu):
        nu = torch.tensor(float(nu), dtype=torch.float64, device=state.device)
    return TaylorHoodResidual.apply(state, nu, amap, coords, conn6, bc, bc_vals, precision)
