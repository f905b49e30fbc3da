"""Checks of a Taylor-Hood Newton assembly against the exact weak-form
integrals of th_exact.py and the identities of the operator. Each check
takes `assemble(coords_p2, conn6, num_dofs, nu, state) -> (res, J dense)`
so the same checks pin the oracle (CPU tests) and every GPU precision mode.
"""
from __future__ import annotations

import numpy as np

import th_exact as X
from femx_gb300 import meshes


def _rel(a, b, scale=None):
    a, b = np.asarray(a), np.asarray(b)
    den = np.max(np.abs(b)) if scale is None else scale
    return float(np.max(np.abs(a - b)) / den) if a.size else 0.0


def mesh(nx, jitter_seed=None):
    if jitter_seed is None:
        c3, k3 = meshes.structured_tri(nx)
    else:
        c3, k3 = meshes.jittered_tri(nx, seed=jitter_seed)
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    _, _, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    return cp2, conn6, nv, nd


def check_linear_fields(assemble, tol_r, tol_j, seeds=(1, 2), nus=(1e-3, 1.0),
                        r_scale="ref"):
    """Every row of R and J against the exact integrals, for random linear
    velocity and pressure fields on jittered, permuted meshes.

    R's error is taken relative to ||R_exact||_inf (r_scale="ref"), or, for
    FP32 element arithmetic, relative to the size of R's terms,
    max_i sum_j |J_ij U_j| (r_scale="terms"): a linear velocity makes the
    diffusion terms cancel in the interior rows (lap u = 0), so R is much
    smaller than the terms whose FP32 rounding it carries."""
    worst = 0.0
    for seed in seeds:
        cp2, conn6, nv, nd = mesh(5, jitter_seed=seed)
        rng = np.random.default_rng(100 + seed)
        for nu in nus:
            state = X.linear_state(cp2, nv, rng.standard_normal((2, 3)), rng.standard_normal(3))
            r_ex, j_ex = X.exact_linear_system(cp2, conn6, cp2.shape[0], nd, nu, state)
            res, jac = assemble(cp2, conn6, nd, nu, state)
            scale = None if r_scale == "ref" else float(np.max(np.abs(j_ex) @ np.abs(state)))
            er, ej = _rel(res, r_ex, scale), _rel(jac, j_ex)
            assert er <= tol_r, (seed, nu, er)
            assert ej <= tol_j, (seed, nu, ej)
            worst = max(worst, er, ej)
    return worst


def check_patch_solutions(assemble, tol, nu=0.05, nx=6):
    """Quadratic-velocity / linear-pressure solutions: interior momentum rows
    carry exactly the forcing the strong form implies (zero for the exact
    Poiseuille and Couette flows), and every continuity row vanishes (div u
    = 0). The tolerance is relative to the size of the residual's terms
    (max over rows of sum_j |J_ij U_j|)."""
    cp2, conn6, nv, nd = mesh(nx)
    n2 = cp2.shape[0]
    inner = X.interior_velocity_rows(cp2)
    out = {}
    for name, (vel, pres, load, force) in X.patch_cases(nu).items():
        state = X.patch_state(cp2, nv, vel, pres)
        res, jac = assemble(cp2, conn6, nd, nu, state)
        scale = max(float(np.max(np.abs(jac) @ np.abs(state))), 1e-300)
        expect = X.patch_expected(cp2, conn6, n2, load, force)
        got = res[:2 * n2].reshape(n2, 2)
        e_mom = _rel(got[inner], expect[inner], scale)
        e_div = float(np.max(np.abs(res[2 * n2:]))) / scale
        assert e_mom <= tol, (name, e_mom)
        assert e_div <= tol, (name, e_div)
        # the forced cases really are forced (the check is not vacuous)
        if name in ("shear", "stagnation", "pressure"):
            assert np.max(np.abs(expect[inner])) > 1e-3 * scale
        out[name] = max(e_mom, e_div)
    return out


def check_jacobian_identities(assemble, tol, nu=0.02):
    """Identities of the Newton Jacobian:
    * at a constant velocity, J [c, 0] = 0 on every row (the diffusion block
      annihilates constants; convection and reaction vanish for grad u = 0);
    * the continuity rows annihilate a divergence-free quadratic field;
    * the pressure-gradient block equals the transpose of the divergence
      block (with the continuity row written as -div u both are
      -int psi_b d_c phi_a); the pressure-pressure block is zero;
    * at u = 0 the velocity block is nu times one symmetric stiffness
      matrix on each component, with no coupling between components."""
    cp2, conn6, nv, nd = mesh(6, jitter_seed=4)
    n2 = cp2.shape[0]
    rng = np.random.default_rng(5)
    # constant velocity, random pressure
    state = np.concatenate([np.tile([0.7, -0.4], n2), rng.standard_normal(nv)])
    _, jac = assemble(cp2, conn6, nd, nu, state)
    c = np.concatenate([np.tile([1.3, -2.1], n2), np.zeros(nv)])
    scale = float(np.max(np.abs(jac) @ np.abs(c)))
    e_const = float(np.max(np.abs(jac @ c))) / scale
    assert e_const <= tol, e_const

    # divergence-free quadratic field through the continuity rows
    u = X.divergence_free_quadratic(cp2)
    jpu = jac[2 * n2:, :2 * n2]
    e_div = float(np.max(np.abs(jpu @ u)) / np.max(np.abs(jpu) @ np.abs(u)))
    assert e_div <= tol, e_div

    jup = jac[:2 * n2, 2 * n2:]
    e_bt = _rel(jup, jpu.T)
    assert e_bt <= tol, e_bt
    assert np.all(jac[2 * n2:, 2 * n2:] == 0.0)

    # u = 0: nu K on each component
    state0 = np.concatenate([np.zeros(2 * n2), rng.standard_normal(nv)])
    _, j0 = assemble(cp2, conn6, nd, nu, state0)
    juu = j0[:2 * n2, :2 * n2]
    kx, ky = juu[0::2, 0::2], juu[1::2, 1::2]
    e_sym = _rel(kx, kx.T)
    assert e_sym <= tol, e_sym
    assert _rel(kx, ky) <= tol
    assert np.max(np.abs(juu[0::2, 1::2])) <= tol * np.max(np.abs(kx))
    # linear in nu
    _, j1 = assemble(cp2, conn6, nd, 2.0 * nu, state0)
    assert _rel(j1[:2 * n2, :2 * n2], 2.0 * juu) <= tol
    return {"constant_velocity": e_const, "divergence_free": e_div, "transpose": e_bt,
            "symmetry": e_sym}
