"""Exact Taylor-Hood P2/P1 Navier-Stokes element integrals, written from the
weak form alone — an independent pin of the operator's physics.

The steady Galerkin Navier-Stokes residual that femx's MixedFESpace layout
carries (velocity comps 2 first, dof = 2 node + comp; pressure after), for a
momentum row (node a, component c) and a continuity row (vertex b):

    R_(a,c) = int nu grad(u_c).grad(phi_a) + (u.grad u_c) phi_a - p d_c phi_a
    R_b     = - int psi_b div u

Its Newton Jacobian adds, for column (node b, component e),
nu delta_ce grad phi_b.grad phi_a + delta_ce (u.grad phi_b) phi_a
+ phi_b (d_e u_c) phi_a, and -int psi_b d_c phi_a in the two pressure blocks.

This module evaluates those integrals EXACTLY for states that interpolate a
LINEAR velocity and a LINEAR pressure (every integrand is then a polynomial of
degree <= 4 in the barycentric coordinates, integrated in closed form by
int_T l0^i l1^j l2^k = 2|T| i! j! k! / (i+j+k+2)!). It shares no code and no
quadrature rule with the library or the oracle: a sign, factor or index error
in any term of either shows up as a mismatch. The quadrature rule the library
uses (degree 4) integrates these polynomials exactly too, so the two agree to
rounding.

It also gives the P2 mass matrix and int phi_a, used by the patch tests with
quadratic exact solutions (Poiseuille, Couette, shear), where the terms the
degree-4 rule would not integrate exactly vanish pointwise.

P2 basis on the reference triangle, as the element uses it: vertices 0,1,2
(l0 = 1 - r - s, l1 = r, l2 = s), phi_v = l_v (2 l_v - 1); edge nodes
3 = (0,1), 4 = (1,2), 5 = (2,0), phi = 4 l_i l_j.
"""
from __future__ import annotations

from math import factorial

import numpy as np

EDGES = ((0, 1), (1, 2), (2, 0))


# ------------------------------------------------------------- polynomials
# A polynomial in (l0, l1, l2) is a dict {(i, j, k): coefficient}.

def _mono(i, j, k, c=1.0):
    return {(i, j, k): c}


def _add(*ps):
    out = {}
    for p in ps:
        for e, c in p.items():
            out[e] = out.get(e, 0.0) + c
    return out


def _scale(p, s):
    return {e: c * s for e, c in p.items()}


def _mul(p, q):
    out = {}
    for e1, c1 in p.items():
        for e2, c2 in q.items():
            e = (e1[0] + e2[0], e1[1] + e2[1], e1[2] + e2[2])
            out[e] = out.get(e, 0.0) + c1 * c2
    return out


def _d(p, l):
    """Partial derivative in l_l, the l's taken as independent variables
    (chain rule: grad f = sum_l df/dl_l grad l_l)."""
    out = {}
    for e, c in p.items():
        if e[l] > 0:
            ne = list(e)
            ne[l] -= 1
            out[tuple(ne)] = out.get(tuple(ne), 0.0) + c * e[l]
    return out


def _int_ref(p):
    """int over T of p, divided by |T|."""
    tot = 0.0
    for (i, j, k), c in p.items():
        tot += c * 2.0 * factorial(i) * factorial(j) * factorial(k) / factorial(i + j + k + 2)
    return tot


def _lam(v):
    e = [0, 0, 0]
    e[v] = 1
    return _mono(*e)


PHI = [_add(_scale(_mul(_lam(v), _lam(v)), 2.0), _scale(_lam(v), -1.0)) for v in range(3)] + \
      [_scale(_mul(_lam(i), _lam(j)), 4.0) for i, j in EDGES]
PSI = [_lam(v) for v in range(3)]

# Reference tensors (each divided by |T|).
# MASS[a,b]        = int phi_a phi_b
# LOAD[a]          = int phi_a
# STIFF[a,b,l,m]   = int dphi_a/dl_l dphi_b/dl_m
# CONV[a,b,m,k]    = int l_k dphi_b/dl_m phi_a
# PGRAD[b,a,l]     = int psi_b dphi_a/dl_l
MASS = np.array([[_int_ref(_mul(PHI[a], PHI[b])) for b in range(6)] for a in range(6)])
LOAD = np.array([_int_ref(PHI[a]) for a in range(6)])
STIFF = np.array([[[[_int_ref(_mul(_d(PHI[a], l), _d(PHI[b], m))) for m in range(3)]
                    for l in range(3)] for b in range(6)] for a in range(6)])
CONV = np.array([[[[_int_ref(_mul(_mul(_lam(k), _d(PHI[b], m)), PHI[a])) for k in range(3)]
                   for m in range(3)] for b in range(6)] for a in range(6)])
PGRAD = np.array([[[_int_ref(_mul(PSI[b], _d(PHI[a], l))) for l in range(3)]
                   for a in range(6)] for b in range(3)])


def _geometry(xv):
    """|T| and the gradients of l0, l1, l2 (rows) of a triangle (3x2)."""
    jm = np.array([[xv[1, 0] - xv[0, 0], xv[2, 0] - xv[0, 0]],
                   [xv[1, 1] - xv[0, 1], xv[2, 1] - xv[0, 1]]])
    det = np.linalg.det(jm)
    inv = np.linalg.inv(jm)  # rows: grad r, grad s
    g = np.empty((3, 2))
    g[1], g[2] = inv[0], inv[1]
    g[0] = -g[1] - g[2]
    return abs(det) / 2.0, g


# ------------------------------------------------------------- assembly

def element_dofs(conn6, num_p2_nodes):
    """15 local DOFs in MixedFESpace order: (2 node + comp) for the six
    nodes, then 2 num_p2_nodes + vertex for the three pressure vertices."""
    d = np.empty(15, dtype=np.int64)
    d[0:12:2] = 2 * conn6
    d[1:12:2] = 2 * conn6 + 1
    d[12:15] = 2 * num_p2_nodes + conn6[:3]
    return d


def linear_state(coords_p2, num_vertices, vel_coef, p_coef):
    """Interpolant of u_c = v[c,0] + v[c,1] x + v[c,2] y and
    p = q[0] + q[1] x + q[2] y in the Taylor-Hood DOF order."""
    v = np.asarray(vel_coef, dtype=np.float64)
    q = np.asarray(p_coef, dtype=np.float64)
    x, y = coords_p2[:, 0], coords_p2[:, 1]
    vel = np.stack([v[c, 0] + v[c, 1] * x + v[c, 2] * y for c in range(2)], axis=1)
    p = q[0] + q[1] * x[:num_vertices] + q[2] * y[:num_vertices]
    return np.concatenate([vel.reshape(-1), p])


def exact_linear_system(coords_p2, conn6, num_p2_nodes, num_dofs, nu, state):
    """Residual and dense Jacobian, integrated exactly, for a state that
    interpolates linear velocity and pressure fields (linear_state)."""
    res = np.zeros(num_dofs)
    jac = np.zeros((num_dofs, num_dofs))
    for e in range(conn6.shape[0]):
        nodes = conn6[e]
        area, g = _geometry(coords_p2[nodes[:3]])
        dofs = element_dofs(nodes, num_p2_nodes)
        st = state[dofs]
        uv = st[0:12].reshape(6, 2)[:3]  # vertex velocities (the field is linear)
        pv = st[12:15]
        gg = g @ g.T                                         # grad l_l . grad l_m
        grad_u = uv.T @ g                                    # [c, d] = d_d u_c (constant)
        kel = np.einsum("ablm,lm->ab", STIFF, gg) * area     # int grad phi_a . grad phi_b
        # int (u . grad phi_b) phi_a = sum_k sum_m (u(vertex k) . grad l_m) CONV[a,b,m,k]
        ug = uv @ g.T                                        # [k, m] = u(k) . grad l_m
        cel = np.einsum("abmk,km->ab", CONV, ug) * area
        mel = MASS * area
        # int psi_b d_c phi_a = sum_l (grad l_l)_c PGRAD[b,a,l]
        bel = np.einsum("bal,lc->bac", PGRAD, g) * area      # [b, a, c]
        je = np.zeros((15, 15))
        for a in range(6):
            for c in range(2):
                row = 2 * a + c
                for b in range(6):
                    for ec in range(2):
                        v = mel[a, b] * grad_u[c, ec]
                        if ec == c:
                            v += nu * kel[a, b] + cel[a, b]
                        je[row, 2 * b + ec] = v
                for b in range(3):
                    je[row, 12 + b] = -bel[b, a, c]
        for b in range(3):
            for a in range(6):
                for ec in range(2):
                    je[12 + b, 2 * a + ec] = -bel[b, a, ec]
        # residual: momentum rows are linear in u_c for a frozen advecting u,
        # so R = (nu K + C) U_c - B^T p; continuity R = -B U
        re = np.zeros(15)
        uall = st[0:12].reshape(6, 2)
        for a in range(6):
            for c in range(2):
                re[2 * a + c] = (nu * kel[a] + cel[a]) @ uall[:, c] - bel[:, a, c] @ pv
        for b in range(3):
            re[12 + b] = -np.sum(bel[b] * uall)
        res[dofs] += re
        jac[np.ix_(dofs, dofs)] += je
    return res, jac


def load_vector(coords_p2, conn6, num_p2_nodes):
    """int phi_a over the mesh, per P2 node."""
    out = np.zeros(num_p2_nodes)
    for e in range(conn6.shape[0]):
        area, _ = _geometry(coords_p2[conn6[e, :3]])
        out[conn6[e]] += LOAD * area
    return out


def mass_apply(coords_p2, conn6, num_p2_nodes, f):
    """(M f)_a = sum_b int phi_a phi_b f_b for nodal values f (P2 nodes)."""
    out = np.zeros(num_p2_nodes)
    for e in range(conn6.shape[0]):
        area, _ = _geometry(coords_p2[conn6[e, :3]])
        out[conn6[e]] += (MASS * area) @ f[conn6[e]]
    return out


def dense(row_ptr, col_ind, vals, n):
    out = np.zeros((n, n))
    for r in range(n):
        out[r, col_ind[row_ptr[r]:row_ptr[r + 1]]] += vals[row_ptr[r]:row_ptr[r + 1]]
    return out


def interior_velocity_rows(coords_p2, tol=1e-12):
    x, y = coords_p2[:, 0], coords_p2[:, 1]
    inner = (x > tol) & (x < 1 - tol) & (y > tol) & (y < 1 - tol)
    nodes = np.nonzero(inner)[0]
    return nodes


# ------------------------------------------------------------- patch cases
# Exact steady solutions (or known forcing) of -nu lap u + (u.grad)u + grad p,
# div u = 0 on the unit square, with quadratic velocity and linear pressure.
# For each: the velocity and pressure fields, and the residual that interior
# momentum rows must carry, as (coefficient of int phi_a, mass-applied field)
# for each component: R_(a,c) = load[c] * int phi_a + (M f_c)_a.

def patch_cases(nu):
    return {
        # u = (y(1-y), 0), p = -2 nu x: exact, R = 0 in the interior
        "poiseuille": (lambda x, y: (y * (1 - y), 0 * x), lambda x, y: -2 * nu * x + 0.3,
                       (0.0, 0.0), None),
        # u = (y, 0), p = const: exact
        "couette": (lambda x, y: (y, 0 * x), lambda x, y: 0 * x + 0.7, (0.0, 0.0), None),
        # u = (y^2, 0), p = 0: -nu lap u = (-2 nu, 0), convection zero
        "shear": (lambda x, y: (y * y, 0 * x), lambda x, y: 0 * x, (-2.0 * nu, 0.0), None),
        # u = (x, -y), p = 0: (u.grad)u = (x, y), lap u = 0
        "stagnation": (lambda x, y: (x, -y), lambda x, y: 0 * x, (0.0, 0.0),
                       lambda x, y: (x, y)),
        # u = 0, p = 0.4 x - 1.3 y: grad p = (0.4, -1.3)
        "pressure": (lambda x, y: (0 * x, 0 * x), lambda x, y: 0.4 * x - 1.3 * y,
                     (0.4, -1.3), None),
    }


def patch_state(coords_p2, num_vertices, vel, pres):
    x, y = coords_p2[:, 0], coords_p2[:, 1]
    ux, uy = vel(x, y)
    p = pres(x[:num_vertices], y[:num_vertices])
    return np.concatenate([np.stack([ux, uy], axis=1).reshape(-1), p])


def patch_expected(coords_p2, conn6, num_p2_nodes, load, force):
    """Expected momentum residual per P2 node and component (interior rows)."""
    phi_int = load_vector(coords_p2, conn6, num_p2_nodes)
    out = np.stack([load[0] * phi_int, load[1] * phi_int], axis=1)
    if force is not None:
        fx, fy = force(coords_p2[:, 0], coords_p2[:, 1])
        out[:, 0] += mass_apply(coords_p2, conn6, num_p2_nodes, fx)
        out[:, 1] += mass_apply(coords_p2, conn6, num_p2_nodes, fy)
    return out


def divergence_free_quadratic(coords_p2):
    """u = (psi_y, -psi_x) of psi = x^3 + x^2 y - 2 x y^2 + y^3 (div u = 0)."""
    x, y = coords_p2[:, 0], coords_p2[:, 1]
    ux = x * x - 4 * x * y + 3 * y * y
    uy = -(3 * x * x + 2 * x * y - 2 * y * y)
    return np.stack([ux, uy], axis=1).reshape(-1)
