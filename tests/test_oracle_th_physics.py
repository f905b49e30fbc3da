"""The oracle's Taylor-Hood operator pinned by the weak form itself.

femx has no P2/P1 element, so the oracle's Taylor-Hood operator and the
library's are both written from the weak form; these tests pin it
independently of both: exact integrals for linear fields on jittered meshes
(every row of R and J), exact steady solutions and forced quadratic fields
(Poiseuille, Couette, shear, stagnation flow, a pressure gradient), and the
Jacobian's identities. Tolerances: 1e-12 (FP64, rounding only).
"""
import numpy as np

import th_checks as T
import th_exact as X
from femx_gb300 import meshes
from oracle import pyoracle as orc


def oracle_assemble(cp2, conn6, nd, nu, state):
    offs, dofs, _ = meshes.th_elem_dofs(conn6, cp2.shape[0])
    om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    res, vals = orc.assemble_th_ns(om, cp2, conn6, nu, state)
    return res, X.dense(om.row_ptr, om.col_ind, vals, nd)


def test_reference_tensors_are_consistent():
    # partition of unity and the closed forms of the P2 integrals
    assert np.allclose(X.MASS.sum(axis=1), X.LOAD)
    assert np.allclose(X.LOAD, [0, 0, 0, 1 / 3, 1 / 3, 1 / 3])
    assert np.allclose(X.MASS * 180, np.array([
        [6, -1, -1, 0, -4, 0], [-1, 6, -1, 0, 0, -4], [-1, -1, 6, -4, 0, 0],
        [0, 0, -4, 32, 16, 16], [-4, 0, 0, 16, 32, 16], [0, -4, 0, 16, 16, 32]]) / 180 * 180)


def test_oracle_matches_exact_integrals_for_linear_fields():
    T.check_linear_fields(oracle_assemble, 1e-12, 1e-12)


def test_oracle_patch_solutions():
    T.check_patch_solutions(oracle_assemble, 1e-12)


def test_oracle_jacobian_identities():
    T.check_jacobian_identities(oracle_assemble, 1e-12)


def test_exact_integrals_catch_a_sign_error():
    """The check is sharp: an operator with the convection sign flipped (the
    mistake is planted in the exact integrals, on the CPU) fails it."""
    cp2, conn6, nv, nd = T.mesh(4, jitter_seed=3)
    rng = np.random.default_rng(9)
    state = X.linear_state(cp2, nv, rng.standard_normal((2, 3)), rng.standard_normal(3))
    r_ex, _ = X.exact_linear_system(cp2, conn6, cp2.shape[0], nd, 0.01, state)
    saved = X.CONV.copy()
    try:
        X.CONV *= -1.0
        r_bad, _ = X.exact_linear_system(cp2, conn6, cp2.shape[0], nd, 0.01, state)
    finally:
        X.CONV[...] = saved
    res, _ = oracle_assemble(cp2, conn6, nd, 0.01, state)
    assert np.max(np.abs(res - r_ex)) <= 1e-12 * np.max(np.abs(r_ex))
    assert np.max(np.abs(res - r_bad)) > 1e-3 * np.max(np.abs(r_ex))
