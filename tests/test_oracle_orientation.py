"""The oracle on clockwise elements: reversing an element's local vertex
order (det J < 0) describes the same element, so the assembled global
system must not change (femx integrates with |det J|). Pins the oracle that
the GPU orientation tests compare against, independently of the kernels.
Tolerance: 1e-13 relative (the rounding of reordered sums)."""
import numpy as np

import th_exact as X
from conftest import rel_inf
from femx_gb300 import meshes
from oracle import pyoracle as orc


def test_taylor_hood_system_is_orientation_free():
    c3, k3 = meshes.jittered_tri(8, seed=41)
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    state = meshes.cavity_state(cp2, nv, seed=41)
    om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    r0, v0 = orc.assemble_th_ns(om, cp2, conn6, 1e-2, state)
    # v0 v1 v2 m01 m12 m20 -> v0 v2 v1 m20 m12 m01 on every other element
    flipped = conn6.copy()
    flipped[1::2] = conn6[1::2][:, [0, 2, 1, 5, 4, 3]]
    offs1, dofs1, _ = meshes.th_elem_dofs(flipped, cp2.shape[0])
    om1 = orc.AssemblyMap(nd, nd, offs1, dofs1, offs1, dofs1)
    r1, v1 = orc.assemble_th_ns(om1, cp2, flipped, 1e-2, state)
    assert np.array_equal(om.row_ptr, om1.row_ptr) and np.array_equal(om.col_ind, om1.col_ind)
    assert rel_inf(r1, r0) <= 1e-13
    assert rel_inf(X.dense(om1.row_ptr, om1.col_ind, v1, nd),
                   X.dense(om.row_ptr, om.col_ind, v0, nd)) <= 1e-13


def test_p1_system_is_orientation_free():
    coords, conn = meshes.jittered_tri(12, seed=42)
    n, e = coords.shape[0], conn.shape[0]
    rng = np.random.default_rng(42)
    kappa = np.exp(rng.standard_normal(e))
    f = meshes.fourier_source(coords, 1)
    u = rng.standard_normal(n)
    offs, dofs = meshes.scalar_elem_dofs(conn)
    om = orc.AssemblyMap(n, n, offs, dofs, offs, dofs)
    r0, v0 = orc.assemble_p1_kappa(om, orc.P1Quad(coords, conn), kappa, f, u)
    flipped = conn.copy()
    flipped[1::2] = conn[1::2][:, [0, 2, 1]]
    offs1, dofs1 = meshes.scalar_elem_dofs(flipped)
    om1 = orc.AssemblyMap(n, n, offs1, dofs1, offs1, dofs1)
    r1, v1 = orc.assemble_p1_kappa(om1, orc.P1Quad(coords, flipped), kappa, f, u)
    assert np.array_equal(om.row_ptr, om1.row_ptr) and np.array_equal(om.col_ind, om1.col_ind)
    assert rel_inf(r1, r0) <= 1e-13
    assert rel_inf(v1, v0) <= 1e-13
