"""Clockwise elements. Every generated mesh is counter-clockwise, so here
every other element of a jittered mesh has its local vertex order reversed
(det J < 0): femx integrates with |det J| (ElementValues::calcPhysicalValues),
and every kernel must give the oracle's values on such a mesh — the
thread-per-element FP64 and double-float Taylor-Hood kernels (|det| J^-1 =
sign(det) adj J), the 16-lane FP32 kernel, the state VJP, and the P1 kernels
including the owner-computes tiles.

Gates: FP64 and double-float 1e-12, FP32 quadrature 1e-6 (relative, inf
norm)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from conftest import rel_inf  # noqa: E402
from femx_gb300 import assembly as A  # noqa: E402
from femx_gb300 import meshes  # noqa: E402
from oracle import pyoracle as orc  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from femx_gb300 import build
    build.build()


def dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    return (t if dtype is None else t.to(dtype)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def flipped_mesh(nx, seed):
    """A jittered mesh with every other triangle clockwise."""
    coords, conn = meshes.jittered_tri(nx, seed=seed)
    conn = conn.copy()
    conn[1::2, [1, 2]] = conn[1::2, [2, 1]]
    return coords, conn


def signed_areas(coords, conn):
    p0, p1, p2 = coords[conn[:, 0]], coords[conn[:, 1]], coords[conn[:, 2]]
    return (p1[:, 0] - p0[:, 0]) * (p2[:, 1] - p0[:, 1]) - (p2[:, 0] - p0[:, 0]) * (
        p1[:, 1] - p0[:, 1])


TOL = {"fp64": 1e-12, "double_float": 1e-12, "fp32_quad": 1e-6, "mixed": 1e-6}


@pytest.mark.parametrize("precision", ["fp64", "double_float", "fp32_quad", "mixed"])
def test_taylor_hood_on_clockwise_elements(precision):
    c3, k3 = flipped_mesh(10, seed=31)
    det = signed_areas(c3, k3)
    assert (det < 0).sum() == det.size // 2 and (det > 0).sum() == det.size - det.size // 2
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    state = meshes.cavity_state(cp2, nv, seed=31)
    om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    rres, rvals = orc.assemble_th_ns(om, cp2, conn6, 1e-2, state)
    m = A.makeAssemblyMap(nd, nd, dev(offs, torch.int32), dev(dofs, torch.int32),
                          dev(offs, torch.int32), dev(dofs, torch.int32))
    res = torch.zeros(nd, dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(m.pattern())
    A.assembleTaylorHood(m, dev(cp2), dev(conn6, torch.int32), 1e-2, dev(state), res, jac,
                         precision=precision)
    m.check()
    tol_r = 1e-12 if precision == "mixed" else TOL[precision]
    assert rel_inf(host(jac.vals), rvals) <= TOL[precision]
    assert rel_inf(host(res), rres) <= tol_r
    if precision != "mixed":
        lam = np.random.default_rng(31).standard_normal(nd)
        gref = orc.matvec_t(om.row_ptr, om.col_ind, rvals, lam, nd)
        g = torch.zeros(nd, dtype=torch.float64, device="cuda")
        A.vjpTaylorHood(m, dev(cp2), dev(conn6, torch.int32), 1e-2, dev(state), dev(lam), g,
                        precision=precision)
        m.check()
        assert rel_inf(host(g), gref) <= TOL[precision]


@pytest.mark.parametrize("precision,tiled", [("fp64", False), ("double_float", False),
                                             ("fp32_quad", False), ("double_float", True),
                                             ("fp64", True)])
def test_p1_on_clockwise_elements(precision, tiled):
    coords, conn = flipped_mesh(20, seed=32)
    n, e = coords.shape[0], conn.shape[0]
    rng = np.random.default_rng(32)
    kappa = np.exp(rng.standard_normal(e))
    f = meshes.fourier_source(coords, 1)
    u = rng.standard_normal(n)
    offs, dofs = meshes.scalar_elem_dofs(conn)
    om = orc.AssemblyMap(n, n, offs, dofs, offs, dofs)
    rres, rvals = orc.assemble_p1_kappa(om, orc.P1Quad(coords, conn), kappa, f, u)
    m = A.makeAssemblyMap(n, n, dev(offs), dev(dofs), dev(offs), dev(dofs))
    if tiled:
        m.enableTiles(dev(coords))
    res = torch.zeros(n, dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(m.pattern())
    A.assembleP1Kappa(m, dev(coords), dev(kappa), dev(f), dev(u), res, jac,
                      precision=precision, tiled=tiled)
    m.check()
    assert rel_inf(host(jac.vals), rvals) <= TOL[precision]
    assert rel_inf(host(res), rres) <= TOL[precision]


@pytest.mark.parametrize("precision", ["fp64", "double_float", "fp32_quad"])
def test_translated_and_scaled_mesh(precision):
    """Coordinates far from the origin (offset 1e3, element size 1e-4): the
    edges are formed by FP64 subtraction before any conversion, so every
    precision keeps its gate; the double-float state is scaled by 1e6 as
    well (relative accuracy)."""
    c3, k3 = meshes.jittered_tri(8, seed=33)
    c3 = c3 * 8e-4 + np.array([1.0e3, -2.5e2])
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    state = 1.0e6 * np.random.default_rng(33).standard_normal(nd)
    om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    rres, rvals = orc.assemble_th_ns(om, cp2, conn6, 1e-2, state)
    m = A.makeAssemblyMap(nd, nd, dev(offs, torch.int32), dev(dofs, torch.int32),
                          dev(offs, torch.int32), dev(dofs, torch.int32))
    res = torch.zeros(nd, dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(m.pattern())
    A.assembleTaylorHood(m, dev(cp2), dev(conn6, torch.int32), 1e-2, dev(state), res, jac,
                         precision=precision)
    m.check()
    assert rel_inf(host(jac.vals), rvals) <= TOL[precision]
    assert rel_inf(host(res), rres) <= TOL[precision]

    coords, conn = meshes.jittered_tri(16, seed=34)
    coords = coords * 1e-3 + np.array([-7.0e2, 3.0e3])
    n, e = coords.shape[0], conn.shape[0]
    rng = np.random.default_rng(34)
    kappa = np.exp(rng.standard_normal(e))
    f = meshes.fourier_source(coords, 1)
    u = 1.0e6 * rng.standard_normal(n)
    offs1, dofs1 = meshes.scalar_elem_dofs(conn)
    om1 = orc.AssemblyMap(n, n, offs1, dofs1, offs1, dofs1)
    rr1, rv1 = orc.assemble_p1_kappa(om1, orc.P1Quad(coords, conn), kappa, f, u)
    m1 = A.makeAssemblyMap(n, n, dev(offs1), dev(dofs1), dev(offs1), dev(dofs1))
    m1.enableTiles(dev(coords))
    for tiled in (False, True):
        r1 = torch.zeros(n, dtype=torch.float64, device="cuda")
        j1 = A.CsrMatrix(m1.pattern())
        A.assembleP1Kappa(m1, dev(coords), dev(kappa), dev(f), dev(u), r1, j1,
                          precision=precision, tiled=tiled)
        m1.check()
        assert rel_inf(host(j1.vals), rv1) <= TOL[precision]
        assert rel_inf(host(r1), rr1) <= TOL[precision]
