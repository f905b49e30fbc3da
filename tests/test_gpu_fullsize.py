"""Full-size checks (the benchmark configurations) through size-independent
properties, where the oracle would be slow:

* P1 Poisson 1024x1024 with a log-normal GRF kappa: pattern bit-exact against
  the oracle's AssemblyMap; the stiffness annihilates constants and is
  symmetric; the residual is affine in u (R(u) - R(0) = K u); the lifted
  system keeps identity rows and zero columns at the constraints;
* SpMV linearity at that size;
* Taylor-Hood 256x256 cavity: the Newton Jacobian against central
  differences of the residual along seeded directions (FP64), and the
  FP32-quadrature Jacobian against the FP64 one;

and directly against the oracle at the full sizes:

* Taylor-Hood 256x256 (benchmark cavity): pattern bit-exact; Jacobian and
  residual, before and after the Dirichlet rows, in FP64 (1e-12, atomic and
  deterministic), MIXED (J 1e-6, R 1e-12) and FP32 quadrature (1e-6);
* P1 Poisson 1024x1024: FP64 assembly, lifting and a product (1e-12 /
  1e-13; lifted constraint rows, columns and rhs entries exact).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from femx_gb300 import assembly as A  # noqa: E402
from femx_gb300 import meshes  # noqa: E402
from oracle import pyoracle as orc  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from femx_gb300 import build
    build.build()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def amax(t):
    return float(t.abs().max())


@pytest.fixture(scope="module")
def poisson1024():
    coords, conn = meshes.structured_tri(1024)
    n, e = coords.shape[0], conn.shape[0]
    kappa = np.exp(meshes.grf_centroids(coords, conn, seed=2, ell=0.05, var=1.0, grid=1024))
    offs, dofs = meshes.scalar_elem_dofs(conn)
    amap = A.makeAssemblyMap(n, n, dev(offs), dev(dofs), dev(offs), dev(dofs))
    return dict(coords=coords, conn=conn, n=n, e=e, kappa=kappa, offs=offs, dofs=dofs,
                amap=amap)


def test_poisson_1024_pattern_is_bit_exact(poisson1024):
    p = poisson1024
    om = orc.AssemblyMap(p["n"], p["n"], p["offs"], p["dofs"], p["offs"], p["dofs"])
    pat = p["amap"].pattern()
    assert pat.nnz == 7346177
    assert np.array_equal(pat.row_ptr.cpu().numpy(), om.row_ptr)
    assert np.array_equal(pat.col_ind.cpu().numpy(), om.col_ind)
    assert np.array_equal(p["amap"].view()["jac_map"].cpu().numpy(), om.jac_map)


def test_poisson_1024_operator_properties(poisson1024):
    p = poisson1024
    n, amap = p["n"], p["amap"]
    coords, kappa = dev(p["coords"]), dev(p["kappa"])
    rng = np.random.default_rng(5)
    u = dev(rng.standard_normal(n))
    jac = A.CsrMatrix(amap.pattern())
    r_u = torch.zeros(n, dtype=torch.float64, device="cuda")
    r_0 = torch.zeros(n, dtype=torch.float64, device="cuda")
    A.assembleP1Kappa(amap, coords, kappa, None, u, r_u, jac)
    A.assembleP1Kappa(amap, coords, kappa, None, torch.zeros_like(u), r_0)
    amap.check()
    kmax = amax(jac.vals)
    one = torch.ones(n, dtype=torch.float64, device="cuda")
    k1 = torch.zeros(n, dtype=torch.float64, device="cuda")
    A.matvec(jac, one, k1)
    assert amax(k1) <= 1e-12 * kmax                       # K 1 = 0
    kt = A.transpose(jac)
    assert torch.equal(kt.pattern.row_ptr, jac.pattern.row_ptr)
    assert torch.equal(kt.pattern.col_ind, jac.pattern.col_ind)
    assert amax(kt.vals - jac.vals) <= 1e-13 * kmax       # symmetric
    ku = torch.zeros(n, dtype=torch.float64, device="cuda")
    A.matvec(jac, u, ku)
    assert amax(r_u - r_0 - ku) <= 1e-12 * amax(ku)       # affine in u


def test_poisson_1024_lifting_structure(poisson1024):
    p = poisson1024
    n, amap = p["n"], p["amap"]
    bdofs = meshes.dirichlet_dofs(p["coords"], meshes.boundary_nodes(p["coords"]))
    bc = A.makeBoundaryMap(dev(bdofs), amap.pattern())
    jac = A.CsrMatrix(amap.pattern())
    res = torch.zeros(n, dtype=torch.float64, device="cuda")
    A.assembleP1Kappa(amap, dev(p["coords"]), dev(p["kappa"]), None,
                      torch.zeros(n, dtype=torch.float64, device="cuda"), res, jac)
    g = dev(np.random.default_rng(6).standard_normal(len(bdofs)))
    rhs = -res
    A.prepareForwardSolve(bc, jac, rhs, g)
    rp = amap.pattern().row_ptr.cpu().numpy()
    ci = amap.pattern().col_ind.cpu().numpy()
    v = jac.vals.cpu().numpy()
    is_bc = np.zeros(n, dtype=bool)
    is_bc[bdofs] = True
    rows = np.repeat(np.arange(n), np.diff(rp))
    on_bc_row, on_bc_col = is_bc[rows], is_bc[ci]
    diag = rows == ci
    assert np.all(v[on_bc_row & diag] == 1.0) and np.all(v[on_bc_row & ~diag] == 0.0)
    assert np.all(v[on_bc_col & ~on_bc_row] == 0.0)
    assert np.array_equal(rhs.cpu().numpy()[bdofs], g.cpu().numpy())


def test_spmv_linearity_at_1024(poisson1024):
    p = poisson1024
    n, amap = p["n"], p["amap"]
    jac = A.CsrMatrix(amap.pattern())
    res = torch.zeros(n, dtype=torch.float64, device="cuda")
    A.assembleP1Kappa(amap, dev(p["coords"]), dev(p["kappa"]), None,
                      torch.zeros(n, dtype=torch.float64, device="cuda"), res, jac)
    rng = np.random.default_rng(7)
    x, y = dev(rng.standard_normal(n)), dev(rng.standard_normal(n))
    ax, ay, axy = (torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3))
    A.matvec(jac, x, ax)
    A.matvec(jac, y, ay)
    A.matvec(jac, 2.0 * x - 3.0 * y, axy)
    assert amax(axy - (2.0 * ax - 3.0 * ay)) <= 1e-12 * amax(axy)


def test_taylor_hood_256_jacobian_is_the_derivative():
    c3, k3 = meshes.structured_tri(256)
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    amap = A.makeAssemblyMap(nd, nd, dev(offs), dev(dofs), dev(offs), dev(dofs))
    coords, c6 = dev(cp2), dev(conn6.astype(np.int32))
    u0 = dev(meshes.cavity_state(cp2, nv, seed=3))
    jac = A.CsrMatrix(amap.pattern())
    r = torch.zeros(nd, dtype=torch.float64, device="cuda")
    A.assembleTaylorHood(amap, coords, c6, 1e-3, u0, r, jac, precision="fp64")
    j64 = jac.vals.clone()
    A.assembleTaylorHood(amap, coords, c6, 1e-3, u0, r, jac, precision="fp32_quad")
    assert amax(jac.vals - j64) <= 1e-6 * amax(j64)
    jac.vals.copy_(j64)
    rng = np.random.default_rng(8)
    # the steady NS residual is quadratic in the state: central differences
    # are exact up to rounding for any step, so a large one keeps rounding low
    h = 1e-3
    for _ in range(3):
        v = dev(rng.standard_normal(nd))
        v /= float(v.norm())
        rp = torch.zeros(nd, dtype=torch.float64, device="cuda")
        rm = torch.zeros(nd, dtype=torch.float64, device="cuda")
        A.assembleTaylorHood(amap, coords, c6, 1e-3, u0 + h * v, rp, None, precision="fp64")
        A.assembleTaylorHood(amap, coords, c6, 1e-3, u0 - h * v, rm, None, precision="fp64")
        fd = (rp - rm) / (2 * h)
        jv = torch.zeros(nd, dtype=torch.float64, device="cuda")
        A.matvec(jac, v, jv)
        assert amax(jv - fd) <= 1e-6 * amax(jv)
    amap.check()


# ------------------------------------------------ full size against the oracle

@pytest.fixture(scope="module")
def cavity256():
    c3, k3 = meshes.structured_tri(256)
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    state = meshes.cavity_state(cp2, nv, seed=3)
    th = orc.THQuad(cp2, conn6)
    rres, rvals = orc.assemble_th_threads(om, th, 1e-3, state, 8)
    bd, bv = meshes.cavity_dirichlet(cp2, cp2.shape[0])
    ob = orc.BoundaryMap(bd, om.row_ptr, om.col_ind)
    amap = A.makeAssemblyMap(nd, nd, dev(offs), dev(dofs), dev(offs), dev(dofs))
    return dict(cp2=cp2, conn6=conn6, nd=nd, om=om, state=state, rres=rres, rvals=rvals,
                bd=bd, bv=bv, ob=ob, amap=amap)


def rel_inf(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_taylor_hood_256_pattern_is_bit_exact(cavity256):
    c = cavity256
    pat = c["amap"].pattern()
    assert np.array_equal(pat.row_ptr.cpu().numpy(), c["om"].row_ptr)
    assert np.array_equal(pat.col_ind.cpu().numpy(), c["om"].col_ind)
    assert np.array_equal(c["amap"].view()["jac_map"].cpu().numpy(), c["om"].jac_map)


@pytest.mark.parametrize("precision,det,tol_j,tol_r", [
    ("fp64", False, 1e-12, 1e-12), ("fp64", True, 1e-12, 1e-12),
    ("double_float", False, 1e-12, 1e-12),
    ("mixed", False, 1e-6, 1e-12), ("fp32_quad", False, 1e-6, 1e-6)])
def test_taylor_hood_256_matches_oracle(cavity256, precision, det, tol_j, tol_r):
    """The benchmark's cavity (256x256, Re = 1000, seeded stream-function
    state): Jacobian and residual against the oracle, then the Dirichlet rows
    (replaceRes with the state, replaceRows with 1 on the diagonal) against
    the oracle's, as the Newton step applies them."""
    c = cavity256
    nd, amap = c["nd"], c["amap"]
    st = dev(c["state"])
    res = torch.zeros(nd, dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(amap.pattern())
    A.assembleTaylorHood(amap, dev(c["cp2"]), dev(c["conn6"].astype(np.int32)), 1e-3, st,
                         res, jac, precision=precision, deterministic=det)
    amap.check()
    assert rel_inf(jac.vals.cpu().numpy(), c["rvals"]) <= tol_j
    assert rel_inf(res.cpu().numpy(), c["rres"]) <= tol_r
    bc = A.makeBoundaryMap(dev(c["bd"]), amap.pattern())
    A.replaceRes(bc, st, dev(c["bv"]), res)
    A.replaceRows(bc, jac, 1.0)
    rr = c["ob"].replace_res(c["state"], c["bv"], c["rres"])
    rv = c["ob"].replace_rows(c["rvals"], 1.0)
    assert rel_inf(jac.vals.cpu().numpy(), rv) <= tol_j
    assert rel_inf(res.cpu().numpy(), rr) <= tol_r
    # the constrained rows themselves are exact
    assert np.array_equal(res.cpu().numpy()[c["bd"]], rr[c["bd"]])


def test_poisson_1024_matches_oracle_after_lifting(poisson1024):
    """The Poisson benchmark step at full size (1024x1024, GRF kappa, Fourier
    source): FP64 assembly, prepareForwardSolve and one product against the
    oracle's, values to 1e-12, the lifted constraint rows and rhs exact."""
    p = poisson1024
    n, amap = p["n"], p["amap"]
    f = meshes.fourier_source(p["coords"], 1)
    u = np.zeros(n)
    om = orc.AssemblyMap(n, n, p["offs"], p["dofs"], p["offs"], p["dofs"])
    q = orc.P1Quad(p["coords"], p["conn"])
    rres, rvals = orc.assemble_p1_kappa(om, q, p["kappa"], f, u)
    bdofs = meshes.dirichlet_dofs(p["coords"], meshes.boundary_nodes(p["coords"]))
    g = np.random.default_rng(6).standard_normal(len(bdofs))
    ev, er = orc.BoundaryMap(bdofs, om.row_ptr, om.col_ind).prepare_forward_solve(rvals, -rres, g)

    res = torch.zeros(n, dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(amap.pattern())
    # the double-float (FP64-accurate) assembly meets the same gate
    A.assembleP1Kappa(amap, dev(p["coords"]), dev(p["kappa"]), dev(f), dev(u), res, jac,
                      precision="double_float")
    assert rel_inf(jac.vals.cpu().numpy(), rvals) <= 1e-12
    assert rel_inf(res.cpu().numpy(), rres) <= 1e-12
    A.assembleP1Kappa(amap, dev(p["coords"]), dev(p["kappa"]), dev(f), dev(u), res, jac)
    amap.check()
    assert rel_inf(jac.vals.cpu().numpy(), rvals) <= 1e-12
    assert rel_inf(res.cpu().numpy(), rres) <= 1e-12
    bc = A.makeBoundaryMap(dev(bdofs), amap.pattern())
    rhs = -res
    A.prepareForwardSolve(bc, jac, rhs, dev(g))
    v, r = jac.vals.cpu().numpy(), rhs.cpu().numpy()
    assert rel_inf(v, ev) <= 1e-12
    assert rel_inf(r, er) <= 1e-12
    is_bc = np.zeros(n, dtype=bool)
    is_bc[bdofs] = True
    rows = np.repeat(np.arange(n), np.diff(om.row_ptr))
    touched = is_bc[rows] | is_bc[om.col_ind]
    assert np.array_equal(v[touched], ev[touched])
    assert np.array_equal(r[bdofs], er[bdofs])
    x = np.random.default_rng(9).standard_normal(n)
    y = torch.zeros(n, dtype=torch.float64, device="cuda")
    A.matvec(jac, dev(x), y)
    assert rel_inf(y.cpu().numpy(), orc.matvec(om.row_ptr, om.col_ind, v, x)) <= 1e-13
