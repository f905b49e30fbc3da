"""Tiled (owner-computes) P1 assembly: every CSR value and residual entry is
written once by the tile that owns its row, with no atomics and no zero
fill. Pinned against the oracle (femx's assemble with the kappa-weighted P1
operator, oracle/femx_oracle.cpp) on small structured and jittered, permuted
meshes, with and without a load and a separate geometry connectivity, at
the 1024x1024 benchmark size, and against the reference-built golden vector
of the 32x32 Poisson case; plus the integer-pipe double-float conversions
the FP64-accurate mode is built on, and the tile builder's refusals.

Tolerances (relative, infinity norm, against the oracle's FP64 values):
FP64 and double-float 1e-12 (the plain-FP64 gate), FP32 quadrature 1e-6."""
import ctypes as C
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from femx_gb300 import _lib  # noqa: E402
from femx_gb300 import assembly as A  # noqa: E402
from femx_gb300 import meshes  # noqa: E402
from oracle import pyoracle as orc  # noqa: E402

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL = {"fp64": 1e-12, "double_float": 1e-12, "fp32_quad": 1e-6}


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from femx_gb300 import build
    build.build()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def rel_inf(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def setup(coords, conn, seed, load=True, sep=False):
    n, e = coords.shape[0], conn.shape[0]
    rng = np.random.default_rng(seed)
    kappa = np.exp(rng.standard_normal(e))
    f = meshes.fourier_source(coords, seed) if load else None
    u = rng.standard_normal(n)
    offs, dofs = meshes.scalar_elem_dofs(conn)
    amap = A.makeAssemblyMap(n, n, dev(offs), dev(dofs), dev(offs), dev(dofs))
    om = orc.AssemblyMap(n, n, offs, dofs, offs, dofs)
    rres, rvals = orc.assemble_p1_kappa(om, orc.P1Quad(coords, conn), kappa,
                                        f if load else np.zeros(n), u)
    ntiles = amap.enableTiles(dev(coords), dev(conn) if sep else None)
    return dict(n=n, amap=amap, coords=dev(coords), conn=dev(conn) if sep else None,
                kappa=dev(kappa), f=dev(f) if load else None, u=dev(u), rres=rres,
                rvals=rvals, ntiles=ntiles)


def run(p, precision, jac=True):
    res = torch.full((p["n"],), np.nan, dtype=torch.float64, device="cuda")
    mat = A.CsrMatrix(p["amap"].pattern()) if jac else None
    if mat is not None:
        mat.vals.fill_(np.nan)  # every slot must be written
    A.assembleP1Kappa(p["amap"], p["coords"], p["kappa"], p["f"], p["u"], res, mat,
                      conn=p["conn"], precision=precision, tiled=True)
    p["amap"].check()
    torch.cuda.synchronize()
    return res.cpu().numpy(), (mat.vals.cpu().numpy() if mat is not None else None)


# --- integer-pipe double-float conversions -------------------------------

def dd_probe(x, jhi, jlo):
    n = x.size
    xd = dev(x.astype(np.float64))
    hi = torch.empty(n, dtype=torch.float32, device="cuda")
    lo = torch.empty(n, dtype=torch.float32, device="cuda")
    jh, jl = dev(jhi.astype(np.float32)), dev(jlo.astype(np.float32))
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(_lib.lib().gbfem_probe_dd(n, C.c_void_p(xd.data_ptr()), C.c_void_p(hi.data_ptr()),
                                         C.c_void_p(lo.data_ptr()), C.c_void_p(jh.data_ptr()),
                                         C.c_void_p(jl.data_ptr()), C.c_void_p(out.data_ptr()),
                                         s))
    torch.cuda.synchronize()
    return hi.cpu().numpy(), lo.cpu().numpy(), out.cpu().numpy()


def test_double_float_split_keeps_47_bits():
    """24 + 23 leading bits: hi + lo within 2^-46 |x| (six low bits dropped)."""
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.standard_normal(1 << 18),
                        rng.standard_normal(1 << 16) * 10.0 ** rng.integers(-30, 30, 1 << 16),
                        np.array([0.0, -0.0, 1.0, -1.0, 2.0 ** -100, -(2.0 ** 100),
                                  np.nextafter(1.0, 2.0), np.nextafter(1.0, 0.0)])])
    hi, lo, _ = dd_probe(x, np.zeros_like(x), np.zeros_like(x))
    s = hi.astype(np.float64) + lo.astype(np.float64)   # exact: 24 + 23 bits
    big = np.abs(x) >= 2.0 ** -103                       # below, lo is 0
    assert np.all(np.abs(s - x)[big] <= 2.0 ** -46 * np.abs(x)[big])
    assert np.all(np.abs(s - x)[~big] <= 2.0 ** -23 * np.abs(x)[~big])
    # hi is x truncated to float: same sign, not larger in magnitude
    assert np.all(np.abs(hi.astype(np.float64)) <= np.abs(x))
    assert np.all((hi == 0) | (np.sign(hi) == np.sign(x)))
    assert hi[-8] == 0 and lo[-8] == 0


def test_double_float_join_is_faithful():
    rng = np.random.default_rng(1)
    v = np.concatenate([rng.standard_normal(1 << 18),
                        rng.standard_normal(1 << 16) * 10.0 ** rng.integers(-30, 30, 1 << 16)])
    jhi = v.astype(np.float32)
    jlo = (v - jhi.astype(np.float64)).astype(np.float32)     # normalised pairs
    # powers of two with a negative low part (the result drops a binade),
    # zero low parts, zeros
    p2 = (2.0 ** rng.integers(-60, 60, 4096)).astype(np.float32)
    pl = -(rng.uniform(0.0, 0.25, 4096) * np.spacing(p2)).astype(np.float32)
    jhi = np.concatenate([jhi, p2, p2, -p2, np.float32([0.0, 1.5])])
    jlo = np.concatenate([jlo, pl, np.zeros(4096, np.float32), -pl, np.float32([0.0, 0.0])])
    _, _, out = dd_probe(np.zeros(jhi.size), jhi, jlo)
    exact = jhi.astype(np.float64) + jlo.astype(np.float64)    # exact in FP64
    big = np.abs(jhi) >= 2.0 ** -74                            # faithful
    tiny = np.abs(jhi) < 2.0 ** -103                           # lo is dropped
    mid = ~big & ~tiny                                         # lo partly counted
    assert np.all(np.abs(out - exact)[big] <= np.spacing(np.abs(exact))[big])
    assert np.all(out[tiny] == jhi[tiny].astype(np.float64))
    assert np.all(np.abs(out - exact)[mid] <= np.abs(jlo[mid]))
    assert mid.sum() > 1000 and big.sum() > 100000
    assert out[-2] == 0.0 and out[-1] == 1.5


def test_double_float_join_special_values():
    """Infinite and NaN hi widen as they are; zero and subnormal hi give a
    zero of hi's sign."""
    f32 = np.float32
    jhi = np.array([np.inf, -np.inf, np.nan, -0.0, 1e-40, -1e-40, 2.0 ** 127, -(2.0 ** -126)],
                   dtype=f32)
    jlo = np.array([0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 2.0 ** 100, 0.0], dtype=f32)
    _, _, out = dd_probe(np.zeros(jhi.size), jhi, jlo)
    assert out[0] == np.inf and out[1] == -np.inf and np.isnan(out[2])
    assert out[3] == 0.0 and np.signbit(out[3])
    assert out[4] == 0.0 and not np.signbit(out[4])
    assert out[5] == 0.0 and np.signbit(out[5])
    assert out[6] == 2.0 ** 127 + 2.0 ** 100
    assert out[7] == -(2.0 ** -126)


# --- parity ----------------------------------------------------------------

@pytest.mark.parametrize("precision", ["fp64", "double_float", "fp32_quad"])
@pytest.mark.parametrize("mesh", ["structured", "jittered_permuted"])
@pytest.mark.parametrize("load,sep", [(True, False), (False, True), (True, True)])
def test_tiled_matches_oracle(precision, mesh, load, sep):
    if mesh == "structured":
        coords, conn = meshes.structured_tri(40)
    else:
        coords, conn = meshes.jittered_tri(44, seed=7)
    p = setup(coords, conn, 3, load=load, sep=sep)
    assert p["ntiles"] > 4
    res, vals = run(p, precision)
    assert np.isfinite(vals).all() and np.isfinite(res).all()
    assert rel_inf(vals, p["rvals"]) <= TOL[precision]
    assert rel_inf(res, p["rres"]) <= TOL[precision]
    # residual-only calls write the same residual
    res2, _ = run(p, precision, jac=False)
    assert np.array_equal(res2, res)


@pytest.mark.parametrize("precision", ["fp64", "double_float"])
def test_tiled_is_bitwise_reproducible_and_agrees_with_atomic(precision):
    coords, conn = meshes.jittered_tri(96, seed=21)
    p = setup(coords, conn, 4)
    r1, v1 = run(p, precision)
    r2, v2 = run(p, precision)
    assert np.array_equal(r1, r2) and np.array_equal(v1, v2)
    res = torch.zeros(p["n"], dtype=torch.float64, device="cuda")
    mat = A.CsrMatrix(p["amap"].pattern())
    A.assembleP1Kappa(p["amap"], p["coords"], p["kappa"], p["f"], p["u"], res, mat)
    # double-float carries about 2^-46 per operation
    assert rel_inf(v1, mat.vals.cpu().numpy()) <= 1e-13
    assert rel_inf(r1, res.cpu().numpy()) <= 1e-13


@pytest.mark.parametrize("case", ["p1_32", "p1_jit9", "real_sq_p1"])
@pytest.mark.parametrize("precision", ["fp64", "double_float"])
def test_tiled_matches_reference_goldens(case, precision):
    """Against the vectors the reference library produced: the 32x32
    Poisson case, a jittered 9x9 mesh and femx's own square mesh
    (data/meshes/2d_square_res_very_low.msh), kappa, source and state as
    recorded."""
    g = np.load(os.path.join(GOLDEN, case + ".npz"))
    coords, conn = g["coords"], g["conn"].astype(np.int32)
    n = coords.shape[0]
    offs, dofs = meshes.scalar_elem_dofs(conn)
    amap = A.makeAssemblyMap(n, n, dev(offs), dev(dofs), dev(offs), dev(dofs))
    amap.enableTiles(dev(coords))
    res = torch.zeros(n, dtype=torch.float64, device="cuda")
    mat = A.CsrMatrix(amap.pattern())
    A.assembleP1Kappa(amap, dev(coords), dev(g["kappa"]), dev(g["f"]), dev(g["u"]), res, mat,
                      precision=precision, tiled=True)
    amap.check()
    assert rel_inf(mat.vals.cpu().numpy(), g["vals"]) <= 1e-12
    assert rel_inf(res.cpu().numpy(), g["res"]) <= 1e-12


@pytest.mark.parametrize("precision", ["double_float", "fp64"])
def test_tiled_poisson_1024_matches_oracle(precision):
    """The benchmark configuration (1024x1024, log-normal GRF kappa, Fourier
    source) at full size against the oracle, 1e-12."""
    coords, conn = meshes.structured_tri(1024)
    n = coords.shape[0]
    kappa = np.exp(meshes.grf_centroids(coords, conn, seed=2, ell=0.05, var=1.0, grid=1024))
    f = meshes.fourier_source(coords, 1)
    u = np.random.default_rng(5).standard_normal(n)
    offs, dofs = meshes.scalar_elem_dofs(conn)
    om = orc.AssemblyMap(n, n, offs, dofs, offs, dofs)
    rres, rvals = orc.assemble_p1_kappa(om, orc.P1Quad(coords, conn), kappa, f, u)
    amap = A.makeAssemblyMap(n, n, dev(offs), dev(dofs), dev(offs), dev(dofs))
    amap.enableTiles(dev(coords))
    res = torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
    mat = A.CsrMatrix(amap.pattern())
    mat.vals.fill_(np.nan)
    A.assembleP1Kappa(amap, dev(coords), dev(kappa), dev(f), dev(u), res, mat,
                      precision=precision, tiled=True)
    amap.check()
    assert rel_inf(mat.vals.cpu().numpy(), rvals) <= 1e-12
    assert rel_inf(res.cpu().numpy(), rres) <= 1e-12


def test_tiled_rows_without_elements_get_zero_residual():
    coords, conn = meshes.structured_tri(8)
    n = coords.shape[0] + 5           # five DOFs no element touches
    offs, dofs = meshes.scalar_elem_dofs(conn)
    amap = A.makeAssemblyMap(n, n, dev(offs), dev(dofs), dev(offs), dev(dofs))
    xy = np.concatenate([coords, np.zeros((5, 2))])
    amap.enableTiles(dev(xy))
    res = torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
    mat = A.CsrMatrix(amap.pattern())
    A.assembleP1Kappa(amap, dev(xy), dev(np.ones(conn.shape[0])), None,
                      dev(np.ones(n)), res, mat, precision="double_float", tiled=True)
    r = res.cpu().numpy()
    assert np.all(r[-5:] == 0.0) and np.all(np.abs(r[:-5]) <= 1e-13)   # K 1 = 0


def test_tiled_builder_refusals():
    # three triangles on one edge: not a conforming mesh
    coords = np.array([[0, 0], [1, 0], [0, 1], [1, 1], [0.5, -1]], dtype=np.float64)
    conn = np.array([[0, 1, 2], [1, 0, 3], [0, 1, 4]], dtype=np.int32)
    offs, dofs = meshes.scalar_elem_dofs(conn)
    amap = A.makeAssemblyMap(5, 5, dev(offs), dev(dofs), dev(offs), dev(dofs))
    with pytest.raises(_lib.GbfemError, match="more than two elements share an edge"):
        amap.enableTiles(dev(coords))
    # tiled assembly before the tiles exist
    coords, conn = meshes.structured_tri(4)
    offs, dofs = meshes.scalar_elem_dofs(conn)
    n = coords.shape[0]
    amap = A.makeAssemblyMap(n, n, dev(offs), dev(dofs), dev(offs), dev(dofs))
    res = torch.zeros(n, dtype=torch.float64, device="cuda")
    with pytest.raises(_lib.GbfemError, match="enable_tiles"):
        A.assembleP1Kappa(amap, dev(coords), dev(np.ones(conn.shape[0])), None,
                          dev(np.zeros(n)), res, tiled=True)
    # connectivity given at assembly but not when tiling
    amap.enableTiles(dev(coords))
    with pytest.raises(_lib.GbfemError, match="connectivity"):
        A.assembleP1Kappa(amap, dev(coords), dev(np.ones(conn.shape[0])), None,
                          dev(np.zeros(n)), res, conn=dev(conn), tiled=True)
    # the Taylor-Hood layout is not P1
    c2, k6, _ = meshes.p2_mesh(*meshes.structured_tri(2))
    offs6, dofs6, _ = meshes.th_elem_dofs(k6, c2.shape[0])
    nd = int(dofs6.max()) + 1
    tmap = A.makeAssemblyMap(nd, nd, dev(offs6), dev(dofs6), dev(offs6), dev(dofs6))
    with pytest.raises(_lib.GbfemError, match="P1 layout"):
        tmap.enableTiles(dev(c2))


@pytest.mark.parametrize("precision", ["fp64", "double_float"])
@pytest.mark.parametrize("mesh", ["structured", "jittered_permuted"])
def test_tiled_vjp_matches_oracle(precision, mesh):
    """The residual VJPs in tiled form: g_u = K^T lambda row by row, g_m[e] =
    lambda_e^T K_e u_e written by the element's owner tile, against the
    oracle's (femx's element loop restated), 1e-12; both outputs fully
    written (filled with NaN first), bitwise equal over runs."""
    if mesh == "structured":
        coords, conn = meshes.structured_tri(40)
    else:
        coords, conn = meshes.jittered_tri(44, seed=9)
    n, e = coords.shape[0], conn.shape[0]
    rng = np.random.default_rng(17)
    kappa, u, lam = np.exp(rng.standard_normal(e)), rng.standard_normal(n), rng.standard_normal(n)
    offs, dofs = meshes.scalar_elem_dofs(conn)
    om = orc.AssemblyMap(n, n, offs, dofs, offs, dofs)
    gu_ref, gm_ref = orc.vjp_p1_kappa(om, orc.P1Quad(coords, conn), kappa, u, lam)
    amap = A.makeAssemblyMap(n, n, dev(offs), dev(dofs), dev(offs), dev(dofs))
    amap.enableTiles(dev(coords))
    outs = []
    for _ in range(2):
        g_u = torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
        g_m = torch.full((e,), np.nan, dtype=torch.float64, device="cuda")
        A.vjpP1Kappa(amap, dev(coords), dev(kappa), dev(u), dev(lam), g_u, g_m,
                     precision=precision, tiled=True)
        amap.check()
        outs.append((g_u.cpu().numpy(), g_m.cpu().numpy()))
    assert rel_inf(outs[0][0], gu_ref) <= 1e-12
    assert rel_inf(outs[0][1], gm_ref) <= 1e-12
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_tiled_vjp_refuses_fp32():
    coords, conn = meshes.structured_tri(4)
    n, e = coords.shape[0], conn.shape[0]
    offs, dofs = meshes.scalar_elem_dofs(conn)
    amap = A.makeAssemblyMap(n, n, dev(offs), dev(dofs), dev(offs), dev(dofs))
    amap.enableTiles(dev(coords))
    g = torch.zeros(n, dtype=torch.float64, device="cuda")
    with pytest.raises(_lib.GbfemError, match="FP64 or DOUBLE_FLOAT"):
        A.vjpP1Kappa(amap, dev(coords), dev(np.ones(e)), dev(np.zeros(n)), dev(np.zeros(n)), g,
                     None, precision="fp32_quad", tiled=True)


def fan(nt):
    """nt triangles around node 0 (a closed fan: a valid conforming mesh)."""
    ang = 2 * np.pi * np.arange(nt) / nt
    coords = np.vstack([[0.0, 0.0], np.stack([np.cos(ang), np.sin(ang)], 1)])
    conn = np.array([[0, 1 + i, 1 + (i + 1) % nt] for i in range(nt)], dtype=np.int32)
    return coords, conn


def test_tiled_high_valence_row_fits_and_matches_oracle():
    """A row with 300 incident elements (one tile holds up to 512): the row's
    300 slots and its neighbours' are all written, against the oracle."""
    coords, conn = fan(300)
    p = setup(coords, conn, 5)
    res, vals = run(p, "double_float")
    assert rel_inf(vals, p["rvals"]) <= 1e-12 and rel_inf(res, p["rres"]) <= 1e-12


def test_tiled_refuses_a_row_larger_than_a_tile():
    coords, conn = fan(600)
    n = coords.shape[0]
    offs, dofs = meshes.scalar_elem_dofs(conn)
    amap = A.makeAssemblyMap(n, n, dev(offs), dev(dofs), dev(offs), dev(dofs))
    with pytest.raises(_lib.GbfemError, match="more elements than a tile holds"):
        amap.enableTiles(dev(coords))
