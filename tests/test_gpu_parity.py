"""GPU parity: libgbfem (through its C ABI) against the CPU oracle and the
reference's golden vectors.

Gates (femx semantics):
  * CSR row_ptr/col_ind, jac_map, Dirichlet sets and BoundaryMap arrays:
    bit-exact.
  * FP64 values/residuals/VJPs: ||d||_inf / ||ref||_inf <= 1e-12.
  * FP32-quadrature values: <= 1e-6.
  * prepareForwardSolve on identical inputs: bit-exact (vals and rhs).
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from conftest import load_golden, rel_inf  # noqa: E402
from femx_gb300 import assembly as A  # noqa: E402
from femx_gb300 import meshes  # noqa: E402
from oracle import pyoracle as orc  # noqa: E402

TOL64 = 1e-12
TOL32 = 1e-6


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from femx_gb300 import build
    build.build()


def dev(a, dtype=None):
    a = np.ascontiguousarray(a)
    t = torch.from_numpy(a)
    if dtype is not None:
        t = t.to(dtype)
    return t.cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def gpu_map(num_res, num_states, ro, rd, so, sd):
    return A.makeAssemblyMap(num_res, num_states, dev(ro, torch.int32), dev(rd, torch.int32),
                             dev(so, torch.int32), dev(sd, torch.int32))


def assert_map_equal(m, ref_row_ptr, ref_col_ind, ref_jac_map):
    p = m.pattern()
    np.testing.assert_array_equal(host(p.row_ptr), ref_row_ptr)
    np.testing.assert_array_equal(host(p.col_ind), ref_col_ind)
    if ref_jac_map is not None:  # the real-mesh Taylor-Hood fixture omits it (size)
        np.testing.assert_array_equal(host(m.view()["jac_map"]), ref_jac_map)


# ---------------------------------------------------------------- patterns

def test_known_answer_maps():
    kat = load_golden("kat")
    m = gpu_map(3, 3, [0, 2, 4], [0, 1, 1, 2], [0, 2, 4], [0, 1, 1, 2])
    assert_map_equal(m, kat["shared_row_ptr"], kat["shared_col_ind"], kat["shared_jac_map"])
    m = gpu_map(2, 2, [0, 2, 3], [0, 1, 1], [0, 1, 3], [0, 0, 1])
    assert_map_equal(m, kat["rect_row_ptr"], kat["rect_col_ind"], kat["rect_jac_map"])
    np.testing.assert_array_equal(host(m.view()["jac_offsets"]), [0, 2, 4])


@pytest.mark.parametrize("case", ["p1_32", "p1_jit9", "real_sq_p1"])
def test_p1_pattern_matches_reference(case):
    g = load_golden(case)
    offs, dofs = meshes.scalar_elem_dofs(g["conn"])
    n = g["coords"].shape[0]
    m = gpu_map(n, n, offs, dofs, offs, dofs)
    assert_map_equal(m, g["row_ptr"], g["col_ind"], g["jac_map"])
    np.testing.assert_array_equal(host(m.view()["jac_offsets"]), g["jac_offsets"])


@pytest.mark.parametrize("case", ["th_4", "th_jit3", "real_sq_th"])
def test_th_pattern_matches_reference(case):
    g = load_golden(case)
    nd = int(g["num_dofs"])
    offs = (np.arange(g["conn6"].shape[0] + 1) * 15).astype(np.int32)
    m = gpu_map(nd, nd, offs, g["elem_dofs"], offs, g["elem_dofs"])
    assert_map_equal(m, g["row_ptr"], g["col_ind"], g.get("jac_map"))


@pytest.mark.parametrize("nx,jitter", [(96, False), (64, True)])
def test_p1_pattern_matches_oracle_larger(nx, jitter):
    coords, conn = meshes.jittered_tri(nx, seed=nx) if jitter else meshes.structured_tri(nx)
    offs, dofs = meshes.scalar_elem_dofs(conn)
    n = coords.shape[0]
    ref = orc.AssemblyMap(n, n, offs, dofs, offs, dofs)
    m = gpu_map(n, n, offs, dofs, offs, dofs)
    assert_map_equal(m, ref.row_ptr, ref.col_ind, ref.jac_map)


def test_th_pattern_matches_oracle_16():
    c3, k3 = meshes.jittered_tri(16, seed=3)
    cp2, conn6, _ = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    ref = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    m = gpu_map(nd, nd, offs, dofs, offs, dofs)
    assert_map_equal(m, ref.row_ptr, ref.col_ind, ref.jac_map)


def test_rectangular_variable_blocks_match_oracle():
    rng = np.random.default_rng(5)
    e, nr_glob, ns_glob = 300, 120, 90
    nrs = rng.integers(0, 5, size=e)
    nss = rng.integers(1, 6, size=e)
    ro = np.concatenate([[0], np.cumsum(nrs)]).astype(np.int32)
    so = np.concatenate([[0], np.cumsum(nss)]).astype(np.int32)
    rd = rng.integers(0, nr_glob, size=ro[-1]).astype(np.int32)  # duplicates allowed
    sd = rng.integers(0, ns_glob, size=so[-1]).astype(np.int32)
    ref = orc.AssemblyMap(nr_glob, ns_glob, ro, rd, so, sd)
    m = gpu_map(nr_glob, ns_glob, ro, rd, so, sd)
    assert_map_equal(m, ref.row_ptr, ref.col_ind, ref.jac_map)
    assert m.maxRes() == ref.max_res and m.maxState() == ref.max_state
    assert m.maxJac() == ref.max_jac


def test_empty_map():
    m = gpu_map(4, 4, [0], [], [0], [])
    assert m.numElems() == 0 and m.pattern().nnz == 0
    np.testing.assert_array_equal(host(m.pattern().row_ptr), [0, 0, 0, 0, 0])


def test_map_rejects_bad_dofs():
    with pytest.raises(A.GbfemError, match="residual DOF is out of range"):
        gpu_map(2, 2, [0, 1], [2], [0, 1], [0])
    with pytest.raises(A.GbfemError, match="state DOF is out of range"):
        gpu_map(2, 2, [0, 1], [0], [0, 1], [-1])
    with pytest.raises(A.GbfemError, match="non-negative"):
        gpu_map(2, 2, [0, 2, 1], [0, 1], [0, 1, 2], [0, 1])


# ---------------------------------------------------------------- boundary

DENSE_ROW_PTR = np.array([0, 3, 6, 9], np.int32)
DENSE_COL_IND = np.array([0, 1, 2, 0, 1, 2, 0, 1, 2], np.int32)
DENSE_VALS = np.array([4.0, 1.0, 2.0, 3.0, 5.0, 6.0, 7.0, 8.0, 9.0])


def dense_pattern():
    return A.CsrPattern(3, 3, dev(DENSE_ROW_PTR), dev(DENSE_COL_IND), 0)


@pytest.mark.parametrize("bcs,g,tag", [([1], [2.0], "bc1_"), ([0, 2], [2.0, -1.0], "bc02_")])
def test_boundary_known_answers(bcs, g, tag):
    kat = load_golden("kat")
    pat = dense_pattern()
    bc = A.makeBoundaryMap(dev(np.array(bcs, np.int32)), pat)
    for d, key in ((1.0, "rows1"), (0.0, "rows0")):
        mat = A.CsrMatrix(pat, dev(DENSE_VALS))
        A.replaceRows(bc, mat, d)
        np.testing.assert_array_equal(host(mat.vals), kat[tag + key])
    res = dev(np.array([10.0, 20.0, 30.0]))
    A.replaceRes(bc, dev(np.array([4.0, 7.0, 9.0])), dev(np.array(g)), res)
    np.testing.assert_array_equal(host(res), kat[tag + "res"])
    mat = A.CsrMatrix(pat, dev(DENSE_VALS))
    rhs = dev(np.array([10.0, 20.0, 30.0]))
    A.prepareForwardSolve(bc, mat, rhs, dev(np.array(g)))
    np.testing.assert_array_equal(host(mat.vals), kat[tag + "fwd_vals"])
    np.testing.assert_array_equal(host(rhs), kat[tag + "fwd_rhs"])


def test_boundary_rejects_bad_input():
    pat = dense_pattern()
    with pytest.raises(A.GbfemError, match="must be unique"):
        A.makeBoundaryMap(dev(np.array([1, 1], np.int32)), pat)
    with pytest.raises(A.GbfemError, match="out of range"):
        A.makeBoundaryMap(dev(np.array([3], np.int32)), pat)
    nodiag = A.CsrPattern(2, 2, dev(np.array([0, 1, 2], np.int32)),
                          dev(np.array([1, 0], np.int32)), 0)
    with pytest.raises(A.GbfemError, match="no diagonal entry"):
        A.makeBoundaryMap(dev(np.array([0], np.int32)), nodiag)
    bc = A.makeBoundaryMap(dev(np.array([1], np.int32)), pat)
    other = A.CsrMatrix(A.CsrPattern(3, 3, pat.row_ptr, pat.col_ind, 99), dev(DENSE_VALS))
    with pytest.raises(A.GbfemError, match="does not match the mapped CSR layout"):
        A.replaceRows(bc, other, 1.0)


# ---------------------------------------------------------------- P1 Poisson

def p1_setup(coords, conn):
    offs, dofs = meshes.scalar_elem_dofs(conn)
    n = coords.shape[0]
    return gpu_map(n, n, offs, dofs, offs, dofs), orc.AssemblyMap(n, n, offs, dofs, offs, dofs)


def p1_gpu(m, coords, kappa, f, u, precision="fp64"):
    res = torch.zeros(m.numRes(), dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(m.pattern())
    A.assembleP1Kappa(m, dev(coords), dev(kappa), None if f is None else dev(f), dev(u), res,
                      jac, precision=precision)
    m.check()
    return host(res), host(jac.vals), jac, res


# (precision, Jacobian tolerance, residual tolerance): MIXED keeps the
# residual in FP64 while the Jacobian comes from FP32 quadrature.
PRECS = [("fp64", TOL64, TOL64), ("fp32_quad", TOL32, TOL32), ("mixed", TOL32, TOL64)]
# the assemblies add the double-float mode (FP64-accurate element
# arithmetic on the FP32 pipe), held to the FP64 gate
TH_PRECS = PRECS + [("double_float", TOL64, TOL64)]


@pytest.mark.parametrize("case", ["p1_32", "p1_jit9", "real_sq_p1"])
@pytest.mark.parametrize("precision,tol_j,tol_r", TH_PRECS)
def test_p1_assembly_matches_reference(case, precision, tol_j, tol_r):
    g = load_golden(case)
    m, _ = p1_setup(g["coords"], g["conn"])
    res, vals, _, _ = p1_gpu(m, g["coords"], g["kappa"], g["f"], g["u"], precision)
    assert rel_inf(res, g["res"]) <= tol_r
    assert rel_inf(vals, g["vals"]) <= tol_j


@pytest.mark.parametrize("precision,tol", [("fp64", TOL64), ("fp32_quad", TOL32)])
def test_p1_assembly_grf_kappa_matches_oracle(precision, tol):
    coords, conn = meshes.jittered_tri(128, seed=2)
    e, n = conn.shape[0], coords.shape[0]
    kappa = np.exp(meshes.grf_centroids(coords, conn, seed=2, ell=0.05))
    f = meshes.fourier_source(coords, 1)
    u = np.random.default_rng(0).standard_normal(n)
    m, om = p1_setup(coords, conn)
    q = orc.P1Quad(coords, conn)
    rres, rvals = orc.assemble_p1_kappa(om, q, kappa, f, u)
    res, vals, _, _ = p1_gpu(m, coords, kappa, f, u, precision)
    assert rel_inf(res, rres) <= tol
    assert rel_inf(vals, rvals) <= tol
    # residual-only call gives the same residual
    r2 = torch.zeros(n, dtype=torch.float64, device="cuda")
    A.assembleP1Kappa(m, dev(coords), dev(kappa), dev(f), dev(u), r2, None, precision=precision)
    assert rel_inf(host(r2), rres) <= tol


def test_p1_separate_connectivity_matches():
    g = load_golden("p1_jit9")
    m, _ = p1_setup(g["coords"], g["conn"])
    res = torch.zeros(m.numRes(), dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(m.pattern())
    A.assembleP1Kappa(m, dev(g["coords"]), dev(g["kappa"]), dev(g["f"]), dev(g["u"]), res, jac,
                      conn=dev(g["conn"], torch.int32))
    assert rel_inf(host(res), g["res"]) <= TOL64
    assert rel_inf(host(jac.vals), g["vals"]) <= TOL64


def test_p1_degenerate_element_is_reported():
    coords, conn = meshes.structured_tri(4)
    coords = coords.copy()
    conn = conn.copy()
    conn[5] = [conn[5][0], conn[5][0], conn[5][2]]  # zero-area element
    offs, dofs = meshes.scalar_elem_dofs(conn)
    n = coords.shape[0]
    m = gpu_map(n, n, offs, dofs, offs, dofs)
    res = torch.zeros(n, dtype=torch.float64, device="cuda")
    A.assembleP1Kappa(m, dev(coords), dev(np.ones(conn.shape[0])), None, dev(np.zeros(n)), res)
    with pytest.raises(A.GbfemError, match="Singular 2D Jacobian"):
        m.check()
    m.check()  # the status word was cleared


@pytest.mark.parametrize("case", ["p1_32", "p1_jit9", "real_sq_p1"])
def test_boundary_map_and_operations_match_reference(case):
    g = load_golden(case)
    m, om = p1_setup(g["coords"], g["conn"])
    dofs_bc = meshes.dirichlet_dofs(g["coords"], meshes.boundary_nodes(g["coords"]))
    np.testing.assert_array_equal(dofs_bc, g["bc_dofs"])
    bc = A.makeBoundaryMap(dev(dofs_bc), m.pattern())
    v = bc.view()
    for key, ref in (("bc_rows", "bc_rows"), ("diag", "bc_diag"), ("col_offsets", "bc_col_offsets"),
                     ("col_entries", "bc_col_entries"), ("col_rows", "bc_col_rows"),
                     ("bc_mask", "bc_mask")):
        np.testing.assert_array_equal(host(v[key]), g[ref])
    pat = m.pattern()
    # replaceRows on the reference's own matrix values: bit-exact
    mat = A.CsrMatrix(pat, dev(g["vals"]))
    A.replaceRows(bc, mat, 1.0)
    np.testing.assert_array_equal(host(mat.vals), g["vals_rows1"])
    res = dev(g["res"])
    A.replaceRes(bc, dev(g["u"]), dev(g["bc_vals"]), res)
    np.testing.assert_array_equal(host(res), g["res_replaced"])
    mat = A.CsrMatrix(pat, dev(g["vals"]))
    rhs = dev(-g["res"])
    A.prepareForwardSolve(bc, mat, rhs, dev(g["bc_vals"]))
    np.testing.assert_array_equal(host(mat.vals), g["vals_fwd"])
    np.testing.assert_array_equal(host(rhs), g["rhs_fwd"])
    z = dev(g["u"])
    A.zeroBoundary(bc, z)
    expect = g["u"].copy()
    expect[g["bc_dofs"]] = 0.0
    np.testing.assert_array_equal(host(z), expect)


# ---------------------------------------------------------------- SpMV

@pytest.mark.parametrize("case", ["p1_32", "p1_jit9", "real_sq_p1"])
def test_spmv_matches_reference(case):
    g = load_golden(case)
    m, _ = p1_setup(g["coords"], g["conn"])
    mat = A.CsrMatrix(m.pattern(), dev(g["vals"]))
    n = g["coords"].shape[0]
    y = torch.zeros(n, dtype=torch.float64, device="cuda")
    A.matvec(mat, dev(g["x"]), y)
    assert rel_inf(host(y), g["y_matvec"]) <= 1e-13
    yt = torch.zeros(n, dtype=torch.float64, device="cuda")
    A.matvecT(mat, dev(g["x"]), yt)
    assert rel_inf(host(yt), g["y_matvec_t"]) <= 1e-13
    # alpha/beta semantics
    y0 = np.random.default_rng(1).standard_normal(n)
    y = dev(y0)
    A.matvec(mat, dev(g["x"]), y, alpha=2.0, beta=-0.5)
    assert rel_inf(host(y), orc.matvec(g["row_ptr"], g["col_ind"], g["vals"], g["x"], y0, 2.0,
                                       -0.5)) <= 1e-13
    y = dev(y0)
    A.matvecT(mat, dev(g["x"]), y, alpha=-1.0, beta=3.0)
    assert rel_inf(host(y), orc.matvec_t(g["row_ptr"], g["col_ind"], g["vals"], g["x"], n, y0,
                                         -1.0, 3.0)) <= 1e-13


# ---------------------------------------------------------------- VJP

@pytest.mark.parametrize("case", ["p1_32", "p1_jit9", "real_sq_p1"])
@pytest.mark.parametrize("precision,tol", [("fp64", TOL64), ("fp32_quad", TOL32)])
def test_vjp_matches_reference(case, precision, tol):
    g = load_golden(case)
    m, _ = p1_setup(g["coords"], g["conn"])
    n, e = g["coords"].shape[0], g["conn"].shape[0]
    g_u = torch.zeros(n, dtype=torch.float64, device="cuda")
    g_m = torch.zeros(e, dtype=torch.float64, device="cuda")
    A.vjpP1Kappa(m, dev(g["coords"]), dev(g["kappa"]), dev(g["u"]), dev(g["lam"]), g_u, g_m,
                 precision=precision)
    assert rel_inf(host(g_u), g["g_u"]) <= tol
    assert rel_inf(host(g_m), g["g_m"]) <= tol


# ---------------------------------------------------------------- Taylor-Hood

def th_gpu(g_coords, conn6, elem_dofs, nd, nu, state, precision="fp64"):
    offs = (np.arange(conn6.shape[0] + 1) * 15).astype(np.int32)
    m = gpu_map(nd, nd, offs, elem_dofs, offs, elem_dofs)
    res = torch.zeros(nd, dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(m.pattern())
    A.assembleTaylorHood(m, dev(g_coords), dev(conn6, torch.int32), nu, dev(state), res, jac,
                         precision=precision)
    m.check()
    return m, host(res), host(jac.vals)


@pytest.mark.parametrize("case", ["th_4", "th_jit3", "real_sq_th"])
@pytest.mark.parametrize("precision,tol_j,tol_r", TH_PRECS)
def test_taylor_hood_matches_reference(case, precision, tol_j, tol_r):
    g = load_golden(case)
    _, res, vals = th_gpu(g["coords"], g["conn6"], g["elem_dofs"], int(g["num_dofs"]),
                          float(g["nu"]), g["state"], precision)
    assert rel_inf(res, g["res"]) <= tol_r
    assert rel_inf(vals, g["vals"]) <= tol_j


def test_taylor_hood_cavity_matches_oracle():
    c3, k3 = meshes.structured_tri(24)
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    vel = meshes.stream_velocity(cp2, seed=3)
    state = np.concatenate([vel.reshape(-1), np.random.default_rng(3).standard_normal(nv)])
    om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    rres, rvals = orc.assemble_th_ns(om, cp2, conn6, 1e-3, state)
    for precision, tol_j, tol_r in TH_PRECS:
        _, res, vals = th_gpu(cp2, conn6, dofs, nd, 1e-3, state, precision)
        assert rel_inf(res, rres) <= tol_r
        assert rel_inf(vals, rvals) <= tol_j


@pytest.mark.parametrize("precision", ["fp64", "fp32_quad", "mixed"])
def test_taylor_hood_assembly_is_bitwise_reproducible(precision):
    """Deterministic mode: element records summed per CSR row in element
    order, no atomics, so repeated assemblies agree bit for bit (also
    residual-only calls)."""
    c3, k3 = meshes.jittered_tri(20, seed=9)
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    state = meshes.cavity_state(cp2, nv, seed=9)
    m = gpu_map(nd, nd, offs, dofs, offs, dofs)
    coords, c6, st = dev(cp2), dev(conn6, torch.int32), dev(state)
    outs = []
    for _ in range(3):
        res = torch.full((nd,), 7.0, dtype=torch.float64, device="cuda")
        jac = A.CsrMatrix(m.pattern(), torch.full((m.pattern().nnz,), -3.0,
                                                  dtype=torch.float64, device="cuda"))
        A.assembleTaylorHood(m, coords, c6, 1e-3, st, res, jac, precision=precision,
                             deterministic=True)
        r_only = torch.full((nd,), 5.0, dtype=torch.float64, device="cuda")
        A.assembleTaylorHood(m, coords, c6, 1e-3, st, r_only, None, precision=precision,
                             deterministic=True)
        outs.append((res, jac.vals, r_only))
    m.check()
    for res, vals, r_only in outs[1:]:
        assert torch.equal(res, outs[0][0])
        assert torch.equal(vals, outs[0][1])
        assert torch.equal(r_only, outs[0][2])
    om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    rres, rvals = orc.assemble_th_ns(om, cp2, conn6, 1e-3, state)
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert rel_inf(host(outs[0][1]), rvals) <= tol
    assert rel_inf(host(outs[0][0]), rres) <= (1e-12 if precision != "fp32_quad" else 1e-6)


def test_deterministic_mode_needs_a_supported_layout():
    coords, conn = meshes.structured_tri(4)
    offs, dofs = meshes.scalar_elem_dofs(conn)
    n = coords.shape[0]
    m = gpu_map(n, n, offs, dofs, offs, dofs)
    with pytest.raises(A.GbfemError, match="row-gather"):
        m.enableDeterministic()


def test_csr_transpose_known_answer():
    """femx's csrMatrixTranspose (tests/unit/linalg/runLinalgTests.cpp:307-355)."""
    pat = A.CsrPattern(3, 4, dev(np.array([0, 2, 4, 7]), torch.int32),
                       dev(np.array([0, 2, 1, 3, 0, 2, 3]), torch.int32), 12345)
    src = A.CsrMatrix(pat, dev(np.array([2.0, -1.0, 3.0, 4.0, -2.0, 5.0, 1.0])))
    dst = A.transpose(src)
    assert (dst.rows, dst.cols, dst.nnz) == (4, 3, 7)
    assert host(dst.pattern.row_ptr).tolist() == [0, 2, 3, 5, 7]
    assert host(dst.pattern.col_ind).tolist() == [0, 2, 1, 0, 2, 1, 2]
    assert host(dst.vals).tolist() == [2.0, -2.0, 3.0, -1.0, 5.0, 4.0, 1.0]
    ptrs = (dst.pattern.row_ptr.data_ptr(), dst.pattern.col_ind.data_ptr(), dst.vals.data_ptr())
    src.vals.copy_(dev(np.array([-1.0, 2.0, 0.5, -3.0, 4.0, 1.0, -2.0])))
    again = A.transpose(src, dst)
    assert again is dst
    assert ptrs == (dst.pattern.row_ptr.data_ptr(), dst.pattern.col_ind.data_ptr(),
                    dst.vals.data_ptr())
    assert host(dst.vals).tolist() == [-1.0, 4.0, 0.5, 2.0, 1.0, -3.0, -2.0]
    with pytest.raises(A.GbfemError, match="in-place"):
        A.transpose(src, src)


def test_csr_transpose_of_taylor_hood_jacobian():
    import scipy.sparse as sp
    c3, k3 = meshes.jittered_tri(10, seed=4)
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    m = gpu_map(nd, nd, offs, dofs, offs, dofs)
    res = torch.zeros(nd, dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(m.pattern())
    A.assembleTaylorHood(m, dev(cp2), dev(conn6, torch.int32), 1e-2,
                         dev(meshes.cavity_state(cp2, nv, seed=4)), res, jac)
    jt = A.transpose(jac)
    ref = jac.to_scipy().T.tocsr()
    ref.sort_indices()
    assert np.array_equal(host(jt.pattern.row_ptr), ref.indptr)
    assert np.array_equal(host(jt.pattern.col_ind), ref.indices)
    assert np.array_equal(host(jt.vals), ref.data)
    # A^T x through the explicit transpose equals matvecT
    x = dev(np.random.default_rng(4).standard_normal(nd))
    y1 = torch.zeros(nd, dtype=torch.float64, device="cuda")
    y2 = torch.zeros(nd, dtype=torch.float64, device="cuda")
    A.matvec(jt, x, y1)
    A.matvecT(jac, x, y2)
    assert rel_inf(host(y1), host(y2)) <= 1e-14
    assert isinstance(ref, sp.csr_matrix)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32_quad", 1e-6), ("mixed", 1e-6),
                                           ("double_float", 1e-12)])
def test_taylor_hood_state_vjp_matches_oracle(precision, tol):
    """J(u)^T lam without forming J, against the oracle's J transposed."""
    c3, k3 = meshes.jittered_tri(12, seed=21)
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    state = meshes.cavity_state(cp2, nv, seed=21)
    lam = np.random.default_rng(21).standard_normal(nd)
    m = gpu_map(nd, nd, offs, dofs, offs, dofs)
    g = torch.full((nd,), 3.0, dtype=torch.float64, device="cuda")
    A.vjpTaylorHood(m, dev(cp2), dev(conn6, torch.int32), 1e-2, dev(state), dev(lam), g,
                    precision=precision)
    om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    _, rvals = orc.assemble_th_ns(om, cp2, conn6, 1e-2, state)
    ref = orc.matvec_t(om.row_ptr, om.col_ind, rvals, lam, nd)
    assert rel_inf(host(g), ref) <= tol


@pytest.mark.parametrize("precision,det", [("fp64", False), ("fp32_quad", False), ("mixed", False),
                                           ("fp32_quad", True), ("double_float", False)])
def test_taylor_hood_degenerate_element_is_reported(precision, det):
    """A zero-area element is reported through the map's status word (femx
    throws "Singular 2D Jacobian." from ElementValues::invJacobian) and adds
    nothing; the other elements are assembled."""
    c3, k3 = meshes.structured_tri(4)
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    cp2 = cp2.copy()
    a, b = conn6[5][0], conn6[5][1]
    cp2[b] = cp2[a]  # collapse an edge of element 5 (and of its neighbours)
    state = meshes.cavity_state(cp2, nv, seed=2)
    m = gpu_map(nd, nd, offs, dofs, offs, dofs)
    res = torch.zeros(nd, dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(m.pattern())
    A.assembleTaylorHood(m, dev(cp2), dev(conn6, torch.int32), 1e-2, dev(state), res, jac,
                         precision=precision, deterministic=det)
    with pytest.raises(A.GbfemError, match="Singular 2D Jacobian"):
        m.check()
    m.check()
    assert torch.isfinite(res).all() and torch.isfinite(jac.vals).all()
    if not det:
        # the state VJP reports the same element
        g = torch.zeros(nd, dtype=torch.float64, device="cuda")
        lam = dev(np.random.default_rng(2).standard_normal(nd))
        A.vjpTaylorHood(m, dev(cp2), dev(conn6, torch.int32), 1e-2, dev(state), lam, g,
                        precision=precision)
        with pytest.raises(A.GbfemError, match="Singular 2D Jacobian"):
            m.check()
        assert torch.isfinite(g).all()


def test_navier_degenerate_element_is_reported():
    coords, conn = meshes.structured_tri(4)
    coords = coords.copy()
    coords[conn[3][1]] = coords[conn[3][0]]
    n = coords.shape[0]
    offs, dofs, nd = meshes.navier_elem_dofs(conn, n)
    m = gpu_map(nd, nd, offs, dofs, offs, dofs)
    res = torch.zeros(nd, dtype=torch.float64, device="cuda")
    z = torch.zeros(2 * nd, dtype=torch.float64, device="cuda")
    A.assembleNavier(m, dev(coords), dev(conn, torch.int32), 1.0, 1e-2, 0.1, 1, z,
                     z[:nd].clone(), res)
    with pytest.raises(A.GbfemError, match="Singular 2D Jacobian"):
        m.check()
    out = torch.zeros(2 * nd, dtype=torch.float64, device="cuda")
    A.vjpNavierHist(m, dev(coords), dev(conn, torch.int32), 1.0, 1e-2, 0.1, 1, z, z[:nd].clone(),
                    z[:nd].clone(), out)
    with pytest.raises(A.GbfemError, match="Singular 2D Jacobian"):
        m.check()


@pytest.mark.parametrize("precision", ["fp64", "fp32_quad", "mixed"])
def test_taylor_hood_odd_element_count_matches_oracle(precision):
    """An element count that fills neither the 8-element blocks nor the two
    element halves of the last warp (the lanes of the missing element still
    take part in the warp-wide shuffles of the geometry stage)."""
    c3, k3 = meshes.jittered_tri(7, seed=4)
    k3 = k3[:-3]                                   # 95 triangles
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    assert conn6.shape[0] % 2 == 1
    state = meshes.cavity_state(cp2, nv, seed=6)
    om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    rres, rvals = orc.assemble_th_ns(om, cp2, conn6, 1e-2, state)
    tol_j, tol_r = {"fp64": (TOL64, TOL64), "fp32_quad": (TOL32, TOL32),
                    "mixed": (TOL32, TOL64)}[precision]
    _, res, vals = th_gpu(cp2, conn6, dofs, nd, 1e-2, state, precision)
    assert rel_inf(res, rres) <= tol_r
    assert rel_inf(vals, rvals) <= tol_j


@pytest.mark.parametrize("precision", ["fp64", "fp32_quad"])
def test_taylor_hood_connectivity_out_of_range_is_reported(precision):
    """A P2 node index past the coordinate array is reported through the
    status word (no coordinate is read for that element) and the element
    adds nothing; the others are assembled."""
    c3, k3 = meshes.structured_tri(4)
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    bad = conn6.copy()
    bad[9][4] = cp2.shape[0] + 5                   # an edge node of element 9
    state = meshes.cavity_state(cp2, nv, seed=1)
    m = gpu_map(nd, nd, offs, dofs, offs, dofs)
    res = torch.zeros(nd, dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(m.pattern())
    A.assembleTaylorHood(m, dev(cp2), dev(bad, torch.int32), 1e-2, dev(state), res, jac,
                         precision=precision)
    with pytest.raises(A.GbfemError, match="connectivity is out of range"):
        m.check()
    # the oracle: the whole mesh minus element 9 alone (scattered into the
    # whole mesh's pattern, which element 9 still shapes)
    om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    rres, rvals = orc.assemble_th_ns(om, cp2, conn6, 1e-2, state)
    d9 = dofs[15 * 9:15 * 10].copy()
    o9 = np.array([0, 15], dtype=np.int32)
    om9 = orc.AssemblyMap(nd, nd, o9, d9, o9, d9)
    r9, v9 = orc.assemble_th_ns(om9, cp2, conn6[9:10], 1e-2, state)
    rres = rres - r9
    for r in np.unique(d9):
        full = {int(c): k for k, c in enumerate(om.col_ind[om.row_ptr[r]:om.row_ptr[r + 1]],
                                                  start=int(om.row_ptr[r]))}
        for k in range(om9.row_ptr[r], om9.row_ptr[r + 1]):
            rvals[full[int(om9.col_ind[k])]] -= v9[k]
    tol = TOL64 if precision == "fp64" else TOL32
    assert rel_inf(host(res), rres) <= tol
    assert rel_inf(host(jac.vals), rvals) <= tol


# ------------------------------------------------ coloured (atomic-free) assembly

@pytest.mark.parametrize("precision,tol", [("fp64", TOL64), ("fp32_quad", TOL32),
                                           ("mixed", TOL32)])
def test_p1_coloured_assembly_matches_oracle_and_repeats_bitwise(precision, tol):
    """Coloured assembly: no two elements of a colour share a DOF, colours run
    one after another with plain adds; residual, Jacobian and both VJPs
    against the oracle, and bitwise equal over repeated calls."""
    coords, conn = meshes.jittered_tri(30, seed=31)
    m, om = p1_setup(coords, conn)
    nc = m.enableColouring()
    assert 3 <= nc <= 16
    n, e = coords.shape[0], conn.shape[0]
    rng = np.random.default_rng(31)
    kappa, u, lam = np.exp(rng.standard_normal(e)), rng.standard_normal(n), rng.standard_normal(n)
    f = meshes.fourier_source(coords, 2)
    q = orc.P1Quad(coords, conn)
    rres, rvals = orc.assemble_p1_kappa(om, q, kappa, f, u)
    rgu, rgm = orc.vjp_p1_kappa(om, q, kappa, u, lam)
    outs = []
    for _ in range(2):
        res = torch.full((n,), 5.0, dtype=torch.float64, device="cuda")
        jac = A.CsrMatrix(m.pattern(), torch.full((m.pattern().nnz,), 2.0, dtype=torch.float64,
                                                  device="cuda"))
        A.assembleP1Kappa(m, dev(coords), dev(kappa), dev(f), dev(u), res, jac,
                          precision=precision, coloured=True)
        g_u = torch.zeros(n, dtype=torch.float64, device="cuda")
        g_m = torch.zeros(e, dtype=torch.float64, device="cuda")
        A.vjpP1Kappa(m, dev(coords), dev(kappa), dev(u), dev(lam), g_u, g_m,
                     precision=precision, coloured=True)
        m.check()
        outs.append((res, jac.vals, g_u, g_m))
    res, vals, g_u, g_m = (host(t) for t in outs[0])
    assert rel_inf(vals, rvals) <= tol
    assert rel_inf(res, rres) <= (TOL64 if precision == "mixed" else tol)
    assert rel_inf(g_u, rgu) <= (TOL64 if precision != "fp32_quad" else TOL32)
    assert rel_inf(g_m, rgm) <= (TOL64 if precision != "fp32_quad" else TOL32)
    assert all(torch.equal(a, b) for a, b in zip(outs[0], outs[1]))


@pytest.mark.parametrize("precision,tol_j,tol_r", TH_PRECS)
def test_taylor_hood_coloured_assembly_matches_oracle_and_repeats_bitwise(precision, tol_j,
                                                                           tol_r):
    c3, k3 = meshes.jittered_tri(14, seed=41)
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    state = meshes.cavity_state(cp2, nv, seed=41)
    lam = np.random.default_rng(41).standard_normal(nd)
    m = gpu_map(nd, nd, offs, dofs, offs, dofs)
    assert m.enableColouring() >= 3
    om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    rres, rvals = orc.assemble_th_ns(om, cp2, conn6, 1e-2, state)
    gref = orc.matvec_t(om.row_ptr, om.col_ind, rvals, lam, nd)
    outs = []
    for _ in range(2):
        res = torch.full((nd,), 5.0, dtype=torch.float64, device="cuda")
        jac = A.CsrMatrix(m.pattern(), torch.full((m.pattern().nnz,), 2.0, dtype=torch.float64,
                                                  device="cuda"))
        A.assembleTaylorHood(m, dev(cp2), dev(conn6, torch.int32), 1e-2, dev(state), res, jac,
                             precision=precision, coloured=True)
        r_only = torch.full((nd,), 3.0, dtype=torch.float64, device="cuda")
        A.assembleTaylorHood(m, dev(cp2), dev(conn6, torch.int32), 1e-2, dev(state), r_only,
                             None, precision=precision, coloured=True)
        g = torch.zeros(nd, dtype=torch.float64, device="cuda")
        A.vjpTaylorHood(m, dev(cp2), dev(conn6, torch.int32), 1e-2, dev(state), dev(lam), g,
                        precision=precision, coloured=True)
        m.check()
        outs.append((res, jac.vals, r_only, g))
    res, vals, r_only, g = (host(t) for t in outs[0])
    assert rel_inf(vals, rvals) <= tol_j
    assert rel_inf(res, rres) <= tol_r
    assert rel_inf(r_only, rres) <= (TOL32 if precision == "fp32_quad" else TOL64)
    assert rel_inf(g, gref) <= (TOL64 if precision in ("fp64", "double_float") else TOL32)
    assert all(torch.equal(a, b) for a, b in zip(outs[0], outs[1]))


def test_coloured_assembly_needs_a_coloured_map():
    coords, conn = meshes.jittered_tri(6, seed=3)
    m, om = p1_setup(coords, conn)
    n, e = coords.shape[0], conn.shape[0]
    res = torch.zeros(n, dtype=torch.float64, device="cuda")
    with pytest.raises(A.GbfemError, match="enable_colouring"):
        A.assembleP1Kappa(m, dev(coords), dev(np.ones(e)), None, dev(np.zeros(n)), res,
                          coloured=True)
