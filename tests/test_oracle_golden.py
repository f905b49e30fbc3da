"""Pin the CPU oracle to the reference before trusting it.

Two sources of truth:
  * the known-answer vectors written in the reference's own unit tests
    (runBackendAssemblyTests.cpp:162-226, runLinalgTests.cpp:235-270,
    runBackendStateTests.cpp:80-117, runCudaAssemblyTests.cu:247-322),
    restated below as literals, and
  * golden dumps of the reference library itself (tests/golden/*.npz, made by
    tests/golden/make_golden.py from the reference sources).
"""
import numpy as np
import pytest

from conftest import rel_inf
from femx_gb300 import meshes
from oracle import pyoracle as orc

DENSE_ROW_PTR = np.array([0, 3, 6, 9], np.int32)
DENSE_COL_IND = np.array([0, 1, 2, 0, 1, 2, 0, 1, 2], np.int32)
DENSE_VALS = np.array([4.0, 1.0, 2.0, 3.0, 5.0, 6.0, 7.0, 8.0, 9.0])


def test_shared_element_map_known_answer(golden):
    # runLinalgTests.cpp:235-270
    offs = np.array([0, 2, 4], np.int32)
    dofs = np.array([0, 1, 1, 2], np.int32)
    m = orc.AssemblyMap(3, 3, offs, dofs, offs, dofs)
    assert m.nnz == 7 and m.jac_nnz == 8
    np.testing.assert_array_equal(m.row_ptr, [0, 2, 5, 7])
    np.testing.assert_array_equal(m.col_ind, [0, 1, 0, 1, 2, 1, 2])
    np.testing.assert_array_equal(m.jac_map, [0, 1, 2, 3, 3, 4, 5, 6])
    np.testing.assert_array_equal(m.jac_offsets, [0, 4, 8])
    kat = golden("kat")
    np.testing.assert_array_equal(m.row_ptr, kat["shared_row_ptr"])
    np.testing.assert_array_equal(m.col_ind, kat["shared_col_ind"])
    np.testing.assert_array_equal(m.jac_map, kat["shared_jac_map"])


def test_rectangular_map_known_answer(golden):
    # runBackendAssemblyTests.cpp:162-188
    m = orc.AssemblyMap(2, 2, [0, 2, 3], [0, 1, 1], [0, 1, 3], [0, 0, 1])
    np.testing.assert_array_equal(m.row_ptr, [0, 1, 3])
    np.testing.assert_array_equal(m.col_ind, [0, 0, 1])
    np.testing.assert_array_equal(m.jac_map, [0, 1, 1, 2])
    np.testing.assert_array_equal(m.jac_offsets, [0, 2, 4])
    kat = golden("kat")
    np.testing.assert_array_equal(m.jac_map, kat["rect_jac_map"])


def test_map_rejects_out_of_range_dofs():
    with pytest.raises(orc.OracleError, match="residual DOF is out of range"):
        orc.AssemblyMap(2, 2, [0, 1], [2], [0, 1], [0])
    with pytest.raises(orc.OracleError, match="state DOF is out of range"):
        orc.AssemblyMap(2, 2, [0, 1], [0], [0, 1], [-1])


@pytest.mark.parametrize("bcs,g,tag", [([1], [2.0], "bc1_"), ([0, 2], [2.0, -1.0], "bc02_")])
def test_boundary_known_answers(golden, bcs, g, tag):
    # runBackendStateTests.cpp:80-117 and runCudaAssemblyTests.cu:247-322
    kat = golden("kat")
    b = orc.BoundaryMap(bcs, DENSE_ROW_PTR, DENSE_COL_IND)
    np.testing.assert_array_equal(b.replace_rows(DENSE_VALS, 1.0), kat[tag + "rows1"])
    np.testing.assert_array_equal(b.replace_rows(DENSE_VALS, 0.0), kat[tag + "rows0"])
    np.testing.assert_array_equal(
        b.replace_res([4.0, 7.0, 9.0], g, [10.0, 20.0, 30.0]), kat[tag + "res"])
    v, r = b.prepare_forward_solve(DENSE_VALS, [10.0, 20.0, 30.0], g)
    np.testing.assert_array_equal(v, kat[tag + "fwd_vals"])
    np.testing.assert_array_equal(r, kat[tag + "fwd_rhs"])
    if tag == "bc1_":
        np.testing.assert_allclose(v, [4.0, 0.0, 2.0, 0.0, 1.0, 0.0, 7.0, 0.0, 9.0])
        np.testing.assert_allclose(r, [8.0, 2.0, 14.0])


def test_boundary_rejects_duplicates_and_missing_diagonal():
    with pytest.raises(orc.OracleError, match="must be unique"):
        orc.BoundaryMap([1, 1], DENSE_ROW_PTR, DENSE_COL_IND)
    with pytest.raises(orc.OracleError, match="no diagonal entry"):
        orc.BoundaryMap([0], [0, 1, 2], [1, 0])


@pytest.mark.parametrize("case", ["p1_32", "p1_jit9", "real_sq_p1"])
def test_p1_assembly_matches_reference(golden, case):
    g = golden(case)
    offs, dofs = meshes.scalar_elem_dofs(g["conn"])
    n = g["coords"].shape[0]
    m = orc.AssemblyMap(n, n, offs, dofs, offs, dofs)
    np.testing.assert_array_equal(m.row_ptr, g["row_ptr"])
    np.testing.assert_array_equal(m.col_ind, g["col_ind"])
    np.testing.assert_array_equal(m.jac_offsets, g["jac_offsets"])
    np.testing.assert_array_equal(m.jac_map, g["jac_map"])
    q = orc.P1Quad(g["coords"], g["conn"], order=2)
    res, vals = orc.assemble_p1_kappa(m, q, g["kappa"], g["f"], g["u"])
    assert rel_inf(res, g["res"]) <= 1e-14
    assert rel_inf(vals, g["vals"]) <= 1e-14

    # Dirichlet index set: ascending boundary nodes (DirichletBC.cpp:127-146)
    dofs_bc = meshes.dirichlet_dofs(g["coords"], meshes.boundary_nodes(g["coords"]))
    np.testing.assert_array_equal(dofs_bc, g["bc_dofs"])
    b = orc.BoundaryMap(dofs_bc, m.row_ptr, m.col_ind)
    for ours, ref in ((b.bc_rows, "bc_rows"), (b.diag, "bc_diag"),
                      (b.col_offsets, "bc_col_offsets"), (b.col_entries, "bc_col_entries"),
                      (b.col_rows, "bc_col_rows"), (b.bc_mask, "bc_mask")):
        np.testing.assert_array_equal(ours, g[ref])

    np.testing.assert_array_equal(b.replace_rows(vals, 1.0), g["vals_rows1"])
    assert rel_inf(b.replace_res(g["u"], g["bc_vals"], res), g["res_replaced"]) <= 1e-14
    v, r = b.prepare_forward_solve(vals, -res, g["bc_vals"])
    assert rel_inf(v, g["vals_fwd"]) <= 1e-14
    assert rel_inf(r, g["rhs_fwd"]) <= 1e-14

    y = orc.matvec(m.row_ptr, m.col_ind, g["vals"], g["x"])
    np.testing.assert_array_equal(y, g["y_matvec"])
    yt = orc.matvec_t(m.row_ptr, m.col_ind, g["vals"], g["x"], n)
    np.testing.assert_array_equal(yt, g["y_matvec_t"])

    g_u, g_m = orc.vjp_p1_kappa(m, q, g["kappa"], g["u"], g["lam"])
    assert rel_inf(g_u, g["g_u"]) <= 1e-14
    assert rel_inf(g_m, g["g_m"]) <= 1e-14


def test_p1_config1_sizes(golden):
    g = golden("p1_32")
    c = meshes.structured_counts(32)
    assert g["conn"].shape[0] == c["elems"] == 2048
    assert g["coords"].shape[0] == c["nodes"] == 1089
    assert g["row_ptr"][-1] == c["nnz_p1"] == 7361
    assert len(g["bc_dofs"]) == 128


@pytest.mark.parametrize("case", ["th_4", "th_jit3", "real_sq_th"])
def test_taylor_hood_matches_reference_loop(golden, case):
    g = golden(case)
    nd = int(g["num_dofs"])
    e = g["conn6"].shape[0]
    offs = (np.arange(e + 1) * 15).astype(np.int32)
    m = orc.AssemblyMap(nd, nd, offs, g["elem_dofs"], offs, g["elem_dofs"])
    np.testing.assert_array_equal(m.row_ptr, g["row_ptr"])
    np.testing.assert_array_equal(m.col_ind, g["col_ind"])
    if "jac_map" in g:
        np.testing.assert_array_equal(m.jac_map, g["jac_map"])
    res, vals = orc.assemble_th_ns(m, g["coords"], g["conn6"], float(g["nu"]), g["state"])
    assert rel_inf(res, g["res"]) <= 1e-13
    assert rel_inf(vals, g["vals"]) <= 1e-13


def test_taylor_hood_jacobian_matches_finite_differences(golden):
    """The Newton Jacobian is the exact derivative of the residual."""
    g = golden("th_jit3")
    nd = int(g["num_dofs"])
    e = g["conn6"].shape[0]
    offs = (np.arange(e + 1) * 15).astype(np.int32)
    m = orc.AssemblyMap(nd, nd, offs, g["elem_dofs"], offs, g["elem_dofs"])
    nu = float(g["nu"])
    _, vals = orc.assemble_th_ns(m, g["coords"], g["conn6"], nu, g["state"])
    rng = np.random.default_rng(0)
    d = rng.standard_normal(nd)
    h = 1e-6
    rp, _ = orc.assemble_th_ns(m, g["coords"], g["conn6"], nu, g["state"] + h * d)
    rm, _ = orc.assemble_th_ns(m, g["coords"], g["conn6"], nu, g["state"] - h * d)
    fd = (rp - rm) / (2 * h)
    jd = orc.matvec(m.row_ptr, m.col_ind, vals, d)
    assert rel_inf(jd, fd) <= 1e-6


def test_threaded_taylor_hood_loop_matches_serial(golden):
    """The multi-threaded loop (atomic adds, femx's OpenMP NS scheme) gives
    the serial loop's result to rounding."""
    g = golden("th_jit3")
    nd = int(g["num_dofs"])
    e = g["conn6"].shape[0]
    offs = (np.arange(e + 1) * 15).astype(np.int32)
    m = orc.AssemblyMap(nd, nd, offs, g["elem_dofs"], offs, g["elem_dofs"])
    th = orc.THQuad(g["coords"], g["conn6"])
    res1, vals1 = orc.assemble_th_range(m, th, float(g["nu"]), g["state"])
    res4, vals4 = orc.assemble_th_threads(m, th, float(g["nu"]), g["state"], 4)
    assert rel_inf(res4, res1) <= 1e-14
    assert rel_inf(vals4, vals1) <= 1e-14
    assert rel_inf(vals4, g["vals"]) <= 1e-13


NS_CASES = ["ns_gls_jit5_s0", "ns_gls_jit5_s3", "ns_gls_still4", "real_sq_ns"]


def ns_setup(g):
    nd = int(g["num_dofs"][0])
    m = orc.AssemblyMap(nd, nd, g["res_offsets"], g["res_dofs"], g["state_offsets"],
                        g["state_dofs"])
    q = orc.P1Quad(g["coords"], g["conn"], order=2)
    return nd, m, q


@pytest.mark.parametrize("case", NS_CASES)
def test_navier_gls_operator_matches_reference(golden, case):
    """femx's own NS time operator run by the reference library (golden)
    against the restated operator: same map, residual and next-state
    Jacobian."""
    g = golden(case)
    nd, m, q = ns_setup(g)
    np.testing.assert_array_equal(m.row_ptr, g["row_ptr"])
    np.testing.assert_array_equal(m.col_ind, g["col_ind"])
    np.testing.assert_array_equal(m.jac_map, g["jac_map"])
    res, vals = orc.assemble_navier(m, q, g["rho"][0], g["mu"][0], g["dt"][0],
                                    int(g["step"][0]), g["hist"], g["nxt"])
    assert rel_inf(res, g["res"]) <= 1e-13
    assert rel_inf(vals, g["vals"]) <= 1e-13


def test_navier_history_vjp_matches_finite_differences(golden):
    """The dual-number history VJP of the oracle against central
    differences of the restated residual (h = 1e-6), both lags."""
    g = golden("ns_gls_jit5_s3")
    nd, m, q = ns_setup(g)
    args = (g["rho"][0], g["mu"][0], g["dt"][0], int(g["step"][0]))
    rng = np.random.default_rng(5)
    adj = rng.standard_normal(nd)
    vjp = orc.vjp_navier_hist(m, q, *args, g["hist"], g["nxt"], adj)
    for _ in range(6):
        dh = rng.standard_normal(2 * nd)
        h = 1e-6
        rp, _ = orc.assemble_navier(m, q, *args, g["hist"] + h * dh, g["nxt"], jac=False)
        rm, _ = orc.assemble_navier(m, q, *args, g["hist"] - h * dh, g["nxt"], jac=False)
        fd = float((rp - rm) @ adj) / (2 * h)
        assert abs(fd - vjp @ dh) <= 1e-7 * max(1.0, abs(fd))


def test_threaded_navier_loop_matches_serial(golden):
    g = golden("ns_gls_jit5_s3")
    nd, m, q = ns_setup(g)
    args = (g["rho"][0], g["mu"][0], g["dt"][0], int(g["step"][0]), g["hist"], g["nxt"])
    r1, v1 = orc.assemble_navier(m, q, *args)
    r4, v4 = orc.assemble_navier_threads(m, q, *args, 4)
    assert rel_inf(r4, r1) <= 1e-14
    assert rel_inf(v4, v1) <= 1e-14
