"""femx's own GLS Navier-Stokes time operator (NavierOperator) on the GPU.

* residual and next-state Jacobian against the reference library's own
  operator and time assemble (golden vectors tests/golden/ns_gls_*.npz),
  and against the oracle on larger jittered meshes (1e-12);
* the history VJP (femx: Enzyme; here reverse mode by hand) against the
  oracle's exact dual-number VJP, at step 0, with AB2, and at rest;
* femx's input checks.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from conftest import load_golden, rel_inf  # noqa: E402
from femx_gb300 import assembly as A  # noqa: E402
from femx_gb300 import meshes  # noqa: E402
from oracle import pyoracle as orc  # noqa: E402

CASES = ["ns_gls_jit5_s0", "ns_gls_jit5_s3", "ns_gls_still4", "real_sq_ns"]


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


def gpu_setup(coords, conn, offs, dofs, nd):
    m = A.makeAssemblyMap(nd, nd, dev(offs, torch.int32), dev(dofs, torch.int32),
                          dev(offs, torch.int32), dev(dofs, torch.int32))
    return m, dev(coords, torch.float64), dev(conn, torch.int32)


def gpu_assemble(m, coords, conn, prm, hist, nxt, jac=True):
    nd = m.numRes()
    res = torch.full((nd,), 9.0, dtype=torch.float64, device="cuda")
    mat = A.CsrMatrix(m.pattern()) if jac else None
    A.assembleNavier(m, coords, conn, *prm, dev(hist), dev(nxt), res, mat)
    m.check()
    return host(res), (host(mat.vals) if jac else None)


@pytest.mark.parametrize("case", CASES)
def test_navier_matches_reference_golden(case):
    g = load_golden(case)
    nd = int(g["num_dofs"][0])
    m, coords, conn = gpu_setup(g["coords"], g["conn"], g["res_offsets"], g["res_dofs"], nd)
    assert np.array_equal(host(m.pattern().row_ptr), g["row_ptr"])
    assert np.array_equal(host(m.pattern().col_ind), g["col_ind"])
    prm = (g["rho"][0], g["mu"][0], g["dt"][0], int(g["step"][0]))
    res, vals = gpu_assemble(m, coords, conn, prm, g["hist"], g["nxt"])
    assert rel_inf(res, g["res"]) <= 1e-12
    assert rel_inf(vals, g["vals"]) <= 1e-12
    res_only, _ = gpu_assemble(m, coords, conn, prm, g["hist"], g["nxt"], jac=False)
    assert rel_inf(res_only, g["res"]) <= 1e-12


@pytest.mark.parametrize("step", [0, 4])
def test_navier_matches_oracle_on_a_larger_mesh(step):
    coords, conn = meshes.jittered_tri(24, seed=17)
    n = coords.shape[0]
    offs, dofs, nd = meshes.navier_elem_dofs(conn, n)
    rng = np.random.default_rng(17 + step)
    hist = np.concatenate([meshes.stream_velocity(coords, seed=3).reshape(-1),
                           rng.standard_normal(n),
                           meshes.stream_velocity(coords, seed=4).reshape(-1),
                           rng.standard_normal(n)])
    nxt = rng.standard_normal(nd)
    prm = (1.0, 2e-3, 0.01, step)
    m, c, k = gpu_setup(coords, conn, offs, dofs, nd)
    res, vals = gpu_assemble(m, c, k, prm, hist, nxt)
    om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    q = orc.P1Quad(coords, conn, order=2)
    rres, rvals = orc.assemble_navier(om, q, *prm, hist, nxt)
    assert rel_inf(res, rres) <= 1e-12
    assert rel_inf(vals, rvals) <= 1e-12


@pytest.mark.parametrize("case", CASES)
def test_history_vjp_matches_exact_derivative(case):
    g = load_golden(case)
    nd = int(g["num_dofs"][0])
    m, coords, conn = gpu_setup(g["coords"], g["conn"], g["res_offsets"], g["res_dofs"], nd)
    prm = (g["rho"][0], g["mu"][0], g["dt"][0], int(g["step"][0]))
    adj = np.random.default_rng(8).standard_normal(nd)
    out = torch.full((2 * nd,), 5.0, dtype=torch.float64, device="cuda")
    A.vjpNavierHist(m, coords, conn, *prm, dev(g["hist"]), dev(g["nxt"]), dev(adj), out)
    om = orc.AssemblyMap(nd, nd, g["res_offsets"], g["res_dofs"], g["state_offsets"],
                         g["state_dofs"])
    q = orc.P1Quad(g["coords"], g["conn"], order=2)
    ref = orc.vjp_navier_hist(om, q, *prm, g["hist"], g["nxt"], adj)
    got = host(out)
    assert rel_inf(got, ref) <= 1e-12
    if int(g["step"][0]) == 0:
        assert not got[nd:].any()  # no AB2: the older state does not enter


def test_history_vjp_on_a_larger_mesh_matches_finite_differences():
    coords, conn = meshes.jittered_tri(16, seed=23)
    n = coords.shape[0]
    offs, dofs, nd = meshes.navier_elem_dofs(conn, n)
    rng = np.random.default_rng(23)
    hist = rng.standard_normal(2 * nd)
    nxt = rng.standard_normal(nd)
    adj = rng.standard_normal(nd)
    prm = (1.0, 1e-2, 0.02, 2)
    m, c, k = gpu_setup(coords, conn, offs, dofs, nd)
    out = torch.zeros(2 * nd, dtype=torch.float64, device="cuda")
    A.vjpNavierHist(m, c, k, *prm, dev(hist), dev(nxt), dev(adj), out)
    got = host(out)
    om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    q = orc.P1Quad(coords, conn, order=2)
    assert rel_inf(got, orc.vjp_navier_hist(om, q, *prm, hist, nxt, adj)) <= 1e-12
    for _ in range(8):
        dh = rng.standard_normal(2 * nd)
        h = 1e-6
        rp, _ = orc.assemble_navier(om, q, *prm, hist + h * dh, nxt, jac=False)
        rm, _ = orc.assemble_navier(om, q, *prm, hist - h * dh, nxt, jac=False)
        fd = float((rp - rm) @ adj) / (2 * h)
        assert abs(fd - got @ dh) <= 1e-6 * max(1.0, abs(fd))


def test_navier_input_checks():
    coords, conn = meshes.structured_tri(3)
    n = coords.shape[0]
    offs, dofs, nd = meshes.navier_elem_dofs(conn, n)
    m, c, k = gpu_setup(coords, conn, offs, dofs, nd)
    res = torch.zeros(nd, dtype=torch.float64, device="cuda")
    hist, nxt = torch.zeros(2 * nd, dtype=torch.float64, device="cuda"), \
        torch.zeros(nd, dtype=torch.float64, device="cuda")
    with pytest.raises(A.GbfemError, match="positive"):
        A.assembleNavier(m, c, k, 1.0, 1e-2, 0.0, 0, hist, nxt, res)
    p_offs, p_dofs = meshes.scalar_elem_dofs(conn)
    mp = A.makeAssemblyMap(n, n, dev(p_offs, torch.int32), dev(p_dofs, torch.int32),
                           dev(p_offs, torch.int32), dev(p_dofs, torch.int32))
    with pytest.raises(A.GbfemError, match="nine DOFs"):
        A.assembleNavier(mp, c, k, 1.0, 1e-2, 0.1, 0, torch.zeros(2 * n, dtype=torch.float64,
                                                                  device="cuda"),
                         torch.zeros(n, dtype=torch.float64, device="cuda"),
                         torch.zeros(n, dtype=torch.float64, device="cuda"))
