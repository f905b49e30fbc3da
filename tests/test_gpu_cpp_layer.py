"""The C++ layer and the header-only user-operator assembly, from a CUDA
program compiled here with nvcc (tests/cpp/generic_assembly_test.cu).

* femx's own known answers for the generic assembly loop (steady, rectangular
  local layouts, time step with history blocks; runBackendAssemblyTests.cpp)
  with user operators of the same definition, run on the GPU;
* a user operator restating femx's PoissonComponents::evalRow and the
  KappaPoissonP1 tag (kappa = 1) against the CPU oracle, then the C++
  BoundaryMap calls (replaceRows, replaceRes, prepareForwardSolve) and
  matvec against the oracle on the same data.
"""
import os
import subprocess

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from conftest import rel_inf  # noqa: E402
from femx_gb300 import meshes  # noqa: E402
from oracle import pyoracle as orc  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "generic_assembly_test.cu")
LIBDIR = os.path.join(ROOT, "femx_gb300")


@pytest.fixture(scope="module")
def program(tmp_path_factory):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from femx_gb300 import build
    build.build()
    out = str(tmp_path_factory.mktemp("cpp") / "generic_assembly_test")
    cmd = ["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
           "-I" + os.path.join(ROOT, "include"), SRC, "-L" + LIBDIR, "-lgbfem",
           "-Xlinker", "-rpath," + LIBDIR, "-o", out]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


def test_known_answers_of_the_generic_loop(program):
    p = subprocess.run([program], capture_output=True, text=True, timeout=120)
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("KAT ")]
    assert len(lines) == 4, p.stdout + p.stderr
    assert all(ln.endswith(" PASS") for ln in lines), p.stdout
    assert p.returncode == 0, p.stderr


def test_user_operator_tag_and_boundary_calls_match_the_oracle(program, tmp_path):
    coords, conn = meshes.jittered_tri(24, seed=11)
    n, e = coords.shape[0], conn.shape[0]
    rng = np.random.default_rng(11)
    u = rng.standard_normal(n)
    bdofs = meshes.dirichlet_dofs(coords, meshes.boundary_nodes(coords)).astype(np.int32)
    g = rng.standard_normal(len(bdofs))
    d = str(tmp_path)
    np.ascontiguousarray(coords, dtype=np.float64).tofile(os.path.join(d, "coords.f64"))
    np.ascontiguousarray(conn, dtype=np.int32).tofile(os.path.join(d, "conn.i32"))
    u.tofile(os.path.join(d, "state.f64"))
    bdofs.tofile(os.path.join(d, "bdofs.i32"))
    g.tofile(os.path.join(d, "g.f64"))
    p = subprocess.run([program, d, str(n), str(e), str(len(bdofs))], capture_output=True,
                       text=True, timeout=120)
    assert p.returncode == 0, p.stdout + p.stderr

    def rd(name, dt):
        return np.fromfile(os.path.join(d, name), dtype=dt)

    offs, dofs = meshes.scalar_elem_dofs(conn)
    om = orc.AssemblyMap(n, n, offs, dofs, offs, dofs)
    assert np.array_equal(rd("row_ptr.i32", np.int32), om.row_ptr)
    assert np.array_equal(rd("col_ind.i32", np.int32), om.col_ind)
    q = orc.P1Quad(coords, conn)
    rres, rvals = orc.assemble_p1_kappa(om, q, np.ones(e), None, u)
    for tag in ("generic", "tag"):
        assert rel_inf(rd(f"res_{tag}.f64", np.float64), rres) <= 1e-12, tag
        assert rel_inf(rd(f"vals_{tag}.f64", np.float64), rvals) <= 1e-12, tag
    # BoundaryMap calls on the tag matrix, oracle on the oracle's matrix
    ob = orc.BoundaryMap(bdofs, om.row_ptr, om.col_ind)
    assert rel_inf(rd("rows_vals.f64", np.float64), ob.replace_rows(rvals, 1.0)) <= 1e-12
    assert rel_inf(rd("res_bc.f64", np.float64), ob.replace_res(u, g, rres)) <= 1e-12
    sv, rhs = ob.prepare_forward_solve(rvals, -rres, g)
    assert rel_inf(rd("solve_vals.f64", np.float64), sv) <= 1e-12
    assert rel_inf(rd("rhs.f64", np.float64), rhs) <= 1e-12
    y = orc.matvec(om.row_ptr, om.col_ind, rvals, u)
    assert rel_inf(rd("y.f64", np.float64), y) <= 1e-12


def test_navier_tag_through_the_cpp_layer(program, tmp_path):
    from conftest import load_golden
    g = load_golden("ns_gls_jit5_s3")
    nd = int(g["num_dofs"][0])
    n, e = g["coords"].shape[0], g["conn"].shape[0]
    d = str(tmp_path)
    adj = np.random.default_rng(3).standard_normal(nd)
    np.ascontiguousarray(g["coords"], dtype=np.float64).tofile(os.path.join(d, "coords.f64"))
    np.ascontiguousarray(g["conn"], dtype=np.int32).tofile(os.path.join(d, "conn.i32"))
    np.ascontiguousarray(g["res_dofs"], dtype=np.int32).tofile(os.path.join(d, "dofs.i32"))
    g["hist"].tofile(os.path.join(d, "hist.f64"))
    g["nxt"].tofile(os.path.join(d, "nxt.f64"))
    adj.tofile(os.path.join(d, "adj.f64"))
    np.array([g["rho"][0], g["mu"][0], g["dt"][0], float(g["step"][0])]).tofile(
        os.path.join(d, "prm.f64"))
    p = subprocess.run([program, "navier", d, str(n), str(e)], capture_output=True, text=True,
                       timeout=120)
    assert p.returncode == 0, p.stdout + p.stderr

    def rd(name):
        return np.fromfile(os.path.join(d, name), dtype=np.float64)

    assert rel_inf(rd("ns_res.f64"), g["res"]) <= 1e-12
    assert rel_inf(rd("ns_vals.f64"), g["vals"]) <= 1e-12
    assert rel_inf(rd("ns_res_hist.f64"), g["res"]) <= 1e-12
    assert not rd("ns_vals_hist.f64").any()
    om = orc.AssemblyMap(nd, nd, g["res_offsets"], g["res_dofs"], g["state_offsets"],
                         g["state_dofs"])
    q = orc.P1Quad(g["coords"], g["conn"], order=2)
    ref = orc.vjp_navier_hist(om, q, g["rho"][0], g["mu"][0], g["dt"][0], int(g["step"][0]),
                              g["hist"], g["nxt"], adj)
    assert rel_inf(rd("ns_vjp.f64"), ref) <= 1e-12
