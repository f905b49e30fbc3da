"""Gmsh ingestion (gbfem_mesh_read_gmsh) against femx's own GmshReader run on
the same files (golden gmsh_v2 / gmsh_v4: the file text and femx's parsed
mesh), and femx's errors. Host code: runs without a GPU; the last test
assembles on the read mesh on the GPU."""
import os

import numpy as np
import pytest

from conftest import load_golden, rel_inf
from femx_gb300 import build

build.build()
from femx_gb300 import mesh_io, meshes  # noqa: E402
from femx_gb300._lib import GbfemError  # noqa: E402


def write(tmp_path, name, data):
    p = os.path.join(str(tmp_path), name)
    with open(p, "wb") as fh:
        fh.write(bytes(data))
    return p


@pytest.mark.parametrize("case", ["gmsh_v2", "gmsh_v4"])
def test_reader_matches_femx_gmsh_reader(case, tmp_path):
    g = load_golden(case)
    m = mesh_io.read_gmsh(write(tmp_path, "mesh.msh", g["msh"]))
    assert m.dim == int(g["dim"][0])
    assert np.array_equal(m.coords.reshape(-1), g["coords"])
    assert np.array_equal(m.conn.reshape(-1), g["conn"])
    assert np.array_equal(m.elem_etag, g["etag"]) and np.array_equal(m.elem_ptag, g["ptag"])
    assert np.array_equal(m.facet_conn.reshape(-1), g["fconn"])
    assert np.array_equal(m.facet_etag, g["fetag"]) and np.array_equal(m.facet_ptag, g["fptag"])
    names = {}
    for line in bytes(g["names"]).decode().splitlines():
        d, t, nm = line.split(" ", 2)
        names[(int(d), int(t))] = nm
    assert m.names == names


def test_reader_matches_femx_on_a_reference_data_mesh():
    """A real unstructured mesh of the reference's own data (data/meshes,
    Gmsh 4.1 with entities and physical groups) read by our reader against
    femx's GmshReader output stored in the fixture real_sq_mesh. Needs the
    reference tree, named by FEMX_REFERENCE (skipped where it is absent)."""
    root = os.environ.get("FEMX_REFERENCE")
    g = load_golden("real_sq_mesh")
    path = os.path.join(root or "", "data", "meshes", bytes(g["source"]).decode())
    if not root or not os.path.exists(path):
        pytest.skip("the reference tree is not available (set FEMX_REFERENCE)")
    m = mesh_io.read_gmsh(path)
    assert m.dim == int(g["dim"][0])
    assert np.array_equal(m.coords.reshape(-1), g["coords"])
    assert np.array_equal(m.conn.reshape(-1), g["conn"])
    assert np.array_equal(m.elem_etag, g["etag"]) and np.array_equal(m.elem_ptag, g["ptag"])
    assert np.array_equal(m.facet_conn.reshape(-1), g["fconn"])
    assert np.array_equal(m.facet_etag, g["fetag"]) and np.array_equal(m.facet_ptag, g["fptag"])


@pytest.mark.parametrize("text,msg", [
    ("$MeshFormat\n4.1 1 8\n$EndMeshFormat\n", "only ASCII"),
    ("$MeshFormat\n3.0 0 8\n$EndMeshFormat\n", "Gmsh 2.x and 4.x"),
    ("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n1\n1 0 0 0\n$EndNodes\n"
     "$Elements\n1\n1 2 0 1 2 3\n$EndElements\n", "unknown node 2"),
    ("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n2\n1 0 0 0\n2 1 0 0\n$EndNodes\n"
     "$Elements\n1\n1 1 0 1 2\n$EndElements\n", "no supported volume or surface"),
    ("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Elements\n1\n1 9 0 1 2 3\n$EndElements\n",
     "unsupported elem type 9"),
    ("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Foo\n1 2 3\n", "missing \\$EndFoo"),
])
def test_reader_errors_match_femx(text, msg, tmp_path):
    with pytest.raises(GbfemError, match=msg):
        mesh_io.read_gmsh(write(tmp_path, "bad.msh", text.encode()))
    with pytest.raises(GbfemError, match="failed to open"):
        mesh_io.read_gmsh(os.path.join(str(tmp_path), "missing.msh"))


def test_mixed_shapes_are_rejected(tmp_path):
    text = ("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n4\n1 0 0 0\n2 1 0 0\n3 1 1 0\n"
            "4 0 1 0\n$EndNodes\n$Elements\n2\n1 2 0 1 2 3\n2 3 0 1 2 3 4\n$EndElements\n")
    with pytest.raises(GbfemError, match="mixing element shapes"):
        mesh_io.read_gmsh(write(tmp_path, "mixed.msh", text.encode()))


@pytest.mark.gpu
def test_assembly_on_a_read_mesh_matches_the_oracle(tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from femx_gb300 import assembly as A
    from oracle import pyoracle as orc
    coords, conn = meshes.jittered_tri(20, seed=71)
    path = os.path.join(str(tmp_path), "m.msh")
    meshes.write_gmsh(path, coords, conn, version=4, seed=72)
    m = mesh_io.read_gmsh(path)
    c2 = m.coords[:, :2].copy()
    n, e = c2.shape[0], m.conn.shape[0]
    offs, dofs = meshes.scalar_elem_dofs(m.conn)
    cd, kd = m.device()
    amap = A.makeAssemblyMap(n, n, torch.from_numpy(offs).cuda(), torch.from_numpy(dofs).cuda(),
                             torch.from_numpy(offs).cuda(), torch.from_numpy(dofs).cuda())
    rng = np.random.default_rng(7)
    u, kappa = rng.standard_normal(n), np.exp(rng.standard_normal(e))
    res = torch.zeros(n, dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(amap.pattern())
    A.assembleP1Kappa(amap, cd, torch.from_numpy(kappa).cuda(), None,
                      torch.from_numpy(u).cuda(), res, jac)
    om = orc.AssemblyMap(n, n, offs, dofs, offs, dofs)
    rres, rvals = orc.assemble_p1_kappa(om, orc.P1Quad(c2, m.conn), kappa, None, u)
    assert rel_inf(res.cpu().numpy(), rres) <= 1e-12
    assert rel_inf(jac.vals.cpu().numpy(), rvals) <= 1e-12
    # the Dirichlet set from the physical boundary groups equals the geometric one
    bnd = np.unique(m.facet_conn.reshape(-1))
    assert np.array_equal(bnd, np.flatnonzero(meshes.boundary_nodes(c2)))
