"""Generate the golden fixtures in tests/golden/ from the femx reference.

Runs in the development container only (it needs the reference sources):
builds the reference library and driver with oracle/ref/Makefile into
oracle/_ref/, writes seeded inputs, runs the driver and stores inputs and the
reference's outputs as compressed .npz files next to this script.

    python tests/golden/make_golden.py [--ref /path/to/reference]

Cases
  kat          known-answer cases of the reference's unit tests
  p1_32        32x32 structured P1 Poisson, kappa = 1, Fourier source,
               homogeneous Dirichlet on all edges (the CPU-runnable config)
  p1_jit9      9x9 jittered mesh with permuted node/element ids, random
               kappa, u, lam, x and a linear Dirichlet lift g = 0.5 + x - 2y
  th_4         4x4 structured Taylor-Hood P2/P1, random state, nu = 1e-2
  th_jit3      3x3 jittered, permuted Taylor-Hood mesh, nu = 1e-3
  inverse_12   12x12 Poisson inverse: femx ReducedFunctional gradient with
               DenseLinearSolver, misfit 0.5|u - d|^2, kappa = exp(m)
  gmsh_v2, gmsh_v4
               femx's GmshReader on ASCII Gmsh 2.2 / 4.1 files written by
               meshes.write_gmsh (6x6 jittered mesh, permuted node tags,
               boundary segments with physical groups); the file text is
               stored with the reader's output
  ns_gls_*     femx's own equal-order GLS Navier-Stokes time operator
               (NavierOperator, CN + AB2) on P1 triangles through femx's time
               assemble: 5x5 jittered permuted mesh at step 0 (no AB2) and
               step 3 (AB2 advection), and a fluid at rest (zero velocity
               history: the elemLength fallback direction)

    python tests/golden/make_golden.py --only ns_gls   # one family of cases
    python tests/golden/make_golden.py --only gmsh
    python tests/golden/make_golden.py --only real

  real_sq_*    femx's GmshReader on the reference's data/meshes/
               2d_square_res_very_low.msh (parsed arrays only, the file is not
               copied) and, on that mesh moved onto the unit square, the
               p1 / ns_gls / th cases above
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from femx_gb300 import meshes  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")


def build(ref: str):
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref"), f"REF={ref}", "-j8"])


def write(d, name, arr):
    np.ascontiguousarray(arr).tofile(os.path.join(d, name + ".bin"))


def read(d, name, dtype):
    return np.fromfile(os.path.join(d, name + ".bin"), dtype=dtype)


def run(kind, d, params=None):
    if params:
        with open(os.path.join(d, "params.txt"), "w") as fh:
            for k, v in params.items():
                fh.write(f"{k} {v!r}\n")
    out = subprocess.run([DRIVER, kind, d], check=True, capture_output=True, text=True)
    return out.stdout


KAT_NAMES = {
    "shared_row_ptr": np.int32, "shared_col_ind": np.int32, "shared_jac_map": np.int32,
    "rect_row_ptr": np.int32, "rect_col_ind": np.int32, "rect_jac_map": np.int32,
}
for tag in ("bc1_", "bc02_"):
    for nm in ("rows1", "rows0", "res", "fwd_vals", "fwd_rhs"):
        KAT_NAMES[tag + nm] = np.float64

MAP_OUT = {"row_ptr": np.int32, "col_ind": np.int32, "jac_offsets": np.int32, "jac_map": np.int32}
BC_OUT = {"bc_rows": np.int32, "bc_diag": np.int32, "bc_col_offsets": np.int32,
          "bc_col_entries": np.int32, "bc_col_rows": np.int32, "bc_mask": np.int32}


def case_kat(tmp):
    d = os.path.join(tmp, "kat")
    os.makedirs(d)
    run("kat", d)
    return {k: read(d, k, t) for k, t in KAT_NAMES.items()}


def case_p1(tmp, name, coords, conn, kappa, f, u, x, lam, g):
    d = os.path.join(tmp, name)
    os.makedirs(d)
    for nm, arr in (("coords", coords), ("conn", conn), ("kappa", kappa), ("f", f), ("u", u),
                    ("x", x), ("lam", lam)):
        write(d, nm, arr)
    run("p1", d, {"g0": g[0], "gx": g[1], "gy": g[2]})
    out = dict(coords=coords, conn=conn, kappa=kappa, f=f, u=u, x=x, lam=lam,
               g=np.array(g, dtype=np.float64))
    for k, t in {**MAP_OUT, **BC_OUT, "bc_dofs": np.int32}.items():
        out[k] = read(d, k, t)
    for k in ("res", "vals", "bc_vals", "y_matvec", "y_matvec_t", "vals_rows1", "res_replaced",
              "vals_fwd", "rhs_fwd", "g_u", "g_m"):
        out[k] = read(d, k, np.float64)
    return out


def case_th(tmp, name, coords3, conn3, nu, seed):
    rng = np.random.default_rng(seed)
    cp2, conn6, nv = meshes.p2_mesh(coords3, conn3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    state = rng.standard_normal(nd)
    d = os.path.join(tmp, name)
    os.makedirs(d)
    write(d, "coords", cp2)
    write(d, "conn6", conn6)
    write(d, "elem_dofs", dofs)
    write(d, "state", state)
    run("th", d, {"nu": nu, "num_dofs": nd})
    out = dict(coords=cp2, conn6=conn6, elem_dofs=dofs, state=state, nu=np.float64(nu),
               num_dofs=np.int64(nd))
    for k, t in MAP_OUT.items():
        out[k] = read(d, k, t)
    out["res"] = read(d, "res", np.float64)
    out["vals"] = read(d, "vals", np.float64)
    return out


def case_inverse(tmp, nx, seed):
    coords, conn = meshes.structured_tri(nx)
    f = meshes.fourier_source(coords, seed)
    m_true = meshes.grf_centroids(coords, conn, seed + 1, ell=0.2, grid=64)
    d = os.path.join(tmp, f"inverse_{nx}_true")
    os.makedirs(d)
    write(d, "coords", coords)
    write(d, "conn", conn)
    write(d, "m", m_true)
    write(d, "d", np.zeros(coords.shape[0]))
    write(d, "f", f)
    run("inverse", d)
    u_true = read(d, "u", np.float64)
    rng = np.random.default_rng(seed + 2)
    data = u_true + 1e-3 * rng.standard_normal(u_true.shape)
    m = 0.5 * m_true + 0.1
    d2 = os.path.join(tmp, f"inverse_{nx}")
    os.makedirs(d2)
    for nm, arr in (("coords", coords), ("conn", conn), ("m", m), ("d", data), ("f", f)):
        write(d2, nm, arr)
    run("inverse", d2)
    return dict(coords=coords, conn=conn, m=m, d=data, f=f,
                value=read(d2, "value", np.float64), grad=read(d2, "grad", np.float64),
                u=read(d2, "u", np.float64))


def case_navier(tmp, name, coords, conn, rho, mu, dt, step, seed, still=False):
    d = os.path.join(tmp, name)
    os.makedirs(d, exist_ok=True)
    n = coords.shape[0]
    nd = 3 * n
    rng = np.random.default_rng(seed)
    hist = rng.standard_normal(2 * nd)
    if still:
        hist[: 2 * n] = 0.0  # velocity of the current state (lag 0) at rest
    nxt = rng.standard_normal(nd)
    write(d, "coords", coords.astype(np.float64))
    write(d, "conn", conn.astype(np.int32))
    write(d, "hist", hist)
    write(d, "nxt", nxt)
    run("navier", d, {"rho": rho, "mu": mu, "dt": dt, "step": step})
    out = {"coords": coords, "conn": conn, "hist": hist, "nxt": nxt,
           "rho": np.array([rho]), "mu": np.array([mu]), "dt": np.array([dt]),
           "step": np.array([step])}
    for k in ("res_offsets", "res_dofs", "state_offsets", "state_dofs", "row_ptr", "col_ind",
              "jac_offsets", "jac_map", "num_dofs"):
        out[k] = read(d, k, np.int32)
    for k in ("res", "vals"):
        out[k] = read(d, k, np.float64)
    assert int(out["num_dofs"][0]) == nd
    return out


def navier_cases(tmp):
    coords, conn = meshes.jittered_tri(5, seed=31, permute=True)
    np.savez_compressed(os.path.join(HERE, "ns_gls_jit5_s0.npz"),
                        **case_navier(tmp, "ns_s0", coords, conn, 1.0, 1e-2, 0.05, 0, 41))
    np.savez_compressed(os.path.join(HERE, "ns_gls_jit5_s3.npz"),
                        **case_navier(tmp, "ns_s3", coords, conn, 1.2, 5e-3, 0.02, 3, 42))
    c2, k2 = meshes.structured_tri(4)
    np.savez_compressed(os.path.join(HERE, "ns_gls_still4.npz"),
                        **case_navier(tmp, "ns_still", c2, k2, 1.0, 1e-3, 0.1, 2, 43, still=True))


def case_gmsh(tmp, name, version):
    d = os.path.join(tmp, name)
    os.makedirs(d, exist_ok=True)
    coords, conn = meshes.jittered_tri(6, seed=61)
    path = os.path.join(d, "mesh.msh")
    meshes.write_gmsh(path, coords, conn, version=version, seed=62)
    run("gmsh", d)
    out = {"msh": np.frombuffer(open(path, "rb").read(), dtype=np.uint8)}
    out["dim"] = read(d, "dim", np.int32)
    out["coords"] = read(d, "coords", np.float64)
    for k in ("conn", "etag", "ptag", "fconn", "fetag", "fptag"):
        out[k] = read(d, k, np.int32)
    out["names"] = np.frombuffer(open(os.path.join(d, "names.txt"), "rb").read(), dtype=np.uint8)
    return out


def gmsh_cases(tmp):
    for v in (2, 4):
        np.savez_compressed(os.path.join(HERE, f"gmsh_v{v}.npz"), **case_gmsh(tmp, f"g{v}", v))


# A real unstructured mesh of the reference's own data (data/meshes), read by
# femx's GmshReader here; the file itself is not copied: the fixtures hold
# femx's parsed arrays and femx's assembly outputs on that mesh.
REAL_MESHES = {"real_sq": "2d_square_res_very_low.msh"}


def real_cases(tmp, ref):
    import shutil
    for name, fn in REAL_MESHES.items():
        d = os.path.join(tmp, name + "_gmsh")
        os.makedirs(d, exist_ok=True)
        shutil.copyfile(os.path.join(ref, "data", "meshes", fn), os.path.join(d, "mesh.msh"))
        run("gmsh", d)
        mesh = {"source": np.frombuffer(fn.encode(), dtype=np.uint8),
                "dim": read(d, "dim", np.int32), "coords": read(d, "coords", np.float64)}
        for k in ("conn", "etag", "ptag", "fconn", "fetag", "fptag"):
            mesh[k] = read(d, k, np.int32)
        mesh["names"] = np.frombuffer(open(os.path.join(d, "names.txt"), "rb").read(),
                                      dtype=np.uint8)
        np.savez_compressed(os.path.join(HERE, name + "_mesh.npz"), **mesh)
        # the square [-0.5, 0.5]^2 moved onto the unit square, whose edges the
        # reference driver's Dirichlet set selects
        coords = mesh["coords"].reshape(-1, 3)[:, :2] + 0.5  # stored as (x, y, z)
        conn = mesh["conn"].reshape(-1, 3)
        n, e = coords.shape[0], conn.shape[0]
        rng = np.random.default_rng(81)
        np.savez_compressed(os.path.join(HERE, name + "_p1.npz"), **case_p1(
            tmp, name + "_p1", coords, conn, np.exp(rng.standard_normal(e)),
            meshes.fourier_source(coords, 5), rng.standard_normal(n), rng.standard_normal(n),
            rng.standard_normal(n), (0.25, -1.0, 0.5)))
        np.savez_compressed(os.path.join(HERE, name + "_ns.npz"),
                            **case_navier(tmp, name + "_ns", coords, conn, 1.0, 2e-3, 0.01, 3, 82))
        th = case_th(tmp, name + "_th", coords, conn, 1e-3, 83)
        for k in ("jac_offsets", "jac_map"):  # the test checks row_ptr/col_ind and values
            th.pop(k)
        np.savez_compressed(os.path.join(HERE, name + "_th.npz"), **th)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("FEMX_REFERENCE"),
                    required=os.environ.get("FEMX_REFERENCE") is None,
                    help="femx source tree (default: $FEMX_REFERENCE)")
    ap.add_argument("--only", default="", help="generate one family: ns_gls, gmsh, real")
    args = ap.parse_args()
    build(args.ref)
    if args.only == "ns_gls":
        with tempfile.TemporaryDirectory() as tmp:
            navier_cases(tmp)
        return
    if args.only == "gmsh":
        with tempfile.TemporaryDirectory() as tmp:
            gmsh_cases(tmp)
        return
    if args.only == "real":
        with tempfile.TemporaryDirectory() as tmp:
            real_cases(tmp, args.ref)
        return
    with tempfile.TemporaryDirectory() as tmp:
        navier_cases(tmp)
        gmsh_cases(tmp)
        real_cases(tmp, args.ref)
        np.savez_compressed(os.path.join(HERE, "kat.npz"), **case_kat(tmp))

        coords, conn = meshes.structured_tri(32)
        n, e = coords.shape[0], conn.shape[0]
        rng = np.random.default_rng(1)
        f = meshes.fourier_source(coords, 1)
        np.savez_compressed(os.path.join(HERE, "p1_32.npz"), **case_p1(
            tmp, "p1_32", coords, conn, np.ones(e), f, np.zeros(n), rng.standard_normal(n),
            rng.standard_normal(n), (0.0, 0.0, 0.0)))

        coords, conn = meshes.jittered_tri(9, seed=7)
        n, e = coords.shape[0], conn.shape[0]
        rng = np.random.default_rng(9)
        np.savez_compressed(os.path.join(HERE, "p1_jit9.npz"), **case_p1(
            tmp, "p1_jit9", coords, conn, np.exp(rng.standard_normal(e)),
            meshes.fourier_source(coords, 3), rng.standard_normal(n), rng.standard_normal(n),
            rng.standard_normal(n), (0.5, 1.0, -2.0)))

        c3, k3 = meshes.structured_tri(4)
        np.savez_compressed(os.path.join(HERE, "th_4.npz"), **case_th(tmp, "th_4", c3, k3, 1e-2, 4))
        c3, k3 = meshes.jittered_tri(3, seed=11)
        np.savez_compressed(os.path.join(HERE, "th_jit3.npz"),
                            **case_th(tmp, "th_jit3", c3, k3, 1e-3, 5))

        np.savez_compressed(os.path.join(HERE, "inverse_12.npz"), **case_inverse(tmp, 12, 20))
    for fn in sorted(os.listdir(HERE)):
        if fn.endswith(".npz"):
            print(fn, os.path.getsize(os.path.join(HERE, fn)), "bytes")


if __name__ == "__main__":
    main()
