"""The bench's CPU-baseline helpers run the oracle only, so they are checked
here on small instances: the batch baseline applies per-physics element
rates measured on a sample to the batch's element counts."""
import numpy as np

import bench
from femx_gb300 import meshes


def _sample():
    rng = np.random.default_rng(5)
    coords, conn = meshes.jittered_tri(16, seed=1000)
    nn = coords.shape[0]
    offs, dofs = meshes.scalar_elem_dofs(conn)
    kappa = np.exp(meshes.grf_centroids(coords, conn, seed=2000, ell=0.05, grid=64))
    p1 = ("p1", conn.shape[0], coords, conn, offs, dofs, kappa, rng.standard_normal(nn),
          meshes.fourier_source(coords, 0), rng.standard_normal(nn))
    c3, k3 = meshes.jittered_tri(6, seed=3000)
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    th = ("th", conn6.shape[0], cp2, conn6, offs, dofs, nd, 1e-3,
          meshes.cavity_state(cp2, nv, seed=0), rng.standard_normal(nd))
    return [p1, th]


def test_batch_cpu_baseline_accounts_for_both_physics():
    sample = _sample()
    e_p1, e_th = 100_000, 20_000
    out = bench.batch_cpu(sample, e_p1, e_th)
    assert out["cores"] == 1 and out["kind"] == "port"
    assert out["elements_per_s"] > 0 and out["seconds_per_batch"] > 0
    np.testing.assert_allclose(out["elements_per_s"] * out["seconds_per_batch"], e_p1 + e_th,
                               rtol=1e-12)
    assert f"{e_p1} P1 and {e_th} Taylor-Hood elements" in out["sample"]


def test_batch_cpu_baseline_with_one_physics_only():
    sample = [s for s in _sample() if s[0] == "p1"]
    out = bench.batch_cpu(sample, 50_000, 0)
    assert out["elements_per_s"] > 0
    np.testing.assert_allclose(out["elements_per_s"] * out["seconds_per_batch"], 50_000,
                               rtol=1e-12)
