"""Batched persistent assembly: every instance of a mixed, uneven batch must
equal its standalone assembly (and VJPs), for any launch parameters and when
replayed from a CUDA graph."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from conftest import rel_inf  # noqa: E402
from femx_gb300 import assembly as A  # noqa: E402
from femx_gb300 import meshes  # noqa: E402
from femx_gb300.batch import Batch, P1Instance, THInstance, autotune  # noqa: E402
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


def make_batch(seed=0, coloured=False):
    rng = np.random.default_rng(seed)
    insts, refs = [], []
    for k, nx in enumerate((9, 31, 17, 40)):
        coords, conn = meshes.jittered_tri(nx, seed=seed + k)
        offs, dofs = meshes.scalar_elem_dofs(conn)
        n, e = coords.shape[0], conn.shape[0]
        amap = A.makeAssemblyMap(n, n, dev(offs), dev(dofs), dev(offs), dev(dofs))
        kappa = np.exp(rng.standard_normal(e))
        f = meshes.fourier_source(coords, k) if k % 2 == 0 else None
        u, lam = rng.standard_normal(n), rng.standard_normal(n)
        insts.append(P1Instance(amap, dev(coords), dev(kappa), dev(u),
                                None if f is None else dev(f), dev(lam)))
        refs.append(("p1", coords, conn, kappa, f, u, lam, offs, dofs))
    for k, (nx, re) in enumerate(((5, 100.0), (12, 400.0), (8, 1000.0))):
        c3, k3 = meshes.jittered_tri(nx, seed=50 + k, permute=k == 1)
        cp2, conn6, nv = meshes.p2_mesh(c3, k3)
        offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
        amap = A.makeAssemblyMap(nd, nd, dev(offs), dev(dofs), dev(offs), dev(dofs))
        state = meshes.cavity_state(cp2, nv, seed=k)
        lam = rng.standard_normal(nd)
        insts.append(THInstance(amap, dev(cp2), dev(conn6), 1.0 / re, dev(state), dev(lam)))
        refs.append(("th", cp2, conn6, 1.0 / re, state, lam, offs, dofs, nd))
    return Batch(insts, coloured=coloured), insts, refs


def check_against_oracle(insts, refs, tol_j, tol_r, tol_g, tol_g_th=None):
    tol_g_th = tol_g if tol_g_th is None else tol_g_th
    for inst, ref in zip(insts, refs):
        if ref[0] == "p1":
            _, coords, conn, kappa, f, u, lam, offs, dofs = ref
            n = coords.shape[0]
            om = orc.AssemblyMap(n, n, offs, dofs, offs, dofs)
            q = orc.P1Quad(coords, conn)
            rres, rvals = orc.assemble_p1_kappa(om, q, kappa, f, u)
            gu, gm = orc.vjp_p1_kappa(om, q, kappa, u, lam)
            assert rel_inf(inst.res.cpu().numpy(), rres) <= tol_r
            assert rel_inf(inst.vals.cpu().numpy(), rvals) <= tol_j
            assert rel_inf(inst.g_u.cpu().numpy(), gu) <= tol_g
            assert rel_inf(inst.g_m.cpu().numpy(), gm) <= tol_g
        else:
            _, cp2, conn6, nu, state, lam, offs, dofs, nd = ref
            om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
            rres, rvals = orc.assemble_th_ns(om, cp2, conn6, nu, state)
            gt = orc.matvec_t(om.row_ptr, om.col_ind, rvals, lam, nd)
            assert rel_inf(inst.res.cpu().numpy(), rres) <= tol_r
            assert rel_inf(inst.vals.cpu().numpy(), rvals) <= tol_j
            assert rel_inf(inst.g_u.cpu().numpy(), gt) <= tol_g_th


# (precision, Jacobian, residual, P1 gradients, Taylor-Hood J^T lam)
@pytest.mark.parametrize("precision,tj,tr,tg,tgt", [
    ("fp64", 1e-12, 1e-12, 1e-12, 1e-12),
    ("fp32_quad", 1e-6, 1e-6, 1e-6, 1e-6),
    ("mixed", 1e-6, 1e-12, 1e-12, 1e-6)])
def test_batch_matches_oracle(precision, tj, tr, tg, tgt):
    batch, insts, refs = make_batch()
    batch.run(precision)
    batch.check()
    torch.cuda.synchronize()
    check_against_oracle(insts, refs, tj, tr, tg, tgt)


@pytest.mark.parametrize("params", [dict(p1_chunk=128, th_chunk=8, blocks_per_sm=1),
                                    dict(p1_chunk=2048, th_chunk=64, blocks_per_sm=16),
                                    dict(p1_chunk=256, th_chunk=16, blocks_per_sm=4,
                                         stage_depth=1)])
def test_batch_independent_of_launch_parameters(params):
    batch, insts, refs = make_batch(seed=3)
    batch.run("fp64", **params)
    torch.cuda.synchronize()
    check_against_oracle(insts, refs, 1e-12, 1e-12, 1e-12)


def test_batch_cuda_graph_replay():
    batch, insts, refs = make_batch(seed=5)
    g = batch.graph("fp64")
    for inst in insts:  # poison outputs: the graph must rewrite them
        inst.res.fill_(7.0)
        inst.vals.fill_(-3.0)
        inst.g_u.fill_(1.0)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    check_against_oracle(insts, refs, 1e-12, 1e-12, 1e-12)


@pytest.mark.parametrize("precision,tj,tr,tg,tgt", [
    ("fp64", 1e-12, 1e-12, 1e-12, 1e-12),
    ("fp32_quad", 1e-6, 1e-6, 1e-6, 1e-6)])
def test_coloured_batch_matches_oracle_and_is_bitwise_reproducible(precision, tj, tr, tg, tgt):
    """The colouring scatter scheme: colour rounds with plain adds, no
    atomics; two runs agree bit for bit, with and without staging."""
    batch, insts, refs = make_batch(seed=9, coloured=True)
    assert all(x.amap.numColours() >= 3 for x in insts)
    outs = []
    for stage in (0, 1, 0):
        batch.run(precision, scatter="colour", stage_depth=stage, p1_chunk=256, th_chunk=16)
        batch.check()
        torch.cuda.synchronize()
        outs.append([(x.res.clone(), x.vals.clone(), x.g_u.clone()) for x in insts])
    check_against_oracle(insts, refs, tj, tr, tg, tgt)
    for run in outs[1:]:
        for a, b in zip(run, outs[0]):
            assert all(torch.equal(p, q) for p, q in zip(a, b))


def test_coloured_batch_needs_coloured_maps():
    batch, insts, refs = make_batch(seed=2)
    with pytest.raises(A.GbfemError, match="colouring"):
        batch.run("fp64", scatter="colour")


def test_autotune_returns_valid_params(tmp_path, monkeypatch):
    monkeypatch.setenv("GBFEM_TUNE_CACHE", str(tmp_path / "tune.json"))
    batch, insts, refs = make_batch(seed=7, coloured=True)
    params, timings = autotune(batch, "fp32_quad", reps=1)
    assert set(params) == {"p1_chunk", "th_chunk", "blocks_per_sm", "stage_depth", "scatter"}
    assert params["scatter"] in ("atomic", "colour") and params["stage_depth"] in (0, 1)
    det, _ = autotune(batch, "fp64", reps=1, deterministic=True)
    assert det["scatter"] == "colour"
    again, info = autotune(batch, "fp32_quad")
    assert again == params and info == {"cached": True}
    batch.run("fp64", **params)
    torch.cuda.synchronize()
    check_against_oracle(insts, refs, 1e-12, 1e-12, 1e-12)
