"""The host-state Newton-system entry (gbfem_newton_system_th_ns_host)
against the same steps issued one by one on device buffers: the uploaded
state, the residual and Jacobian with Dirichlet rows, and the downloaded
residual; on the default stream and on a side stream, repeated calls."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from femx_gb300 import assembly as A  # noqa: E402
from femx_gb300 import meshes  # noqa: E402


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from femx_gb300 import build
    build.build()


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def cavity():
    c3, k3 = meshes.structured_tri(24)
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    amap = A.makeAssemblyMap(nd, nd, dev(offs), dev(dofs), dev(offs), dev(dofs))
    bdofs, bvals = meshes.cavity_dirichlet(cp2, cp2.shape[0])
    bc = A.makeBoundaryMap(dev(bdofs), amap.pattern())
    return dict(cp2=cp2, conn6=conn6, nv=nv, nd=nd, amap=amap, bc=bc, bvals=dev(bvals),
                coords=dev(cp2), c6=dev(conn6.astype(np.int32)))


def reference(t, state, precision, det):
    res = torch.zeros(t["nd"], dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(t["amap"].pattern())
    A.assembleTaylorHood(t["amap"], t["coords"], t["c6"], 1e-2, state, res, jac,
                         precision=precision, deterministic=det)
    A.replaceRes(t["bc"], state, t["bvals"], res)
    A.replaceRows(t["bc"], jac, 1.0)
    return res, jac.vals


def rel(a, b):
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize("precision,det", [("fp64", False), ("fp32_quad", False),
                                           ("mixed", False), ("fp32_quad", True)])
def test_host_newton_system_matches_device_steps(cavity, precision, det):
    t = cavity
    nd = t["nd"]
    state_d = torch.empty(nd, dtype=torch.float64, device="cuda")
    res = torch.empty(nd, dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(t["amap"].pattern())
    res_host = torch.empty(nd, dtype=torch.float64).pin_memory()
    for seed in (1, 2):
        state_np = meshes.cavity_state(t["cp2"], t["nv"], seed=seed)
        state_host = torch.from_numpy(state_np).pin_memory()
        A.newtonSystemTaylorHoodHost(t["amap"], t["bc"], t["coords"], t["c6"], 1e-2,
                                     state_host, state_d, t["bvals"], res, jac, res_host,
                                     precision=precision, deterministic=det)
        torch.cuda.synchronize()
        assert torch.equal(state_d.cpu(), state_host)
        assert torch.equal(res_host, res.cpu())
        r_ref, v_ref = reference(t, dev(state_np), precision, det)
        if det:
            assert torch.equal(res, r_ref) and torch.equal(jac.vals, v_ref)
        else:
            assert rel(res, r_ref) <= 1e-13 and rel(jac.vals, v_ref) <= 1e-13
    t["amap"].check()


def test_host_newton_system_on_a_side_stream_and_residual_only(cavity):
    t = cavity
    nd = t["nd"]
    state_np = meshes.cavity_state(t["cp2"], t["nv"], seed=5)
    state_host = torch.from_numpy(state_np).pin_memory()
    res_host = torch.empty(nd, dtype=torch.float64).pin_memory()
    state_d = torch.empty(nd, dtype=torch.float64, device="cuda")
    res = torch.empty(nd, dtype=torch.float64, device="cuda")
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        A.newtonSystemTaylorHoodHost(t["amap"], t["bc"], t["coords"], t["c6"], 1e-2,
                                     state_host, state_d, t["bvals"], res, None, res_host,
                                     precision="fp64")
    side.synchronize()
    r_ref, _ = reference(t, dev(state_np), "fp64", False)
    assert rel(res_host.cuda(), r_ref) <= 1e-13


def test_host_newton_system_rejects_device_host_buffers(cavity):
    t = cavity
    nd = t["nd"]
    d = torch.zeros(nd, dtype=torch.float64, device="cuda")
    with pytest.raises(A.GbfemError):
        A.newtonSystemTaylorHoodHost(t["amap"], t["bc"], t["coords"], t["c6"], 1e-2,
                                     d, d.clone(), t["bvals"], d.clone(), None,
                                     torch.zeros(nd, dtype=torch.float64))


def test_dependent_launches_capture_into_a_cuda_graph(cavity):
    """The zero fill, the element kernel launched as its dependent and the
    Dirichlet kernels launched as dependents replay from a CUDA graph with
    the eager results (FP64: the reductions' order may differ, within 1e-13)."""
    t = cavity
    nd = t["nd"]
    state = dev(meshes.cavity_state(t["cp2"], t["nv"], seed=7))
    res = torch.zeros(nd, dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(t["amap"].pattern())
    r_ref, v_ref = reference(t, state, "fp32_quad", False)

    def step():
        A.assembleTaylorHood(t["amap"], t["coords"], t["c6"], 1e-2, state, res, jac,
                             precision="fp32_quad")
        A.replaceRes(t["bc"], state, t["bvals"], res)
        A.replaceRows(t["bc"], jac, 1.0)

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        step()                      # warm-up outside the capture
    torch.cuda.current_stream().wait_stream(side)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        step()
    res.fill_(3.0)
    jac.vals.fill_(3.0)
    for _ in range(2):
        g.replay()
    torch.cuda.synchronize()
    assert rel(res, r_ref) <= 1e-13 and rel(jac.vals, v_ref) <= 1e-13
    t["amap"].check()


def test_host_newton_system_captures_into_a_cuda_graph(cavity):
    """The host-state entry forks its side stream from the capturing stream
    and joins it back, so the whole call (copies included) replays from a
    graph; the host residual follows the pinned host state on replay."""
    t = cavity
    nd = t["nd"]
    state_np = meshes.cavity_state(t["cp2"], t["nv"], seed=8)
    state_host = torch.from_numpy(state_np).pin_memory()
    res_host = torch.empty(nd, dtype=torch.float64).pin_memory()
    state_d = torch.empty(nd, dtype=torch.float64, device="cuda")
    res = torch.empty(nd, dtype=torch.float64, device="cuda")
    jac = A.CsrMatrix(t["amap"].pattern())

    def call():
        A.newtonSystemTaylorHoodHost(t["amap"], t["bc"], t["coords"], t["c6"], 1e-2,
                                     state_host, state_d, t["bvals"], res, jac, res_host,
                                     precision="fp64")

    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        call()
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        call()
    state2 = meshes.cavity_state(t["cp2"], t["nv"], seed=9)
    state_host.copy_(torch.from_numpy(state2))
    res_host.fill_(0.0)
    g.replay()
    torch.cuda.synchronize()
    r_ref, v_ref = reference(t, dev(state2), "fp64", False)
    assert rel(res_host.cuda(), r_ref) <= 1e-13 and rel(jac.vals, v_ref) <= 1e-13
