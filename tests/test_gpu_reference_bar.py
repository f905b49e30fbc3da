"""The benchmark's GPU bar — femx's own CUDA assembly kernel (assembleKernel,
femx/assembly/CudaAssembly.hpp:100-169, compiled from femx's sources into
oracle/_ref/gpu_bar.cubin for the kappa-weighted P1 operator in femx's
plug-in form) launched through oracle/gpu_bar.py — reproduces the reference
library's CPU golden vectors, so that the bench times the reference's kernel
doing the same work as the product kernels. Skipped where the cubin was not
built (the femx sources are needed to build it)."""
import numpy as np
import pytest

from conftest import load_golden, rel_inf

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["p1_32", "p1_jit9", "real_sq_p1"])
def test_reference_gpu_assembly_reproduces_reference_goldens(case):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import gpu_bar
    if gpu_bar.unavailable_reason():
        pytest.skip(gpu_bar.unavailable_reason())
    from femx_gb300 import assembly as A, build, meshes
    from oracle import pyoracle as orc
    build.build()
    g = load_golden(case)
    conn = g["conn"].astype(np.int32)
    n = g["coords"].shape[0]
    offs, dofs = meshes.scalar_elem_dofs(conn)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    amap = A.makeAssemblyMap(n, n, d(offs), d(dofs), d(offs), d(dofs))
    view = {k: v.data_ptr() for k, v in amap.view().items()}
    view.update(num_res=n, num_states=n)
    coords, kappa, f, u = d(g["coords"]), d(g["kappa"]), d(g["f"]), d(g["u"])
    bar = gpu_bar.RefP1Assembly(torch, coords, d(conn), kappa, f,
                                orc.P1Quad(g["coords"], conn).tables(), view)
    res = torch.empty(n, dtype=torch.float64, device="cuda")
    vals = torch.empty(amap.pattern().nnz, dtype=torch.float64, device="cuda")
    for _ in range(2):
        bar.assemble(u, res, vals, torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        assert rel_inf(vals.cpu().numpy(), g["vals"]) <= 1e-12
        assert rel_inf(res.cpu().numpy(), g["res"]) <= 1e-12


@pytest.mark.parametrize("case", ["ns_gls_jit5_s0", "ns_gls_jit5_s3", "real_sq_ns"])
def test_reference_gpu_ns_assembly_reproduces_reference_goldens(case):
    """femx's own NS time assembly on the GPU (assembleTimeKernel with femx's
    NavierOperator, next-state block) against the reference library's CPU
    goldens of the same operator."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import gpu_bar
    if gpu_bar.unavailable_reason():
        pytest.skip(gpu_bar.unavailable_reason())
    from femx_gb300 import assembly as A, build
    from oracle import pyoracle as orc
    build.build()
    g = load_golden(case)
    nd = int(g["num_dofs"][0])
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    amap = A.makeAssemblyMap(nd, nd, d(g["res_offsets"]), d(g["res_dofs"]),
                             d(g["state_offsets"]), d(g["state_dofs"]))
    view = {k: v.data_ptr() for k, v in amap.view().items()}
    view.update(num_res=nd, num_states=nd)
    tables = orc.P1Quad(g["coords"], g["conn"].astype(np.int32), order=2).tables()
    bar = gpu_bar.RefNavierAssembly(torch, tables, view, g["coords"].shape[0],
                                    float(g["rho"][0]), float(g["mu"][0]), float(g["dt"][0]))
    res = torch.empty(nd, dtype=torch.float64, device="cuda")
    vals = torch.empty(amap.pattern().nnz, dtype=torch.float64, device="cuda")
    bar.assemble(int(g["step"][0]), d(g["hist"]), d(g["nxt"]), res, vals,
                 torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert rel_inf(vals.cpu().numpy(), g["vals"]) <= 1e-12
    assert rel_inf(res.cpu().numpy(), g["res"]) <= 1e-12
