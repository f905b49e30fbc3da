"""The pybind11 module femx_gb300._core: femx's Python surface for the
assembly path (femx._core, python/bindings/Module.cpp:7-30; State.cpp:
649-667 for TimeDims, VariableBlock, TimeResidual).

CPU tests: the module builds against libgbfem and torch's pybind11 headers,
imports without a GPU, exposes femx's names, and its TimeResidual trampoline
dispatches to Python overrides (femx's PyTimeResidual contract).

GPU tests (marked gpu): the assembly path through the module against the
reference library's golden vectors — the P1 Poisson pattern, values and
residual (plain and tiled), the Dirichlet lifting, SpMV — and the native
NavierTimeResidual against femx's own NavierOperator goldens and the
oracle's exact history VJP."""
import numpy as np
import pytest

from conftest import load_golden, rel_inf

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def core():
    from femx_gb300 import build
    build.build_core()
    import femx_gb300._core as c
    return c


def test_module_surface(core):
    assert core.__version__ == "0.4.0"
    for name in ("TimeDims", "VariableBlock", "TimeResidual", "NavierTimeResidual",
                 "AssemblyMap", "BoundaryMap", "make_assembly_map", "make_boundary_map",
                 "assemble_p1_kappa", "vjp_p1_kappa", "assemble_taylor_hood",
                 "vjp_taylor_hood", "replace_rows", "replace_res", "zero_boundary",
                 "prepare_forward_solve", "matvec", "matvec_t"):
        assert hasattr(core, name), name
    d = core.TimeDims()
    d.num_steps, d.num_states, d.num_hist = 4, 7, 2
    assert (d.num_steps, d.num_states, d.num_param, d.num_hist) == (4, 7, 0, 2)
    b = core.VariableBlock.history(1)
    assert b.is_history_state and not b.is_parameter and b.history_lag == 1
    assert core.VariableBlock.parameter().is_parameter
    assert core.VariableBlock.next_state().is_next_state


def test_time_residual_trampoline(core):
    class Twice(core.TimeResidual):
        def dims(self):
            t = core.TimeDims()
            t.num_states = t.num_res = 3
            return t

        def residual(self, ctx):
            return [2.0 * x for x in ctx["next_state"]]

    r = Twice()
    assert r.dims().num_states == 3
    assert r.residual({"step": 0, "next_state": [1.0, 2.0, 3.0]}) == [2.0, 4.0, 6.0]
    assert r.prepare_linear_solve({}, None, None) is None
    with pytest.raises(RuntimeError, match="pure virtual"):
        r.assemble_next({})


def test_arguments_are_checked_on_the_host(core):
    with pytest.raises(RuntimeError, match="CUDA"):
        core.make_assembly_map(3, 3, np.zeros(2, np.int32), np.zeros(3, np.int32),
                               np.zeros(2, np.int32), np.zeros(3, np.int32))


# --- GPU ----------------------------------------------------------------------

def cuda(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["p1_32", "p1_jit9", "real_sq_p1"])
def test_p1_path_through_core_matches_reference(core, case):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from femx_gb300 import meshes
    g = load_golden(case)
    conn = g["conn"].astype(np.int32)
    n = g["coords"].shape[0]
    offs, dofs = meshes.scalar_elem_dofs(conn)
    amap = core.make_assembly_map(n, n, cuda(offs), cuda(dofs), cuda(offs), cuda(dofs))
    assert amap.nnz == g["col_ind"].size
    assert np.array_equal(torch.as_tensor(amap.row_ptr(), device="cuda").cpu().numpy(),
                          g["row_ptr"])
    assert np.array_equal(torch.as_tensor(amap.col_ind(), device="cuda").cpu().numpy(),
                          g["col_ind"])
    coords, kappa, f, u = cuda(g["coords"]), cuda(g["kappa"]), cuda(g["f"]), cuda(g["u"])
    res = torch.zeros(n, dtype=torch.float64, device="cuda")
    vals = torch.zeros(amap.nnz, dtype=torch.float64, device="cuda")
    core.assemble_p1_kappa(amap, coords, kappa, f, u, res, vals)
    amap.check()
    assert rel_inf(vals.cpu().numpy(), g["vals"]) <= 1e-12
    assert rel_inf(res.cpu().numpy(), g["res"]) <= 1e-12
    # the tiled FP64-accurate path through the same module
    assert amap.enable_tiles(coords) >= 1
    res_t, vals_t = torch.zeros_like(res), torch.zeros_like(vals)
    core.assemble_p1_kappa(amap, coords, kappa, f, u, res_t, vals_t, precision="double_float",
                           tiled=True)
    assert rel_inf(vals_t.cpu().numpy(), g["vals"]) <= 1e-12
    assert rel_inf(res_t.cpu().numpy(), g["res"]) <= 1e-12
    # SpMV and its transpose (MatrixHandler::matvec / matvecT)
    y = torch.zeros(n, dtype=torch.float64, device="cuda")
    core.matvec(amap, vals, cuda(g["x"]), y)
    assert rel_inf(y.cpu().numpy(), g["y_matvec"]) <= 1e-13
    core.matvec_t(amap, vals, cuda(g["x"]), y)
    assert rel_inf(y.cpu().numpy(), g["y_matvec_t"]) <= 1e-13
    # the forward-solve lifting (prepareForwardSolve) on the assembled system
    bc = core.make_boundary_map(cuda(g["bc_dofs"]), amap)
    assert bc.num_bcs == g["bc_dofs"].size and bc.layout_id == amap.layout_id
    rhs = -res
    core.prepare_forward_solve(bc, vals, rhs, cuda(g["bc_vals"]))
    assert rel_inf(vals.cpu().numpy(), g["vals_fwd"]) <= 1e-12
    assert rel_inf(rhs.cpu().numpy(), g["rhs_fwd"]) <= 1e-12
    with pytest.raises(RuntimeError, match="size mismatch"):
        core.assemble_p1_kappa(amap, coords, kappa, f, u, res[:-1], vals)


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["ns_gls_jit5_s0", "ns_gls_jit5_s3", "real_sq_ns"])
def test_native_navier_time_residual_matches_femx(core, case):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from oracle import pyoracle as orc
    g = load_golden(case)
    nd = int(g["num_dofs"][0])
    amap = core.make_assembly_map(nd, nd, cuda(g["res_offsets"]), cuda(g["res_dofs"]),
                                  cuda(g["state_offsets"]), cuda(g["state_dofs"]))
    step = int(g["step"][0])
    r = core.NavierTimeResidual(amap, cuda(g["coords"]), cuda(g["conn"].astype(np.int32)),
                                float(g["rho"][0]), float(g["mu"][0]), float(g["dt"][0]),
                                step + 1)
    assert isinstance(r, core.TimeResidual)
    d = r.dims()
    assert (d.num_steps, d.num_states, d.num_param, d.num_res, d.num_hist) == \
        (step + 1, nd, 0, nd, 2)
    # femx's ctx: host arrays, history lag-major
    ctx = {"step": step, "next_state": g["nxt"], "parameters": np.zeros(0),
           "history": g["hist"].reshape(2, nd)}
    assert rel_inf(r.residual(ctx).cpu().numpy(), g["res"]) <= 1e-12
    vals, res = r.assemble_next(ctx)
    assert rel_inf(vals.cpu().numpy(), g["vals"]) <= 1e-12
    assert rel_inf(res.cpu().numpy(), g["res"]) <= 1e-12
    adj = np.random.default_rng(8).standard_normal(nd)
    om = orc.AssemblyMap(nd, nd, g["res_offsets"], g["res_dofs"], g["state_offsets"],
                         g["state_dofs"])
    q = orc.P1Quad(g["coords"], g["conn"], order=2)
    ref = orc.vjp_navier_hist(om, q, g["rho"][0], g["mu"][0], g["dt"][0], step,
                              g["hist"], g["nxt"], adj)
    for lag in (0, 1):
        got = r.apply_jacobian_transpose(ctx, core.VariableBlock.history(lag), adj)
        want = ref[lag * nd:(lag + 1) * nd]
        if np.any(want):
            assert rel_inf(got.cpu().numpy(), want) <= 1e-12
        else:
            assert not got.cpu().numpy().any()
    assert r.apply_jacobian_transpose(ctx, core.VariableBlock.parameter(), adj).numel() == 0
    with pytest.raises(RuntimeError, match="supports only history and parameter blocks"):
        r.apply_jacobian_transpose(ctx, core.VariableBlock.next_state(), adj)
    with pytest.raises(RuntimeError, match="step is out of range"):
        r.residual(dict(ctx, step=step + 1))
    with pytest.raises(RuntimeError, match="parameter-free"):
        r.initial_state(np.ones(2))
