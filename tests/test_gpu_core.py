"""femx's Python time-residual surface (femx_gb300.core: TimeDims,
VariableBlock, TimeResidual; femx._core's names and ctx-dict protocol)
over the GPU path: NavierTimeResidual against the reference library's own
NavierOperator goldens and the oracle's exact history VJP, driven the way
femx's PyTimeResidual trampoline drives a Python residual
(python/bindings/State.cpp:249-460), and femx's errors."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from conftest import load_golden, rel_inf  # noqa: E402
from oracle import pyoracle as orc  # noqa: E402

CASES = ["ns_gls_jit5_s0", "ns_gls_jit5_s3", "ns_gls_still4", "real_sq_ns"]


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from femx_gb300 import build
    build.build()


def femx_ctx(g, nsteps_ok=True):
    nd = int(g["num_dofs"][0])
    return {"step": int(g["step"][0]), "next_state": g["nxt"],
            "parameters": np.zeros(0), "history": g["hist"].reshape(2, nd)}


def residual_of(g):
    from femx_gb300.core import NavierTimeResidual
    return NavierTimeResidual(g["coords"], g["conn"], g["rho"][0], g["mu"][0], g["dt"][0],
                              num_steps=int(g["step"][0]) + 1)


@pytest.mark.parametrize("case", CASES)
def test_navier_time_residual_matches_femx(case):
    from femx_gb300.core import TimeResidual, VariableBlock
    g = load_golden(case)
    r = residual_of(g)
    assert isinstance(r, TimeResidual)
    nd = int(g["num_dofs"][0])
    d = r.dims()
    assert (d.num_steps, d.num_states, d.num_param, d.num_res, d.num_hist) == \
        (int(g["step"][0]) + 1, nd, 0, nd, 2)
    pat = r.pattern()
    assert np.array_equal(pat.row_ptr.cpu().numpy(), g["row_ptr"])
    assert np.array_equal(pat.col_ind.cpu().numpy(), g["col_ind"])
    ctx = femx_ctx(g)
    assert rel_inf(r.residual(ctx).cpu().numpy(), g["res"]) <= 1e-12
    jac, res = r.assemble_next(ctx)
    assert rel_inf(jac.vals.cpu().numpy(), g["vals"]) <= 1e-12
    assert rel_inf(res.cpu().numpy(), g["res"]) <= 1e-12
    # history VJPs, one lag at a time, against the oracle's exact derivative
    adj = np.random.default_rng(8).standard_normal(nd)
    om = orc.AssemblyMap(nd, nd, g["res_offsets"], g["res_dofs"], g["state_offsets"],
                         g["state_dofs"])
    q = orc.P1Quad(g["coords"], g["conn"], order=2)
    ref = orc.vjp_navier_hist(om, q, g["rho"][0], g["mu"][0], g["dt"][0], int(g["step"][0]),
                              g["hist"], g["nxt"], adj)
    for lag in (0, 1):
        got = r.apply_jacobian_transpose(ctx, VariableBlock.history(lag), adj).cpu().numpy()
        want = ref[lag * nd:(lag + 1) * nd]
        if np.any(want):
            assert rel_inf(got, want) <= 1e-12
        else:
            assert not got.any()
    assert r.apply_jacobian_transpose(ctx, VariableBlock.parameter(), adj).numel() == 0
    assert not r.initial_state(np.zeros(0)).any()


def test_navier_time_residual_errors_are_femx_errors():
    from femx_gb300.core import VariableBlock
    g = load_golden("ns_gls_jit5_s3")
    r = residual_of(g)
    ctx = femx_ctx(g)
    adj = np.zeros(int(g["num_dofs"][0]))
    with pytest.raises(RuntimeError, match="supports only history and parameter blocks"):
        r.apply_jacobian_transpose(ctx, VariableBlock.next_state(), adj)
    with pytest.raises(RuntimeError, match="history lag is out of range"):
        r.apply_jacobian_transpose(ctx, VariableBlock.history(2), adj)
    bad = dict(ctx, step=r.dims().num_steps)
    with pytest.raises(RuntimeError, match="step is out of range"):
        r.residual(bad)
    bad = dict(ctx, parameters=np.ones(1))
    with pytest.raises(RuntimeError, match="vector size mismatch"):
        r.residual(bad)
    with pytest.raises(RuntimeError, match="parameter-free"):
        r.initial_state(np.ones(2))
