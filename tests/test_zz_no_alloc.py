"""gbfem_prepare_forward_solve_noalloc — the Dirichlet forward-solve
preparation for callers that cannot call cudaMalloc.

Such callers (code running while another allocator owns the device memory,
or a real-time solver loop that must not allocate) cannot build a
BoundaryMap handle. The no-allocation entry point does the same work from the
DOF list and the CSR pattern, with scratch in a fixed array the library owns.
These tests call it through the C ABI and require its output to equal the
handle-based entry point's bit for bit (the tolerance the other Dirichlet
tests use), on consecutive calls, across different problems, and after a
rejected call.

This file is collected last on purpose; it must pass on its own in a fresh
process as well as after the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

from conftest import load_golden  # noqa: E402
from femx_gb300 import meshes  # noqa: E402

MAX_ROWS = 2097152


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from femx_gb300 import build
    build.build()


def lib():
    from femx_gb300 import _lib
    return _lib


def ptr(t):
    return C.c_void_p(0 if t is None else t.data_ptr())


def stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    return (t if dtype is None else t.to(dtype)).cuda()


def with_handle(dofs, row_ptr, col_ind, vals, rhs, g):
    """The existing path: BoundaryMap handle + gbfem_prepare_forward_solve."""
    L = lib()
    rows = row_ptr.numel() - 1
    h = C.c_void_p()
    L.check(L.lib().gbfem_boundary_map_create(dofs.numel(), ptr(dofs), rows, rows, ptr(row_ptr),
                                              ptr(col_ind), C.c_ulonglong(0), stream(),
                                              C.byref(h)))
    try:
        v, r = vals.clone(), rhs.clone()
        L.check(L.lib().gbfem_prepare_forward_solve(h, ptr(v), ptr(r), ptr(g), stream()))
        torch.cuda.synchronize()
        return v, r
    finally:
        L.lib().gbfem_boundary_map_destroy(h)


def no_alloc(dofs, row_ptr, col_ind, vals, rhs, g):
    v, r = vals.clone(), rhs.clone()
    rc = call_no_alloc(dofs, row_ptr, col_ind, v, r, g)
    return rc, v, r


def call_no_alloc(dofs, row_ptr, col_ind, v, r, g):
    """One C-ABI call on buffers the caller already holds (v, r updated)."""
    rc = lib().lib().gbfem_prepare_forward_solve_noalloc(
        dofs.numel(), ptr(dofs), row_ptr.numel() - 1, ptr(row_ptr), ptr(col_ind), ptr(v),
        ptr(r), ptr(g), stream())
    torch.cuda.synchronize()
    return rc


def golden_case():
    g = load_golden("p1_jit9")
    return (dev(g["bc_dofs"]), dev(g["row_ptr"]), dev(g["col_ind"]), dev(g["vals"]),
            dev(-g["res"]), dev(g["bc_vals"]))


def cavity_case(nx=48):
    """Taylor-Hood layout: many constrained rows and a pressure pin."""
    c3, k3 = meshes.structured_tri(nx)
    cp2, conn6, _ = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    from oracle import pyoracle as orc
    m = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
    bd, bv = meshes.cavity_dirichlet(cp2, cp2.shape[0])
    rng = np.random.default_rng(7)
    return (dev(bd), dev(m.row_ptr), dev(m.col_ind), dev(rng.standard_normal(m.nnz)),
            dev(rng.standard_normal(nd)), dev(bv + rng.standard_normal(len(bv))))


def assert_same(a, b):
    assert torch.equal(a[0], b[0]) and torch.equal(a[1], b[1])


def test_two_calls_in_a_row_match_the_handle_path_and_the_reference():
    case = golden_case()
    ref = with_handle(*case)
    gold = load_golden("p1_jit9")
    dofs, row_ptr, col_ind, vals, rhs, g = case
    # Buffers are made before the calls so that only the C call runs between
    # the two memory readings around it. The first call on the device is the
    # set-up call: it looks up the scratch array's address, which may make
    # CUDA load the library's module that holds the array (with lazy module
    # loading the array's device memory is committed then). The calls after
    # it must leave the device's free memory unchanged.
    v, r = vals.clone(), rhs.clone()
    for call in range(3):
        v.copy_(vals)
        r.copy_(rhs)
        torch.cuda.synchronize()
        free0, reserved0 = torch.cuda.mem_get_info()[0], torch.cuda.memory_reserved()
        rc = call_no_alloc(dofs, row_ptr, col_ind, v, r, g)
        free1, reserved1 = torch.cuda.mem_get_info()[0], torch.cuda.memory_reserved()
        assert rc == 0, lib().lib().gbfem_last_error().decode()
        assert reserved1 == reserved0
        if call > 0:
            assert free1 == free0  # the call allocated nothing
        assert_same((v, r), ref)
        # femx's own prepareForwardSolve output on this case, bit for bit
        assert np.array_equal(v.cpu().numpy(), gold["vals_fwd"])
        assert np.array_equal(r.cpu().numpy(), gold["rhs_fwd"])


def test_repeated_constrained_column_is_lifted_every_time():
    """A row may hold the same constrained column twice (femx's CsrPattern
    checks ranges and order only); femx lifts and zeroes both entries."""
    gold = load_golden("p1_jit9")
    row_ptr, col_ind = gold["row_ptr"].copy(), gold["col_ind"].copy()
    bc = set(int(d) for d in gold["bc_dofs"])
    rng = np.random.default_rng(11)
    vals = rng.standard_normal(len(col_ind))
    picked = []
    for r in range(len(row_ptr) - 1):
        if r in bc:
            continue
        ks = [k for k in range(row_ptr[r], row_ptr[r + 1]) if int(col_ind[k]) in bc]
        if ks:
            picked.append(ks[0])
        if len(picked) == 4:
            break
    assert picked
    new_cols, new_vals, new_ptr = [], [], [0]
    for r in range(len(row_ptr) - 1):
        for k in range(row_ptr[r], row_ptr[r + 1]):
            new_cols.append(col_ind[k])
            new_vals.append(vals[k])
            if k in picked:  # the same column again, right after
                new_cols.append(col_ind[k])
                new_vals.append(0.5 + rng.random())
        new_ptr.append(len(new_cols))
    new_ptr = np.asarray(new_ptr, np.int32)
    new_cols = np.asarray(new_cols, np.int32)
    new_vals = np.asarray(new_vals)
    rhs = rng.standard_normal(len(new_ptr) - 1)
    g = rng.standard_normal(len(gold["bc_dofs"]))

    from oracle import pyoracle as orc
    ev, er = orc.BoundaryMap(gold["bc_dofs"], new_ptr, new_cols).prepare_forward_solve(
        new_vals, rhs, g)
    case = (dev(gold["bc_dofs"]), dev(new_ptr), dev(new_cols), dev(new_vals), dev(rhs), dev(g))
    ref = with_handle(*case)
    for _ in range(2):
        rc, v, r = no_alloc(*case)
        assert rc == 0, lib().lib().gbfem_last_error().decode()
        assert_same((v, r), ref)
        assert np.array_equal(v.cpu().numpy(), ev) and np.array_equal(r.cpu().numpy(), er)
    # every entry of an unconstrained row in a constrained column is zero,
    # the repeated ones included
    row_of = np.repeat(np.arange(len(new_ptr) - 1), np.diff(new_ptr))
    bcl = sorted(bc)
    lifted = np.isin(new_cols, bcl) & ~np.isin(row_of, bcl)
    assert np.all(v.cpu().numpy()[lifted] == 0.0)


def test_alternating_problems_leave_no_state_behind():
    a, b = golden_case(), cavity_case()
    ref_a, ref_b = with_handle(*a), with_handle(*b)
    for case, ref in ((a, ref_a), (b, ref_b), (a, ref_a), (b, ref_b)):
        rc, v, r = no_alloc(*case)
        assert rc == 0
        assert_same((v, r), ref)


def test_rejected_input_then_valid_call():
    dofs, row_ptr, col_ind, vals, rhs, g = golden_case()
    bad = torch.cat([dofs, dofs[:1]])
    g_bad = torch.cat([g, g[:1]])
    rc, v, r = no_alloc(bad, row_ptr, col_ind, vals, rhs, g_bad)
    assert rc == lib().GBFEM_EDATA
    assert "unique" in lib().lib().gbfem_last_error().decode()
    assert torch.equal(v, vals) and torch.equal(r, rhs)  # untouched
    out_of_range = dofs.clone()
    out_of_range[0] = row_ptr.numel() + 5
    rc, _, _ = no_alloc(out_of_range, row_ptr, col_ind, vals, rhs, g)
    assert rc == lib().GBFEM_EDATA
    rc, v, r = no_alloc(dofs, row_ptr, col_ind, vals, rhs, g)
    assert rc == 0
    assert_same((v, r), with_handle(dofs, row_ptr, col_ind, vals, rhs, g))


def test_capacity_limit_is_enforced():
    L = lib()
    one = torch.zeros(1, dtype=torch.int32, device="cuda")
    x = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = L.lib().gbfem_prepare_forward_solve_noalloc(1, ptr(one), MAX_ROWS + 1, ptr(one),
                                                     ptr(one), ptr(x), ptr(x.clone()),
                                                     ptr(x.clone()), stream())
    assert rc == L.GBFEM_EINVAL
    assert "capacity" in L.lib().gbfem_last_error().decode()
