"""femx-shaped Python API over libgbfem (device tensors in, device tensors out).

Names follow femx's C++ API so that code written against
``femx::assembly`` / ``femx::linalg`` reads the same:

  makeAssemblyMap        femx/assembly/AssemblyMap.hpp:230-234
  makeBoundaryMap        femx/assembly/BoundaryMap.hpp:183-184
  replaceRows / replaceRes / zeroBoundary / prepareForwardSolve
                         femx/assembly/BoundaryMap.hpp:215-291
  assemble (per operator) femx/assembly/CudaAssembly.hpp:319-364
  matvec / matvecT       femx/linalg/handler/MatrixHandler.hpp:270-317
  axpby                  femx/linalg/handler/VectorHandler.hpp

Arguments are torch CUDA tensors (int32 indices, float64 values). Every call
runs on the current torch stream; errors raise :class:`GbfemError` with
femx's require() messages. Layout mismatches between matrices and maps are
rejected like femx's ``layoutId`` checks (Assembly.hpp:85-86,
BoundaryMap.cpp:20-24).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from . import _lib
from ._lib import GbfemError, call

__all__ = [
    "GbfemError", "CsrPattern", "CsrMatrix", "AssemblyMap", "BoundaryMap",
    "makeAssemblyMap", "makeAssemblyMapFromElems", "makeBoundaryMap",
    "replaceRows", "replaceRes", "zeroBoundary", "prepareForwardSolve",
    "assembleP1Kappa", "vjpP1Kappa", "assembleTaylorHood", "matvec", "matvecT",
    "axpby", "transpose", "vjpTaylorHood", "assembleNavier", "vjpNavierHist", "PRECISIONS",
]

PRECISIONS = {"fp64": _lib.PREC_FP64, "fp32_quad": _lib.PREC_FP32_QUAD,
              "mixed": _lib.PREC_MIXED, "double_float": _lib.PREC_DOUBLE_FLOAT}


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


def _dev(t, dtype, name, allow_none=False):
    if t is None:
        if allow_none:
            return None
        raise GbfemError(_lib.GBFEM_EINVAL, f"{name} must not be None")
    if not isinstance(t, torch.Tensor):
        t = torch.as_tensor(t)
    if t.dtype != dtype:
        raise GbfemError(_lib.GBFEM_EINVAL, f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_cuda:
        raise GbfemError(_lib.GBFEM_EINVAL, f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise GbfemError(_lib.GBFEM_EINVAL, f"{name} must be contiguous")
    return t


class _CudaArray:
    """Non-owning __cuda_array_interface__ over handle-owned device memory."""

    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {
            "shape": (int(n),), "typestr": typestr, "data": (int(ptr or 0), False),
            "version": 3, "strides": None,
        }


def _view_i32(ptr, n, owner):
    if n == 0 or not ptr:
        return torch.zeros(0, dtype=torch.int32, device="cuda")
    t = torch.as_tensor(_CudaArray(ptr, n, "<i4"), device="cuda")
    t._gbfem_owner = owner  # keep the handle alive as long as the view
    return t


@dataclass(eq=False)
class CsrPattern:
    """Device CSR pattern (femx/linalg/CsrPattern.hpp:42-217)."""

    rows: int
    cols: int
    row_ptr: torch.Tensor
    col_ind: torch.Tensor
    layout_id: int

    @property
    def nnz(self) -> int:
        return int(self.col_ind.numel())

    def layoutId(self) -> int:
        return self.layout_id


class CsrMatrix:
    """Values over a shared pattern (femx/linalg/CsrMatrix.hpp:17-105)."""

    def __init__(self, pattern: CsrPattern, vals: torch.Tensor | None = None):
        self.pattern = pattern
        if vals is None:
            vals = torch.zeros(pattern.nnz, dtype=torch.float64, device="cuda")
        vals = _dev(vals, torch.float64, "CSR values")
        if vals.numel() != pattern.nnz:
            raise GbfemError(_lib.GBFEM_EINVAL, "CSR values do not match the pattern size")
        self.vals = vals

    rows = property(lambda self: self.pattern.rows)
    cols = property(lambda self: self.pattern.cols)
    nnz = property(lambda self: self.pattern.nnz)

    def to_scipy(self):
        import scipy.sparse as sp
        return sp.csr_matrix((self.vals.cpu().numpy(), self.pattern.col_ind.cpu().numpy(),
                              self.pattern.row_ptr.cpu().numpy()),
                             shape=(self.rows, self.cols))


class AssemblyMap:
    """Device AssemblyMap handle (femx/assembly/AssemblyMap.hpp:78-206)."""

    def __init__(self, handle):
        self._h = handle
        v = _lib.AssemblyMapView()
        call("gbfem_assembly_map_get_view", self._h, C.byref(v))
        self._v = v
        self._pattern = CsrPattern(
            v.num_res, v.num_states, _view_i32(v.row_ptr, v.num_res + 1, self),
            _view_i32(v.col_ind, v.nnz, self), int(v.layout_id))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.gbfem_assembly_map_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def numElems(self): return self._v.num_elems
    def numRes(self): return self._v.num_res
    def numStates(self): return self._v.num_states
    def maxRes(self): return self._v.max_res
    def maxState(self): return self._v.max_state
    def maxJac(self): return self._v.max_jac
    def pattern(self) -> CsrPattern: return self._pattern

    @property
    def jac_nnz(self) -> int:
        return self._v.jac_nnz

    def view(self) -> dict:
        v = self._v
        return {
            "res_offsets": _view_i32(v.res_offsets, v.num_elems + 1, self),
            "res_dofs": _view_i32(v.res_dofs, self._count(v.res_offsets), self),
            "state_offsets": _view_i32(v.state_offsets, v.num_elems + 1, self),
            "state_dofs": _view_i32(v.state_dofs, self._count(v.state_offsets), self),
            "jac_offsets": _view_i32(v.jac_offsets, v.num_elems + 1, self),
            "jac_map": _view_i32(v.jac_map, v.jac_nnz, self),
        }

    def _count(self, offs_ptr):
        offs = _view_i32(offs_ptr, self._v.num_elems + 1, self)
        return int(offs[-1].item()) if offs.numel() else 0

    def enableDeterministic(self):
        """Build the row-gather tables behind deterministic assembly (setup,
        once per map; synchronizes the current stream)."""
        if not getattr(self, "_gather", False):
            call("gbfem_assembly_map_enable_gather", self._h, _stream())
            self._gather = True

    def enableColouring(self):
        """Colour the elements (no two of a colour share a DOF) for coloured
        assembly: plain adds colour by colour, no atomics, bitwise
        reproducible (setup, once per map; synchronizes the current stream).
        Returns the number of colours."""
        call("gbfem_assembly_map_enable_colouring", self._h, _stream())
        return self.numColours()

    def numColours(self):
        return int(_lib.lib().gbfem_assembly_map_num_colours(self._h))

    def enableTiles(self, coords, conn=None):
        """Build the owner-computes tiles behind tiled P1 assembly (setup,
        once per map; synchronizes the current stream). coords: [nodes, 2]
        FP64 on the device; conn: the geometry connectivity when it is passed
        to the assembly calls (then always), else None. Returns the number of
        tiles."""
        coords = _dev(coords, torch.float64, "coords")
        conn = _dev(conn, torch.int32, "conn", allow_none=True)
        call("gbfem_assembly_map_enable_tiles", self._h, coords.shape[0], _ptr(coords),
             _ptr(conn), _stream())
        return self.numTiles()

    def numTiles(self):
        return int(_lib.lib().gbfem_assembly_map_num_tiles(self._h))

    def check(self):
        """Raise if a kernel met invalid data (e.g. a degenerate element)."""
        call("gbfem_assembly_map_check", self._h, _stream())


class BoundaryMap:
    """Device BoundaryMap handle (femx/assembly/BoundaryMap.hpp:69-175)."""

    def __init__(self, handle):
        self._h = handle
        v = _lib.BoundaryMapView()
        call("gbfem_boundary_map_get_view", self._h, C.byref(v))
        self._v = v

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.gbfem_boundary_map_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    def rows(self): return self._v.num_rows
    def cols(self): return self._v.num_cols
    def nnz(self): return self._v.nnz
    def numBcs(self): return self._v.num_bcs
    def layoutId(self): return int(self._v.layout_id)

    def view(self) -> dict:
        v = self._v
        return {
            "bc_rows": _view_i32(v.bc_rows, v.num_bcs, self),
            "diag": _view_i32(v.diag, v.num_bcs, self),
            "col_offsets": _view_i32(v.col_offsets, v.num_bcs + 1, self),
            "col_entries": _view_i32(v.col_entries, v.num_col_entries, self),
            "col_rows": _view_i32(v.col_rows, v.num_col_entries, self),
            "bc_mask": _view_i32(v.bc_mask, v.num_rows, self),
        }


def makeAssemblyMap(num_res, num_states, res_offsets, res_dofs, state_offsets, state_dofs):
    ro = _dev(res_offsets, torch.int32, "res_offsets")
    rd = _dev(res_dofs, torch.int32, "res_dofs")
    so = _dev(state_offsets, torch.int32, "state_offsets")
    sd = _dev(state_dofs, torch.int32, "state_dofs")
    if ro.numel() != so.numel() or ro.numel() < 1:
        raise GbfemError(_lib.GBFEM_EINVAL, "AssemblyMap residual/state element counts differ")
    h = C.c_void_p()
    call("gbfem_assembly_map_create", int(num_res), int(num_states), ro.numel() - 1,
         _ptr(ro), _ptr(rd), _ptr(so), _ptr(sd), _stream(), C.byref(h))
    return AssemblyMap(h)


def makeAssemblyMapFromElems(num_dofs: int, elem_dofs: torch.Tensor):
    """Square map from a uniform [E, k] DOF table (the DofLayout overload,
    femx/assembly/AssemblyMap.cpp:178-199)."""
    elem_dofs = _dev(elem_dofs, torch.int32, "elem_dofs")
    e, k = elem_dofs.shape
    offs = (torch.arange(e + 1, device="cuda", dtype=torch.int64) * k).to(torch.int32)
    flat = elem_dofs.reshape(-1)
    return makeAssemblyMap(num_dofs, num_dofs, offs, flat, offs, flat)


def makeBoundaryMap(dofs, pattern: CsrPattern):
    d = _dev(dofs, torch.int32, "constrained DOFs")
    h = C.c_void_p()
    call("gbfem_boundary_map_create", d.numel(), _ptr(d), pattern.rows, pattern.cols,
         _ptr(pattern.row_ptr), _ptr(pattern.col_ind), C.c_ulonglong(pattern.layout_id),
         _stream(), C.byref(h))
    return BoundaryMap(h)


def _check_layout(bc: BoundaryMap, mat: CsrMatrix):
    if mat.pattern.layout_id != bc.layoutId():
        raise GbfemError(_lib.GBFEM_EINVAL, "BoundaryMap matrix does not match the mapped CSR layout")


def _check_vec(v, n, name):
    v = _dev(v, torch.float64, name)
    if v.numel() != n:
        raise GbfemError(_lib.GBFEM_EINVAL, f"{name} has size {v.numel()}, expected {n}")
    return v


def replaceRows(bc: BoundaryMap, jac: CsrMatrix, diag: float):
    _check_layout(bc, jac)
    call("gbfem_replace_rows", bc.handle, _ptr(jac.vals), float(diag), _stream())


def replaceRes(bc: BoundaryMap, state, bc_vals, res):
    state = _check_vec(state, bc.rows(), "state")
    res = _check_vec(res, bc.rows(), "residual")
    bc_vals = _check_vec(bc_vals, bc.numBcs(), "prescribed values")
    call("gbfem_replace_res", bc.handle, _ptr(state), _ptr(bc_vals), _ptr(res), _stream())


def zeroBoundary(bc: BoundaryMap, vals):
    vals = _check_vec(vals, bc.rows(), "vector")
    call("gbfem_zero_boundary", bc.handle, _ptr(vals), _stream())


def prepareForwardSolve(bc: BoundaryMap, solve_mat: CsrMatrix, rhs, bc_vals):
    _check_layout(bc, solve_mat)
    rhs = _check_vec(rhs, bc.rows(), "RHS")
    bc_vals = _check_vec(bc_vals, bc.numBcs(), "prescribed values")
    call("gbfem_prepare_forward_solve", bc.handle, _ptr(solve_mat.vals), _ptr(rhs),
         _ptr(bc_vals), _stream())


def _jac_ptr(amap: AssemblyMap, jac):
    if jac is None:
        return None
    if jac.pattern.layout_id != amap.pattern().layout_id:
        raise GbfemError(_lib.GBFEM_EINVAL, "Assembly matrix must use the AssemblyMap CSR layout")
    return _ptr(jac.vals)


def _mode(precision, coloured=False, deterministic=False, tiled=False):
    mode = PRECISIONS[precision]
    if coloured:
        mode |= _lib.COLOURED
    if deterministic:
        mode |= _lib.DETERMINISTIC
    if tiled:
        mode |= _lib.TILED
    return mode


def assembleP1Kappa(amap: AssemblyMap, coords, kappa, f_nodal, u, res, jac=None, conn=None,
                    precision: str = "fp64", coloured: bool = False, tiled: bool = False):
    """Residual (and Jacobian) of the kappa-weighted P1 Poisson operator.
    coloured=True: colour by colour with plain adds (amap.enableColouring()
    first), bitwise reproducible. tiled=True: owner-computes tiles, each row
    written once, no atomics (amap.enableTiles(coords, conn) first), bitwise
    reproducible; with precision="double_float" the FP64-accurate fast
    path."""
    coords = _dev(coords, torch.float64, "coords")
    kappa = _check_vec(kappa, amap.numElems(), "kappa")
    u = _check_vec(u, amap.numStates(), "state")
    res = _check_vec(res, amap.numRes(), "residual")
    f_nodal = _dev(f_nodal, torch.float64, "source", allow_none=True)
    conn = _dev(conn, torch.int32, "conn", allow_none=True)
    call("gbfem_assemble_p1_kappa", amap.handle, coords.shape[0], _ptr(coords), _ptr(conn),
         _ptr(kappa), _ptr(f_nodal), _ptr(u), _ptr(res), _jac_ptr(amap, jac),
         _mode(precision, coloured, tiled=tiled), _stream())


def vjpP1Kappa(amap: AssemblyMap, coords, kappa, u, lam, g_u=None, g_m=None, conn=None,
               precision: str = "fp64", coloured: bool = False, tiled: bool = False):
    coords = _dev(coords, torch.float64, "coords")
    kappa = _check_vec(kappa, amap.numElems(), "kappa")
    u = _check_vec(u, amap.numStates(), "state")
    lam = _check_vec(lam, amap.numRes(), "adjoint")
    if g_u is not None:
        g_u = _check_vec(g_u, amap.numStates(), "state gradient")
    if g_m is not None:
        g_m = _check_vec(g_m, amap.numElems(), "control gradient")
    conn = _dev(conn, torch.int32, "conn", allow_none=True)
    call("gbfem_vjp_p1_kappa", amap.handle, coords.shape[0], _ptr(coords), _ptr(conn),
         _ptr(kappa), _ptr(u), _ptr(lam), _ptr(g_u), _ptr(g_m),
         _mode(precision, coloured, tiled=tiled),
         _stream())


def assembleTaylorHood(amap: AssemblyMap, coords, conn6, nu, state, res, jac=None,
                       precision: str = "fp64", deterministic: bool = False,
                       coloured: bool = False):
    """Taylor-Hood Newton residual (and Jacobian when jac is given).
    deterministic=True sums element rows per CSR row in element order (no
    atomics): bitwise reproducible; the first call on a map builds its
    row-gather tables (amap.enableDeterministic()). coloured=True runs the
    elements colour by colour with plain adds (amap.enableColouring()
    first), also bitwise reproducible."""
    coords = _dev(coords, torch.float64, "coords")
    conn6 = _dev(conn6, torch.int32, "conn6")
    state = _check_vec(state, amap.numStates(), "state")
    res = _check_vec(res, amap.numRes(), "residual")
    if deterministic:
        amap.enableDeterministic()
    call("gbfem_assemble_th_ns", amap.handle, coords.shape[0], _ptr(coords), _ptr(conn6),
         float(nu), _ptr(state), _ptr(res), _jac_ptr(amap, jac),
         _mode(precision, coloured, deterministic), _stream())


def _check_host_vec(v, n, name):
    if not isinstance(v, torch.Tensor) or v.device.type != "cpu" or v.dtype != torch.float64 \
            or not v.is_contiguous() or v.numel() != n:
        raise GbfemError(_lib.GBFEM_EINVAL,
                         f"{name} must be a contiguous float64 host tensor of size {n}")
    return v


def newtonSystemTaylorHoodHost(amap: AssemblyMap, bc: BoundaryMap, coords, conn6, nu,
                               state_host, state, bc_vals, res, jac, res_host,
                               diag: float = 1.0, precision: str = "fp32_quad",
                               deterministic: bool = False):
    """One Newton system from a host-resident state: state_host -> state
    (device), residual + Jacobian (jac may be None) with Dirichlet rows
    (replaceRes with bc_vals, replaceRows with diag), final residual ->
    res_host. The copies overlap the device work (pin the host tensors for
    that); everything is ordered on the current stream."""
    coords = _dev(coords, torch.float64, "coords")
    conn6 = _dev(conn6, torch.int32, "conn6")
    state = _check_vec(state, amap.numStates(), "state")
    res = _check_vec(res, amap.numRes(), "residual")
    bc_vals = _check_vec(bc_vals, bc.numBcs(), "prescribed values")
    state_host = _check_host_vec(state_host, amap.numStates(), "host state")
    res_host = _check_host_vec(res_host, amap.numRes(), "host residual")
    if jac is not None:
        _check_layout(bc, jac)
    mode = PRECISIONS[precision]
    if deterministic:
        amap.enableDeterministic()
        mode |= _lib.DETERMINISTIC
    call("gbfem_newton_system_th_ns_host", amap.handle, bc.handle, coords.shape[0],
         _ptr(coords), _ptr(conn6), float(nu), _ptr(state_host), _ptr(state), _ptr(bc_vals),
         _ptr(res), _jac_ptr(amap, jac), float(diag), _ptr(res_host), mode, _stream())


def vjpTaylorHood(amap: AssemblyMap, coords, conn6, nu, state, lam, g_state,
                  precision: str = "fp64", coloured: bool = False):
    """g_state = J(state)^T lam of the Taylor-Hood residual, without forming J."""
    coords = _dev(coords, torch.float64, "coords")
    conn6 = _dev(conn6, torch.int32, "conn6")
    state = _check_vec(state, amap.numStates(), "state")
    lam = _check_vec(lam, amap.numRes(), "adjoint")
    g_state = _check_vec(g_state, amap.numStates(), "VJP output")
    call("gbfem_vjp_th_ns", amap.handle, coords.shape[0], _ptr(coords), _ptr(conn6),
         float(nu), _ptr(state), _ptr(lam), _ptr(g_state), _mode(precision, coloured),
         _stream())


def assembleNavier(amap: AssemblyMap, coords, conn, rho, mu, dt, step, hist, nxt, res,
                   jac=None, num_hist: int = 2, wrt_hist_lag: int = -1):
    """femx's GLS Navier-Stokes time step (NavierOperator) on P1 triangles:
    res = K(hist) nxt - F(hist) and, with jac, the Jacobian block wrt
    (-1: next state, K; a history lag: zero, as femx's operator).
    hist is lag-major [num_hist * numStates()], lag 0 the current state."""
    coords = _dev(coords, torch.float64, "coords")
    conn = _dev(conn, torch.int32, "conn")
    hist = _check_vec(hist, num_hist * amap.numStates(), "history")
    nxt = _check_vec(nxt, amap.numStates(), "next state")
    res = _check_vec(res, amap.numRes(), "residual")
    call("gbfem_assemble_navier", amap.handle, coords.shape[0], _ptr(coords), _ptr(conn),
         float(rho), float(mu), float(dt), int(step), int(num_hist), int(wrt_hist_lag),
         _ptr(hist), _ptr(nxt), _ptr(res), _jac_ptr(amap, jac), _stream())


def vjpNavierHist(amap: AssemblyMap, coords, conn, rho, mu, dt, step, hist, nxt, adj, out,
                  num_hist: int = 2):
    """out = d(adj . R)/d hist for femx's NS time operator (both lags)."""
    coords = _dev(coords, torch.float64, "coords")
    conn = _dev(conn, torch.int32, "conn")
    hist = _check_vec(hist, num_hist * amap.numStates(), "history")
    nxt = _check_vec(nxt, amap.numStates(), "next state")
    adj = _check_vec(adj, amap.numRes(), "adjoint")
    out = _check_vec(out, num_hist * amap.numStates(), "VJP output")
    call("gbfem_vjp_navier_hist", amap.handle, coords.shape[0], _ptr(coords), _ptr(conn),
         float(rho), float(mu), float(dt), int(step), int(num_hist), _ptr(hist), _ptr(nxt),
         _ptr(adj), _ptr(out), _stream())


def matvec(mat: CsrMatrix, x, y, alpha: float = 1.0, beta: float = 0.0):
    x = _check_vec(x, mat.cols, "matvec input")
    y = _check_vec(y, mat.rows, "matvec output")
    call("gbfem_spmv", mat.rows, mat.cols, _ptr(mat.pattern.row_ptr), _ptr(mat.pattern.col_ind),
         _ptr(mat.vals), _ptr(x), _ptr(y), float(alpha), float(beta), _stream())


def matvecT(mat: CsrMatrix, x, y, alpha: float = 1.0, beta: float = 0.0):
    x = _check_vec(x, mat.rows, "matvecT input")
    y = _check_vec(y, mat.cols, "matvecT output")
    call("gbfem_spmv_t", mat.rows, mat.cols, _ptr(mat.pattern.row_ptr),
         _ptr(mat.pattern.col_ind), _ptr(mat.vals), _ptr(x), _ptr(y), float(alpha),
         float(beta), _stream())


class _CsrTranspose:
    """Cached transposed pattern + value permutation of one source layout
    (femx MatrixHandler::transpose, MatrixHandler.cpp:140-155)."""

    _next_layout = 1 << 62

    def __init__(self, pattern: CsrPattern):
        h = C.c_void_p()
        call("gbfem_csr_transpose_create", pattern.rows, pattern.cols, _ptr(pattern.row_ptr),
             _ptr(pattern.col_ind), _stream(), C.byref(h))
        self._h = h
        v = _lib.CsrTransposeView()
        call("gbfem_csr_transpose_get_view", self._h, C.byref(v))
        _CsrTranspose._next_layout += 1
        self.pattern = CsrPattern(v.rows, v.cols, _view_i32(v.row_ptr, v.rows + 1, self),
                                  _view_i32(v.col_ind, v.nnz, self), _CsrTranspose._next_layout)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.gbfem_csr_transpose_destroy(h)
            self._h = None


def transpose(src: CsrMatrix, dst: CsrMatrix | None = None) -> CsrMatrix:
    """Explicit transpose dst = src^T. The transposed pattern is built once
    per source layout and reused; a dst on that pattern is updated in place
    (values only), otherwise a new matrix is returned."""
    t = getattr(src.pattern, "_transpose", None)
    if t is None:
        t = _CsrTranspose(src.pattern)
        src.pattern._transpose = t
    if dst is not None and dst.vals.data_ptr() == src.vals.data_ptr():
        raise GbfemError(_lib.GBFEM_EINVAL, "CSR transpose does not support in-place output")
    if dst is None or dst.pattern.layout_id != t.pattern.layout_id:
        dst = CsrMatrix(t.pattern)
    call("gbfem_csr_transpose_apply", t._h, _ptr(src.vals), _ptr(dst.vals), _stream())
    return dst


def axpby(a: float, x, b: float, y):
    x = _dev(x, torch.float64, "x")
    y = _dev(y, torch.float64, "y")
    if x.numel() != y.numel():
        raise GbfemError(_lib.GBFEM_EINVAL, "axpby vectors have different sizes")
    call("gbfem_axpby", y.numel(), float(a), _ptr(x), float(b), _ptr(y), _stream())
