"""ctypes wrapper of the CPU oracle (oracle/femx_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, by the smoke check and by the
benchmark's CPU legs (CPU baseline, reference arm), never by the product
package. See
oracle/femx_oracle.h for what each function restates and how the oracle is
pinned to the reference.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SRC = os.path.join(HERE, "femx_oracle.cpp")


def build(force: bool = False) -> str:
    """Compile liboracle.so with g++ (portable flags: x86 and aarch64)."""
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(SRC):
        subprocess.check_call([
            "g++", "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", SRC,
            "-o", LIB_PATH,
        ])
    return LIB_PATH


_lib = None

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_last_error.restype = C.c_char_p
        L.orc_map_create.restype = C.c_void_p
        L.orc_map_create.argtypes = [C.c_int, C.c_int, C.c_int, _i32p, _i32p, _i32p, _i32p]
        L.orc_map_sizes.argtypes = [C.c_void_p, _i64p]
        L.orc_map_copy.argtypes = [C.c_void_p, _i32p, _i32p, _i32p, _i32p]
        L.orc_map_free.argtypes = [C.c_void_p]
        L.orc_bc_create.restype = C.c_void_p
        L.orc_bc_create.argtypes = [C.c_int, _i32p, C.c_int, C.c_int, _i32p, _i32p]
        L.orc_bc_sizes.argtypes = [C.c_void_p, _i64p]
        L.orc_bc_copy.argtypes = [C.c_void_p] + [_i32p] * 6
        L.orc_bc_free.argtypes = [C.c_void_p]
        L.orc_replace_rows.argtypes = [C.c_void_p, _i32p, _f64p, C.c_double]
        L.orc_replace_res.argtypes = [C.c_void_p, _f64p, _f64p, _f64p]
        L.orc_zero_boundary.argtypes = [C.c_void_p, _f64p]
        L.orc_prepare_forward_solve.argtypes = [C.c_void_p, _i32p, _f64p, _f64p, _f64p]
        L.orc_matvec.argtypes = [C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, C.c_double, C.c_double]
        L.orc_matvec_t.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, C.c_double, C.c_double]
        L.orc_p1_quad_create.restype = C.c_void_p
        L.orc_p1_quad_create.argtypes = [C.c_int, _f64p, C.c_int, _i32p, C.c_int]
        L.orc_p1_quad_free.argtypes = [C.c_void_p]
        L.orc_p1_quad_tables.argtypes = [C.c_void_p, C.POINTER(C.c_int)] + [
            C.POINTER(C.c_void_p)] * 3
        L.orc_assemble_p1_kappa.argtypes = [C.c_void_p, C.c_void_p, _i32p, _f64p, C.c_void_p, _f64p, _f64p, _f64p]
        L.orc_vjp_p1_kappa.argtypes = [C.c_void_p, C.c_void_p, _i32p, _f64p, _f64p, _f64p, C.c_void_p, C.c_void_p]
        L.orc_assemble_th_ns.argtypes = [C.c_void_p, C.c_int, _f64p, _i32p, C.c_double, _f64p, _f64p, _f64p]
        L.orc_th_quad_create.restype = C.c_void_p
        L.orc_th_quad_create.argtypes = [C.c_int, _f64p, C.c_int, _i32p]
        L.orc_th_quad_free.argtypes = [C.c_void_p]
        L.orc_assemble_th_range.argtypes = [C.c_void_p, C.c_void_p, C.c_double, _f64p, _f64p, _f64p, C.c_int, C.c_int]
        L.orc_assemble_navier.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, _f64p, _f64p, _f64p, C.c_void_p]
        L.orc_vjp_navier_hist.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, _f64p, _f64p, _f64p, _f64p]
        L.orc_assemble_navier_threads.argtypes = [C.c_void_p, C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_int, C.c_int, _f64p, _f64p, _f64p, _f64p, C.c_int]
        L.orc_assemble_th_threads.argtypes = [C.c_void_p, C.c_void_p, C.c_double, _f64p, _f64p, _f64p, C.c_int]
        L.orc_assemble_p1_range.argtypes = [C.c_void_p, C.c_void_p, _i32p, _f64p, C.c_void_p, _f64p, _f64p, _f64p, C.c_int, C.c_int]
        _lib = L
    return _lib


class OracleError(RuntimeError):
    pass


def _check(rc):
    if rc != 0:
        raise OracleError(lib().orc_last_error().decode())


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class AssemblyMap:
    """femx::assembly::makeAssemblyMap restated (AssemblyMap.cpp:54-176)."""

    def __init__(self, num_res, num_states, res_offsets, res_dofs, state_offsets, state_dofs):
        self.res_offsets = _i32(res_offsets)
        self.res_dofs = _i32(res_dofs)
        self.state_offsets = _i32(state_offsets)
        self.state_dofs = _i32(state_dofs)
        self.num_res = int(num_res)
        self.num_states = int(num_states)
        self.num_elems = len(self.res_offsets) - 1
        h = lib().orc_map_create(self.num_res, self.num_states, self.num_elems, self.res_offsets,
                                 self.res_dofs, self.state_offsets, self.state_dofs)
        if not h:
            raise OracleError(lib().orc_last_error().decode())
        self.h = h
        s = np.zeros(5, dtype=np.int64)
        lib().orc_map_sizes(h, s)
        self.nnz, self.jac_nnz, self.max_res, self.max_state, self.max_jac = (int(v) for v in s)
        self.row_ptr = np.zeros(self.num_res + 1, np.int32)
        self.col_ind = np.zeros(self.nnz, np.int32)
        self.jac_offsets = np.zeros(self.num_elems + 1, np.int32)
        self.jac_map = np.zeros(self.jac_nnz, np.int32)
        lib().orc_map_copy(h, self.row_ptr, self.col_ind, self.jac_offsets, self.jac_map)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_map_free(self.h)
            self.h = None


class BoundaryMap:
    """femx::assembly::makeBoundaryMap restated (BoundaryMap.cpp:59-139)."""

    def __init__(self, dofs, row_ptr, col_ind, cols=None):
        self.dofs = _i32(dofs)
        self.row_ptr = _i32(row_ptr)
        self.col_ind = _i32(col_ind)
        rows = len(self.row_ptr) - 1
        cols = rows if cols is None else cols
        h = lib().orc_bc_create(len(self.dofs), self.dofs, rows, cols, self.row_ptr, self.col_ind)
        if not h:
            raise OracleError(lib().orc_last_error().decode())
        self.h = h
        s = np.zeros(2, dtype=np.int64)
        lib().orc_bc_sizes(h, s)
        nb, nc = int(s[0]), int(s[1])
        self.bc_rows = np.zeros(nb, np.int32)
        self.diag = np.zeros(nb, np.int32)
        self.col_offsets = np.zeros(nb + 1, np.int32)
        self.col_entries = np.zeros(nc, np.int32)
        self.col_rows = np.zeros(nc, np.int32)
        self.bc_mask = np.zeros(rows, np.int32)
        lib().orc_bc_copy(h, self.bc_rows, self.diag, self.col_offsets, self.col_entries,
                          self.col_rows, self.bc_mask)

    def replace_rows(self, vals, diag):
        v = _f64(vals).copy()
        _check(lib().orc_replace_rows(self.h, self.row_ptr, v, float(diag)))
        return v

    def replace_res(self, state, bc_vals, res):
        r = _f64(res).copy()
        _check(lib().orc_replace_res(self.h, _f64(state), _f64(bc_vals), r))
        return r

    def zero_boundary(self, v):
        out = _f64(v).copy()
        _check(lib().orc_zero_boundary(self.h, out))
        return out

    def prepare_forward_solve(self, vals, rhs, bc_vals):
        v = _f64(vals).copy()
        r = _f64(rhs).copy()
        _check(lib().orc_prepare_forward_solve(self.h, self.row_ptr, v, r, _f64(bc_vals)))
        return v, r

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_bc_free(self.h)
            self.h = None


def matvec(row_ptr, col_ind, vals, x, y=None, alpha=1.0, beta=0.0):
    row_ptr = _i32(row_ptr)
    rows = len(row_ptr) - 1
    out = np.zeros(rows) if y is None else _f64(y).copy()
    lib().orc_matvec(rows, row_ptr, _i32(col_ind), _f64(vals), _f64(x), out, alpha, beta)
    return out


def matvec_t(row_ptr, col_ind, vals, x, cols, y=None, alpha=1.0, beta=0.0):
    row_ptr = _i32(row_ptr)
    rows = len(row_ptr) - 1
    out = np.zeros(cols) if y is None else _f64(y).copy()
    lib().orc_matvec_t(rows, cols, row_ptr, _i32(col_ind), _f64(vals), _f64(x), out, alpha, beta)
    return out


class P1Quad:
    """makeElementQuadratureData for P1 triangles (ElementQuadratureData.cpp)."""

    def __init__(self, coords, conn, order=2):
        self.coords = _f64(coords)
        self.conn = _i32(conn)
        h = lib().orc_p1_quad_create(self.coords.shape[0], self.coords, self.conn.shape[0],
                                     self.conn, order)
        if not h:
            raise OracleError(lib().orc_last_error().decode())
        self.h = h

    def tables(self):
        """(N [nq, 3], dNdx [E, nq, 3, 2], JxW [E, nq]): femx's
        ElementQuadratureData arrays (copies)."""
        nq = C.c_int()
        ptrs = [C.c_void_p() for _ in range(3)]
        _check(lib().orc_p1_quad_tables(self.h, C.byref(nq), *[C.byref(q) for q in ptrs]))
        ne, k = self.conn.shape[0], nq.value

        def arr(ptr, shape):
            n = int(np.prod(shape))
            buf = (C.c_double * n).from_address(ptr.value)
            return np.frombuffer(buf, dtype=np.float64, count=n).reshape(shape).copy()

        return arr(ptrs[0], (k, 3)), arr(ptrs[1], (ne, k, 3, 2)), arr(ptrs[2], (ne, k))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_p1_quad_free(self.h)
            self.h = None


def assemble_p1_kappa(amap: AssemblyMap, quad: P1Quad, kappa, f_nodal, u):
    res = np.zeros(amap.num_res)
    vals = np.zeros(amap.nnz)
    f = None if f_nodal is None else _f64(f_nodal)
    _check(lib().orc_assemble_p1_kappa(amap.h, quad.h, quad.conn, _f64(kappa), _ptr(f),
                                       _f64(u), res, vals))
    return res, vals


def vjp_p1_kappa(amap: AssemblyMap, quad: P1Quad, kappa, u, lam):
    g_u = np.zeros(amap.num_states)
    g_m = np.zeros(amap.num_elems)
    _check(lib().orc_vjp_p1_kappa(amap.h, quad.h, quad.conn, _f64(kappa), _f64(u), _f64(lam),
                                  _ptr(g_u), _ptr(g_m)))
    return g_u, g_m


def assemble_th_ns(amap: AssemblyMap, coords_p2, conn6, nu, state):
    res = np.zeros(amap.num_res)
    vals = np.zeros(amap.nnz)
    c = _f64(coords_p2)
    _check(lib().orc_assemble_th_ns(amap.h, c.shape[0], c, _i32(conn6), float(nu), _f64(state),
                                    res, vals))
    return res, vals


class THQuad:
    """Per-element Taylor-Hood tables (ElementQuadratureData analogue)."""

    def __init__(self, coords_p2, conn6):
        self.coords = _f64(coords_p2)
        self.conn6 = _i32(conn6)
        h = lib().orc_th_quad_create(self.coords.shape[0], self.coords, self.conn6.shape[0],
                                     self.conn6)
        if not h:
            raise OracleError(lib().orc_last_error().decode())
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.orc_th_quad_free(self.h)
            self.h = None


def assemble_th_range(amap: AssemblyMap, th: THQuad, nu, state, elem_begin=0, elem_end=-1,
                      res=None, vals=None):
    res = np.zeros(amap.num_res) if res is None else res
    vals = np.zeros(amap.nnz) if vals is None else vals
    _check(lib().orc_assemble_th_range(amap.h, th.h, float(nu), _f64(state), res, vals,
                                       int(elem_begin), int(elem_end)))
    return res, vals


def assemble_th_threads(amap: AssemblyMap, th: THQuad, nu, state, nthreads, res=None,
                        vals=None):
    """The Taylor-Hood assembly on `nthreads` host threads (atomic adds)."""
    res = np.zeros(amap.num_res) if res is None else res
    vals = np.zeros(amap.nnz) if vals is None else vals
    _check(lib().orc_assemble_th_threads(amap.h, th.h, float(nu), _f64(state), res, vals,
                                         int(nthreads)))
    return res, vals


def assemble_p1_range(amap: AssemblyMap, quad: P1Quad, kappa, f_nodal, u, elem_begin=0,
                      elem_end=-1, res=None, vals=None):
    res = np.zeros(amap.num_res) if res is None else res
    vals = np.zeros(amap.nnz) if vals is None else vals
    f = None if f_nodal is None else _f64(f_nodal)
    _check(lib().orc_assemble_p1_range(amap.h, quad.h, quad.conn, _f64(kappa), _ptr(f), _f64(u),
                                       res, vals, int(elem_begin), int(elem_end)))
    return res, vals


def assemble_navier(amap: AssemblyMap, quad: P1Quad, rho, mu, dt, step, hist, nxt,
                    num_hist=2, jac=True):
    """femx's GLS NS time operator (order-2 P1Quad): (res, vals or None)."""
    res = np.zeros(amap.num_res)
    vals = np.zeros(amap.nnz) if jac else None
    _check(lib().orc_assemble_navier(amap.h, quad.h, float(rho), float(mu), float(dt), int(step),
                                     int(num_hist), _f64(hist), _f64(nxt), res,
                                     None if vals is None else vals.ctypes.data))
    return res, vals


def vjp_navier_hist(amap: AssemblyMap, quad: P1Quad, rho, mu, dt, step, hist, nxt, adj,
                    num_hist=2):
    """Exact history VJP (dual numbers): [num_hist * num_states]."""
    out = np.zeros(num_hist * amap.num_states)
    _check(lib().orc_vjp_navier_hist(amap.h, quad.h, float(rho), float(mu), float(dt), int(step),
                                     int(num_hist), _f64(hist), _f64(nxt), _f64(adj), out))
    return out


def assemble_navier_threads(amap: AssemblyMap, quad: P1Quad, rho, mu, dt, step, hist, nxt,
                            nthreads, num_hist=2, res=None, vals=None):
    """femx's GLS NS time operator on `nthreads` host threads (atomic adds)."""
    res = np.zeros(amap.num_res) if res is None else res
    vals = np.zeros(amap.nnz) if vals is None else vals
    _check(lib().orc_assemble_navier_threads(amap.h, quad.h, float(rho), float(mu), float(dt),
                                             int(step), int(num_hist), _f64(hist), _f64(nxt),
                                             res, vals, int(nthreads)))
    return res, vals
