"""ctypes binding of libgbfem (include/gbfem.h).

The library is the product: there is no Python or CPU fallback. Loading fails
loudly when libgbfem.so has not been built (run ``__graft_entry__.build()``
or ``python -m femx_gb300.build``).
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

LIB_PATH = _build.LIB

GBFEM_OK = 0
GBFEM_EINVAL = 1
GBFEM_ECUDA = 2
GBFEM_EDATA = 3
GBFEM_ENOMEM = 4

PREC_FP64 = 0
PREC_FP32_QUAD = 1
PREC_MIXED = 2
PREC_DOUBLE_FLOAT = 3
DETERMINISTIC = 0x100
COLOURED = 0x200
TILED = 0x400


class GbfemError(RuntimeError):
    """Raised for a nonzero status; ``code`` is the C status code."""

    def __init__(self, code: int, msg: str):
        super().__init__(msg)
        self.code = code


class AssemblyMapView(C.Structure):
    _fields_ = [
        ("num_elems", C.c_int), ("num_res", C.c_int), ("num_states", C.c_int),
        ("nnz", C.c_int), ("jac_nnz", C.c_int), ("max_res", C.c_int),
        ("max_state", C.c_int), ("max_jac", C.c_int), ("layout_id", C.c_ulonglong),
        ("res_offsets", C.c_void_p), ("res_dofs", C.c_void_p),
        ("state_offsets", C.c_void_p), ("state_dofs", C.c_void_p),
        ("jac_offsets", C.c_void_p), ("jac_map", C.c_void_p),
        ("row_ptr", C.c_void_p), ("col_ind", C.c_void_p),
    ]


class BoundaryMapView(C.Structure):
    _fields_ = [
        ("num_rows", C.c_int), ("num_cols", C.c_int), ("nnz", C.c_int),
        ("num_bcs", C.c_int), ("num_col_entries", C.c_int),
        ("layout_id", C.c_ulonglong),
        ("bc_rows", C.c_void_p), ("diag", C.c_void_p), ("col_offsets", C.c_void_p),
        ("col_entries", C.c_void_p), ("col_rows", C.c_void_p), ("bc_mask", C.c_void_p),
    ]


class CsrTransposeView(C.Structure):
    _fields_ = [
        ("rows", C.c_int), ("cols", C.c_int), ("nnz", C.c_int),
        ("row_ptr", C.c_void_p), ("col_ind", C.c_void_p), ("src_slot", C.c_void_p),
    ]


class MeshView(C.Structure):
    _fields_ = [
        ("dim", C.c_int), ("num_nodes", C.c_int), ("num_elems", C.c_int),
        ("nodes_per_elem", C.c_int), ("num_facets", C.c_int), ("nodes_per_facet", C.c_int),
        ("coords", C.c_void_p), ("conn", C.c_void_p), ("elem_etag", C.c_void_p),
        ("elem_ptag", C.c_void_p), ("facet_conn", C.c_void_p), ("facet_etag", C.c_void_p),
        ("facet_ptag", C.c_void_p),
    ]


class BatchInstance(C.Structure):
    _fields_ = [
        ("kind", C.c_int), ("map", C.c_void_p), ("num_nodes", C.c_int),
        ("coords", C.c_void_p), ("conn", C.c_void_p), ("kappa", C.c_void_p),
        ("f_nodal", C.c_void_p), ("nu", C.c_double), ("state", C.c_void_p),
        ("lam", C.c_void_p), ("res", C.c_void_p), ("vals", C.c_void_p),
        ("g_state", C.c_void_p), ("g_control", C.c_void_p),
    ]


BATCH_P1_KAPPA = 1
BATCH_TH_NS = 2

_vp = C.c_void_p
_i = C.c_int
_d = C.c_double

# name -> (restype, argtypes)
SIGNATURES = {
    "gbfem_last_error": (C.c_char_p, []),
    "gbfem_version": (_i, []),
    "gbfem_assembly_map_create": (_i, [_i, _i, _i, _vp, _vp, _vp, _vp, _vp, C.POINTER(_vp)]),
    "gbfem_assembly_map_get_view": (_i, [_vp, C.POINTER(AssemblyMapView)]),
    "gbfem_assembly_map_destroy": (None, [_vp]),
    "gbfem_assembly_map_check": (_i, [_vp, _vp]),
    "gbfem_assembly_map_enable_gather": (_i, [_vp, _vp]),
    "gbfem_boundary_map_create": (_i, [_i, _vp, _i, _i, _vp, _vp, C.c_ulonglong, _vp,
                                       C.POINTER(_vp)]),
    "gbfem_boundary_map_get_view": (_i, [_vp, C.POINTER(BoundaryMapView)]),
    "gbfem_boundary_map_destroy": (None, [_vp]),
    "gbfem_replace_rows": (_i, [_vp, _vp, _d, _vp]),
    "gbfem_replace_res": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "gbfem_zero_boundary": (_i, [_vp, _vp, _vp]),
    "gbfem_prepare_forward_solve": (_i, [_vp, _vp, _vp, _vp, _vp]),
    "gbfem_prepare_forward_solve_noalloc": (_i, [_i, _vp, _i, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gbfem_spmv": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _d, _d, _vp]),
    "gbfem_spmv_t": (_i, [_i, _i, _vp, _vp, _vp, _vp, _vp, _d, _d, _vp]),
    "gbfem_csr_transpose_create": (_i, [_i, _i, _vp, _vp, _vp, _vp]),
    "gbfem_mesh_read_gmsh": (_i, [C.c_char_p, _vp]),
    "gbfem_mesh_get_view": (_i, [_vp, _vp]),
    "gbfem_mesh_physical_name": (_i, [_vp, _i, _i, C.c_char_p, _i]),
    "gbfem_mesh_destroy": (None, [_vp]),
    "gbfem_csr_transpose_get_view": (_i, [_vp, _vp]),
    "gbfem_csr_transpose_apply": (_i, [_vp, _vp, _vp, _vp]),
    "gbfem_csr_transpose_destroy": (None, [_vp]),
    "gbfem_axpby": (_i, [_i, _d, _vp, _d, _vp, _vp]),
    "gbfem_exp": (_i, [_i, _vp, _vp, _vp]),
    "gbfem_assemble_p1_kappa": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp]),
    "gbfem_vjp_p1_kappa": (_i, [_vp, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, _vp]),
    "gbfem_assemble_th_ns": (_i, [_vp, _i, _vp, _vp, _d, _vp, _vp, _vp, _i, _vp]),
    "gbfem_newton_system_th_ns_host": (_i, [_vp, _vp, _i, _vp, _vp, _d, _vp, _vp, _vp, _vp, _vp,
                                            _d, _vp, _i, _vp]),
    "gbfem_vjp_th_ns": (_i, [_vp, _i, _vp, _vp, _d, _vp, _vp, _vp, _i, _vp]),
    "gbfem_assemble_navier": (_i, [_vp, _i, _vp, _vp, _d, _d, _d, _i, _i, _i, _vp, _vp, _vp,
                                   _vp, _vp]),
    "gbfem_vjp_navier_hist": (_i, [_vp, _i, _vp, _vp, _d, _d, _d, _i, _i, _vp, _vp, _vp, _vp,
                                   _vp]),
    "gbfem_probe_fp64_fma": (_i, [_i, _i, _i, _vp, _vp]),
    "gbfem_batch_create": (_i, [_i, C.POINTER(BatchInstance), _vp, C.POINTER(_vp)]),
    "gbfem_batch_run": (_i, [_vp, _i, _i, _i, _i, _i, _vp]),
    "gbfem_assembly_map_enable_colouring": (_i, [_vp, _vp]),
    "gbfem_assembly_map_num_colours": (_i, [_vp]),
    "gbfem_assembly_map_enable_tiles": (_i, [_vp, _i, _vp, _vp, _vp]),
    "gbfem_assembly_map_num_tiles": (_i, [_vp]),
    "gbfem_batch_check": (_i, [_vp, _vp]),
    "gbfem_batch_num_elems": (C.c_longlong, [_vp]),
    "gbfem_batch_destroy": (None, [_vp]),
    "gbfem_probe_convert": (_i, [_i, _vp, _vp, _vp, _vp]),
    "gbfem_probe_convert_ftz": (_i, [_i, _vp, _vp, _vp]),
    "gbfem_probe_rcp": (_i, [_i, _vp, _vp, _i, _vp]),
    "gbfem_probe_dd": (_i, [_i, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
}

_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                f"libgbfem.so not found at {LIB_PATH}: build it first "
                "(python -m femx_gb300.build); there is no CPU fallback")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int):
    if rc != GBFEM_OK:
        raise GbfemError(rc, lib().gbfem_last_error().decode())


def call(name: str, *args):
    check(getattr(lib(), name)(*args))
