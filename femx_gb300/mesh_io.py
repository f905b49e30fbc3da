"""Gmsh mesh ingestion through libgbfem (gbfem_mesh_read_gmsh), with femx's
GmshReader semantics (femx/fem/GmshReader.cpp:446-548): flat arrays ready
for the device path."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import call

__all__ = ["GmshMesh", "read_gmsh"]


@dataclass
class GmshMesh:
    dim: int
    coords: np.ndarray      # [num_nodes, 3]
    conn: np.ndarray        # [num_elems, nodes_per_elem] int32
    elem_etag: np.ndarray
    elem_ptag: np.ndarray
    facet_conn: np.ndarray  # [num_facets, nodes_per_facet] int32
    facet_etag: np.ndarray
    facet_ptag: np.ndarray
    names: dict             # (dim, tag) -> physical name

    def device(self):
        """(coords [N, dim] float64, conn int32) as CUDA tensors."""
        import torch
        c = torch.from_numpy(np.ascontiguousarray(self.coords[:, :self.dim])).cuda()
        return c, torch.from_numpy(np.ascontiguousarray(self.conn)).cuda()


def _arr(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    ct = C.c_double if dtype == np.float64 else C.c_int
    return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ct)), shape=(n,)).astype(dtype).copy()


def read_gmsh(path: str) -> GmshMesh:
    h = C.c_void_p()
    call("gbfem_mesh_read_gmsh", str(path).encode(), C.byref(h))
    try:
        v = _lib.MeshView()
        call("gbfem_mesh_get_view", h, C.byref(v))
        npe, npf = max(v.nodes_per_elem, 1), max(v.nodes_per_facet, 1)
        m = GmshMesh(
            dim=v.dim,
            coords=_arr(v.coords, 3 * v.num_nodes, np.float64).reshape(-1, 3),
            conn=_arr(v.conn, v.num_elems * v.nodes_per_elem, np.int32).reshape(-1, npe),
            elem_etag=_arr(v.elem_etag, v.num_elems, np.int32),
            elem_ptag=_arr(v.elem_ptag, v.num_elems, np.int32),
            facet_conn=_arr(v.facet_conn, v.num_facets * v.nodes_per_facet,
                            np.int32).reshape(-1, npf),
            facet_etag=_arr(v.facet_etag, v.num_facets, np.int32),
            facet_ptag=_arr(v.facet_ptag, v.num_facets, np.int32),
            names={})
        buf = C.create_string_buffer(256)
        for d, tags in ((m.dim, m.elem_ptag), (m.dim - 1, m.facet_ptag)):
            for t in sorted(set(int(x) for x in tags)):
                call("gbfem_mesh_physical_name", h, d, t, buf, 256)
                if buf.value:
                    m.names[(d, t)] = buf.value.decode()
        return m
    finally:
        _lib.lib().gbfem_mesh_destroy(h)
