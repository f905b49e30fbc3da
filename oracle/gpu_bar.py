"""The reference's own CUDA assembly kernel as the benchmark's GPU bar.

Test and measurement infrastructure, not product code (bench.py's reference
legs use it). femx's ``assembleKernel`` (femx/assembly/CudaAssembly.hpp:
100-169) is compiled from femx's sources by oracle/ref/Makefile into
``oracle/_ref/gpu_bar.cubin`` for the kappa-weighted P1 operator written in
femx's plug-in form (oracle/ref/gpu_bar.cu), together with the byte layout of
its arguments (``gpu_bar_layout.json``). Here the arguments are filled with
device addresses and sizes and the kernel is launched the way femx's
``assemble`` launches it (one block of 128 threads per element, shared memory
for the element state, coordinates, residual and Jacobian, outputs zeroed
first: CudaAssembly.hpp:319-364), through ``oracle/gpu_bar_launch.cpp``
(CUDA driver API). The element quadrature tables are femx's
ElementQuadratureData, built by the oracle's restatement of it.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_OUT = os.path.join(HERE, "_ref")
CUBIN = os.path.join(REF_OUT, "gpu_bar.cubin")
LAYOUT = os.path.join(REF_OUT, "gpu_bar_layout.json")
SRC = os.path.join(HERE, "gpu_bar_launch.cpp")
LIB = os.path.join(HERE, "libgpubar.so")
THREADS = 128  # femx's configureAssemblyLaunch (CudaAssembly.hpp:249-271)


def unavailable_reason() -> str | None:
    if not (os.path.exists(CUBIN) and os.path.exists(LAYOUT)):
        return ("femx's CUDA assembly kernel was not compiled (oracle/_ref/gpu_bar.cubin is "
                "built from the femx sources by oracle/ref/Makefile where they are present)")
    return None


def _lib():
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", SRC,
                               "-I" + os.path.join(cuda, "include"), "-o", LIB, "-lcuda"])
    L = C.CDLL(LIB)
    L.refbar_last_error.restype = C.c_char_p
    L.refbar_load.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int,
                              C.POINTER(C.c_void_p)]
    L.refbar_param.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_longlong),
                               C.POINTER(C.c_longlong)]
    L.refbar_launch.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), C.c_uint, C.c_uint, C.c_uint,
                                C.c_void_p]
    return L


def _load(L, name_part, sizes):
    """The kernel whose name contains `name_part`, after checking its
    parameter sizes against `sizes` (the layout file's)."""
    name = C.create_string_buffer(512)
    func = C.c_void_p()
    if L.refbar_load(CUBIN.encode(), name_part.encode(), name, 512, C.byref(func)):
        raise RuntimeError(L.refbar_last_error().decode())
    for i, want in enumerate(sizes):
        off, size = C.c_longlong(), C.c_longlong()
        if L.refbar_param(func, i, C.byref(off), C.byref(size)) or size.value != want:
            raise RuntimeError("femx kernel parameter table does not match the layout")
    return func, name.value.decode()


def _fill(spec, values):
    """The bytes of one argument struct: every field at its offset."""
    buf = (C.c_ubyte * spec["size"])()
    for name, field in spec["fields"].items():
        off, size = field[0], field[1]
        spec_f = spec["fields"][name]
        if len(spec_f) > 2 and spec_f[2] == "f64":
            src = C.c_double(float(values[name]))
        else:
            v = int(values[name])
            src = C.c_uint64(v) if size == 8 else C.c_int32(v)
        C.memmove(C.addressof(buf) + off, C.addressof(src), size)
    return buf


class RefP1Assembly:
    """femx's GPU assembly of the kappa-weighted P1 operator on one mesh.
    Arrays are CUDA tensors owned by the caller: coords [N, 2] float64,
    conn [E, 3] int32, kappa [E], f [N] (or None), the AssemblyMap's DOF
    tables and jac_map (femx's AssemblyMapView), the quadrature tables."""

    def __init__(self, torch, coords, conn, kappa, f, tables, map_view):
        reason = unavailable_reason()
        if reason:
            raise RuntimeError(reason)
        self.torch = torch
        self.L = _lib()
        with open(LAYOUT) as fh:
            layout = json.load(fh)
        sizes = [layout["op"]["size"], layout["geom"]["size"], layout["map"]["size"], 8, 8, 8]
        self.func, self.kernel = _load(self.L, "assembleKernel", sizes)
        N, dNdx, JxW = tables
        dev = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
        ne, nn = conn.shape[0], coords.shape[0]
        self.keep = [coords, conn, kappa, f]
        self.N, self.dNdx, self.JxW = dev(N.reshape(-1)), dev(dNdx.reshape(-1)), dev(JxW.reshape(-1))
        self.offs = torch.arange(0, 3 * ne + 1, 3, dtype=torch.int32, device="cuda")
        nq = N.shape[0]
        geom = {"dim": 2, "num_nodes": nn, "num_elems": ne, "max_elem_nodes": 3,
                "coords": coords.data_ptr(), "coords_size": 2 * nn,
                "elem_offsets": self.offs.data_ptr(), "elem_offsets_size": ne + 1,
                "conn": conn.data_ptr(), "conn_size": 3 * ne}
        op = {"q_num_elems": ne, "q_num_qpts": nq, "q_num_shapes": 3, "q_dim": 2,
              "q_N": self.N.data_ptr(), "q_N_size": self.N.numel(),
              "q_dNdx": self.dNdx.data_ptr(), "q_dNdx_size": self.dNdx.numel(),
              "q_JxW": self.JxW.data_ptr(), "q_JxW_size": self.JxW.numel(),
              "kappa": kappa.data_ptr(), "f": f.data_ptr() if f is not None else 0}
        op.update({"g_" + k: v for k, v in geom.items()})
        mv = map_view
        amap = {"num_elems": ne, "num_res": mv["num_res"], "num_states": mv["num_states"],
                "res_offsets": mv["res_offsets"], "res_dofs": mv["res_dofs"],
                "state_offsets": mv["state_offsets"], "state_dofs": mv["state_dofs"],
                "jac_offsets": mv["jac_offsets"], "jac_map": mv["jac_map"],
                "max_res": 3, "max_state": 3, "max_jac": 9}
        self.params = [_fill(layout["op"], op), _fill(layout["geom"], geom),
                       _fill(layout["map"], amap)]
        self.ne = ne
        # assemblySharedBytes (CudaAssembly.hpp:75-86): state + coords + res + jac
        self.smem = (3 + 3 * 2 + 3 + 9) * 8

    def assemble(self, state, res, vals, stream):
        """femx's assemble: zero res and the CSR values, then one block per
        element with FP64 atomics (all on `stream`)."""
        res.zero_()
        vals.zero_()
        ptrs = [C.c_uint64(state.data_ptr()), C.c_uint64(res.data_ptr()),
                C.c_uint64(vals.data_ptr())]
        args = (C.c_void_p * 6)(*[C.addressof(b) for b in self.params],
                                *[C.addressof(p) for p in ptrs])
        if self.L.refbar_launch(self.func, args, self.ne, THREADS, self.smem, C.c_void_p(stream)):
            raise RuntimeError(self.L.refbar_last_error().decode())


class RefNavierAssembly:
    """femx's own GPU time assembly of its NS model: assembleTimeKernel
    (CudaAssembly.hpp:171-236) with femx's NavierOperator<Device>
    (femx/model/ns/Components.hpp:400-577), next-state block, launched as
    femx's time `assemble` does (CudaAssembly.hpp:367-413: outputs zeroed,
    one 128-thread block per element). `tables` are femx's order-2 P1
    quadrature arrays (femx's NavierData uses the same layout), `map_view`
    the AssemblyMap's device arrays in femx's mixed DOF layout."""

    def __init__(self, torch, tables, map_view, num_nodes, rho, mu, dt):
        reason = unavailable_reason()
        if reason:
            raise RuntimeError(reason)
        self.L = _lib()
        with open(LAYOUT) as fh:
            layout = json.load(fh)
        sizes = [layout["navier_op"]["size"], 4, 4, len(layout["wrt_next"]),
                 layout["map"]["size"], 8, 8, 8, 8]
        self.func, self.kernel = _load(self.L, "assembleTimeKernel", sizes)
        N, dNdx, JxW = tables
        dev = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
        self.N, self.dNdx, self.JxW = dev(N.reshape(-1)), dev(dNdx.reshape(-1)), dev(JxW.reshape(-1))
        ne, nq = JxW.shape
        op = {"num_elems": ne, "num_qpts": nq, "num_nodes": 3, "dim": 2,
              "N": self.N.data_ptr(), "N_size": self.N.numel(),
              "dNdx": self.dNdx.data_ptr(), "dNdx_size": self.dNdx.numel(),
              "JxW": self.JxW.data_ptr(), "JxW_size": self.JxW.numel(),
              "rho": rho, "mu": mu, "dt": dt}
        mv = map_view
        amap = {"num_elems": ne, "num_res": mv["num_res"], "num_states": mv["num_states"],
                "res_offsets": mv["res_offsets"], "res_dofs": mv["res_dofs"],
                "state_offsets": mv["state_offsets"], "state_dofs": mv["state_dofs"],
                "jac_offsets": mv["jac_offsets"], "jac_map": mv["jac_map"],
                "max_res": 9, "max_state": 9, "max_jac": 81}
        wrt = layout["wrt_next"]
        self.wrt = (C.c_ubyte * len(wrt))(*wrt)
        self.params = [_fill(layout["navier_op"], op), _fill(layout["map"], amap)]
        self.ne = ne
        self.num_hist = 2
        # timeAssemblySharedBytes (CudaAssembly.hpp:88-98)
        self.smem = ((self.num_hist + 1) * 9 + 9 + 81) * 8

    def assemble(self, step, hist, nxt, res, vals, stream):
        """Next-state residual and Jacobian: zero fill, then the kernel."""
        res.zero_()
        vals.zero_()
        step_c, nh = C.c_int32(step), C.c_int32(self.num_hist)
        ptrs = [C.c_uint64(hist.data_ptr()), C.c_uint64(nxt.data_ptr()),
                C.c_uint64(res.data_ptr()), C.c_uint64(vals.data_ptr())]
        args = (C.c_void_p * 9)(C.addressof(self.params[0]), C.addressof(step_c),
                                C.addressof(nh), C.addressof(self.wrt),
                                C.addressof(self.params[1]), *[C.addressof(p) for p in ptrs])
        if self.L.refbar_launch(self.func, args, self.ne, THREADS, self.smem, C.c_void_p(stream)):
            raise RuntimeError(self.L.refbar_last_error().decode())
