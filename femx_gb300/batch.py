"""Batched assembly of many instances in one persistent launch, and its
autotuner.

``Batch`` wraps gbfem_batch_create/run: every instance is a P1 κ-Poisson or a
Taylor–Hood NS assembly (residual + Jacobian, and the residual VJPs when an
adjoint ``lam`` is given) on its own AssemblyMap. ``run()`` enqueues two
kernels and allocates nothing, so it can be captured in a CUDA graph
(``Batch.graph()``).

``autotune()`` times the launch parameters on the actual batch — elements
per P1 work item, Taylor–Hood elements per work item, resident blocks per
SM, the staging depth (work items claimed ahead with their inputs
prefetched into L2) and the scatter scheme (FP64 atomics, or colouring:
colour rounds with plain adds, bitwise reproducible) — and caches the
fastest per (GPU, precision, batch size class, determinism) in a JSON file
(``$GBFEM_TUNE_CACHE`` or ``~/.cache/gbfem/tune.json``). With
``deterministic=True`` only the colouring scheme is a candidate.
"""
from __future__ import annotations

import ctypes as C
import json
import math
import os

import torch

from . import _lib
from ._lib import call
from .assembly import PRECISIONS, AssemblyMap, _dev, _ptr, _stream

__all__ = ["Batch", "P1Instance", "THInstance", "autotune", "DEFAULT_PARAMS"]

DEFAULT_PARAMS = {"p1_chunk": 512, "th_chunk": 16, "blocks_per_sm": 8, "stage_depth": 0,
                  "scatter": "atomic"}
SEARCH = {"p1_chunk": (256, 512, 1024, 2048), "th_chunk": (8, 16, 32, 64),
          "blocks_per_sm": (4, 6, 8, 12), "stage_depth": (0, 1),
          "scatter": ("atomic", "colour")}


class P1Instance:
    """κ-Poisson instance: outputs res, vals (and g_u, g_m when lam is set)."""

    def __init__(self, amap: AssemblyMap, coords, kappa, u, f=None, lam=None, conn=None):
        self.amap = amap
        self.coords = _dev(coords, torch.float64, "coords")
        self.kappa = _dev(kappa, torch.float64, "kappa")
        self.u = _dev(u, torch.float64, "state")
        self.f = _dev(f, torch.float64, "source", allow_none=True)
        self.lam = _dev(lam, torch.float64, "adjoint", allow_none=True)
        self.conn = _dev(conn, torch.int32, "conn", allow_none=True)
        self.res = torch.zeros(amap.numRes(), dtype=torch.float64, device="cuda")
        self.vals = torch.zeros(amap.pattern().nnz, dtype=torch.float64, device="cuda")
        self.g_u = torch.zeros_like(self.u) if lam is not None else None
        self.g_m = torch.zeros_like(self.kappa) if lam is not None else None

    def desc(self):
        return _lib.BatchInstance(
            _lib.BATCH_P1_KAPPA, self.amap.handle, self.coords.shape[0], _ptr(self.coords),
            _ptr(self.conn), _ptr(self.kappa), _ptr(self.f), 0.0, _ptr(self.u), _ptr(self.lam),
            _ptr(self.res), _ptr(self.vals), _ptr(self.g_u), _ptr(self.g_m))


class THInstance:
    """Taylor–Hood instance: outputs res, vals (and g_state = J^T lam)."""

    def __init__(self, amap: AssemblyMap, coords, conn6, nu, state, lam=None):
        self.amap = amap
        self.coords = _dev(coords, torch.float64, "coords")
        self.conn6 = _dev(conn6, torch.int32, "conn6")
        self.nu = float(nu)
        self.state = _dev(state, torch.float64, "state")
        self.lam = _dev(lam, torch.float64, "adjoint", allow_none=True)
        self.res = torch.zeros(amap.numRes(), dtype=torch.float64, device="cuda")
        self.vals = torch.zeros(amap.pattern().nnz, dtype=torch.float64, device="cuda")
        self.g_u = torch.zeros_like(self.state) if lam is not None else None

    def desc(self):
        return _lib.BatchInstance(
            _lib.BATCH_TH_NS, self.amap.handle, self.coords.shape[0], _ptr(self.coords),
            _ptr(self.conn6), None, None, self.nu, _ptr(self.state), _ptr(self.lam),
            _ptr(self.res), _ptr(self.vals), _ptr(self.g_u), None)


class Batch:
    """coloured=True colours every instance's map first, so that runs may
    take the colouring scatter scheme (scatter="colour")."""

    def __init__(self, instances, coloured=False):
        self.instances = list(instances)
        self.coloured = bool(coloured)
        if self.coloured:
            for x in self.instances:
                x.amap.enableColouring()
        arr = (_lib.BatchInstance * len(self.instances))(*[x.desc() for x in self.instances])
        h = C.c_void_p()
        call("gbfem_batch_create", len(self.instances), arr, _stream(), C.byref(h))
        self._h = h
        self.num_elems = int(_lib.lib().gbfem_batch_num_elems(h))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and _lib._lib is not None:
            _lib._lib.gbfem_batch_destroy(h)
            self._h = None

    def run(self, precision="fp32_quad", p1_chunk=None, th_chunk=None, blocks_per_sm=None,
            stage_depth=None, scatter=None):
        p = dict(DEFAULT_PARAMS)
        p.update({k: v for k, v in (("p1_chunk", p1_chunk), ("th_chunk", th_chunk),
                                    ("blocks_per_sm", blocks_per_sm),
                                    ("stage_depth", stage_depth), ("scatter", scatter))
                  if v is not None})
        mode = PRECISIONS[precision] | (_lib.COLOURED if p["scatter"] == "colour" else 0)
        call("gbfem_batch_run", self._h, mode, p["p1_chunk"], p["th_chunk"],
             p["blocks_per_sm"], p["stage_depth"], _stream())

    def check(self):
        call("gbfem_batch_check", self._h, _stream())

    def graph(self, precision="fp32_quad", **params):
        """Capture one run() into a CUDA graph (warm up outside the capture)."""
        self.run(precision, **params)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run(precision, **params)
        return g

    def signature(self):
        n_p1 = sum(isinstance(x, P1Instance) for x in self.instances)
        return f"p1={n_p1},th={len(self.instances) - n_p1},elems~2^{round(math.log2(max(self.num_elems, 1)))}"


def _cache_path():
    return os.environ.get("GBFEM_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "gbfem", "tune.json"))


def _candidates(batch: Batch, precision, deterministic):
    search = dict(SEARCH)
    if deterministic:
        search["scatter"] = ("colour",)
    elif not batch.coloured or precision == "mixed":
        search["scatter"] = ("atomic",)
    return search


def autotune(batch: Batch, precision="fp32_quad", reps=3, use_cache=True,
             deterministic=False):
    """Coordinate search over SEARCH, starting from DEFAULT_PARAMS (the
    scatter axis needs a Batch made with coloured=True; deterministic=True
    keeps it at colouring, which MIXED does not offer). Returns (params,
    timings) and stores the winner in the cache."""
    if deterministic and (not batch.coloured or precision == "mixed"):
        raise ValueError("deterministic batch runs need Batch(coloured=True) and FP64 or "
                         "FP32_QUAD")
    gpu = torch.cuda.get_device_name()
    key = f"{gpu}|batch|{precision}|det={int(deterministic)}|{batch.signature()}"
    path = _cache_path()
    cache = {}
    if os.path.exists(path):
        try:
            with open(path) as fh:
                cache = json.load(fh)
        except (OSError, ValueError):
            cache = {}
    if use_cache and key in cache:
        return dict(cache[key]["params"]), {"cached": True}

    def time_of(params):
        batch.run(precision, **params)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            batch.run(precision, **params)
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    search = _candidates(batch, precision, deterministic)
    best = dict(DEFAULT_PARAMS)
    best["scatter"] = search["scatter"][0]
    best_t = time_of(best)
    timings = {json.dumps(best, sort_keys=True): best_t}
    for name, choices in search.items():
        for v in choices:
            cand = dict(best)
            cand[name] = v
            k = json.dumps(cand, sort_keys=True)
            if k not in timings:
                timings[k] = time_of(cand)
            if timings[k] < best_t:
                best, best_t = cand, timings[k]
    cache[key] = {"params": best, "ms": best_t}
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        with open(path, "w") as fh:
            json.dump(cache, fh, indent=1, sort_keys=True)
    except OSError:
        pass
    return best, timings
