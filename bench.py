"""Benchmark of the femx assembly hot path on GB300.

Workload (default, one GPU): P1 Poisson on a structured 1024x1024 grid split
into 2,097,152 triangles (1,050,625 nodes, 7,346,177 nonzeros), FP64,
per-element conductivity kappa = exp(g) with g a seeded Gaussian random field
(correlation length 0.05, variance 1), Fourier-mode source, homogeneous
Dirichlet data on the boundary. One step is the reference's forward-solve
preparation plus a Krylov-like product chain:
    assemble residual + Jacobian (CSR)   (assembly::assemble)
    rhs = -res                           (VectorHandler::axpby)
    prepareForwardSolve                  (BoundaryMap lifting)
    10 x CSR SpMV, x <- A x / 8          (MatrixHandler::matvec)
Synthetic seeded inputs stand in for real data (no dataset is involved).

value   elements/s, inputs resident in HBM, CUDA events on the launch stream,
        L2 flushed (512 MB write) before every step, outside the events.
e2e     the same steps through the public API with pinned host buffers:
        kappa, f, u copied in and rhs, x copied out inside the timed region.
--impl reference: the CPU oracle (a serial restatement of femx's own CPU
        path, which has no threading) on the host cores, same workload.
Multi-GPU (torchrun): replicas only — each rank runs its own instance, no
collective on the data path; value = all ranks' elements / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "NS P2/P1 Jacobian elems/s & VJP grads/s vs plain FP64 GPU path at stated rel err"
NX = 1024
NSPMV = 10
SPMV_SCALE = 0.125


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_table():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh)
    return {}


def make_inputs():
    from femx_gb300 import meshes
    coords, conn = meshes.structured_tri(NX)
    kappa = np.exp(meshes.grf_centroids(coords, conn, seed=2, ell=0.05, var=1.0, grid=1024))
    f = meshes.fourier_source(coords, 1)
    u = np.zeros(coords.shape[0])
    bdofs = meshes.dirichlet_dofs(coords, meshes.boundary_nodes(coords))
    g = np.zeros(len(bdofs))
    return coords, conn, kappa, f, u, bdofs, g


class Clocks:
    """nvidia-smi sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)),
                "reasons": sorted(reasons), "samples": len(sm)}


def fp64_peak_tflops(torch, A_lib):
    """Measured FP64 FMA ceiling (TFLOP/s) of this GPU."""
    import ctypes as C
    props = torch.cuda.get_device_properties(0)
    blocks, threads, iters = props.multi_processor_count * 16, 256, 4096
    out = torch.empty(blocks * threads, dtype=torch.float64, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    call = A_lib.lib().gbfem_probe_fp64_fma
    for _ in range(2):
        A_lib.check(call(blocks, threads, iters, C.c_void_p(out.data_ptr()), s))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    A_lib.check(call(blocks, threads, iters, C.c_void_p(out.data_ptr()), s))
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) * 1e-3
    return 16.0 * iters * blocks * threads / t / 1e12


def run_reference(args, rank):
    """CPU oracle arm: same workload, serial restatement of femx's CPU path."""
    from oracle import pyoracle as orc
    from femx_gb300 import meshes
    coords, conn, kappa, f, u, bdofs, g = make_inputs()
    n, e = coords.shape[0], conn.shape[0]
    offs, dofs = meshes.scalar_elem_dofs(conn)
    t0 = time.perf_counter()
    om = orc.AssemblyMap(n, n, offs, dofs, offs, dofs)
    q = orc.P1Quad(coords, conn)
    ob = orc.BoundaryMap(bdofs, om.row_ptr, om.col_ind)
    setup_s = time.perf_counter() - t0
    x0 = np.random.default_rng(5).standard_normal(n)

    def step():
        res, vals = orc.assemble_p1_kappa(om, q, kappa, f, u)
        vals, rhs = ob.prepare_forward_solve(vals, -res, g)
        x = rhs
        for _ in range(NSPMV):
            x = orc.matvec(om.row_ptr, om.col_ind, vals, x, alpha=SPMV_SCALE)
        return x

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = (time.perf_counter() - t0) / args.steps
    value = e / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "elements/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)",
        "config": config_block(),
        "cpu_baseline": {"value": value, "unit": "elements/s", "cores": 1, "kind": "port",
                         "sample": f"full workload, {args.steps} steps after {args.warmup} "
                                   f"warm-up (setup {setup_s:.1f}s excluded)"},
        "e2e": {"value": value, "unit": "elements/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "notes": "femx's generic CPU assembly and host matvec are single-threaded "
                 "(no OpenMP on this path); the oracle restates them serially, so one "
                 "core is what the reference implementation uses",
    }
    print(json.dumps(line), flush=True)


def config_block():
    from femx_gb300 import meshes
    c = meshes.structured_counts(NX)
    return {"workload": f"poisson_p1_kappa_{NX}x{NX}_assemble_bc_{NSPMV}spmv",
            "elements": c["elems"], "nodes": c["nodes"], "nnz": c["nnz_p1"],
            "kappa": "exp(GRF, ell=0.05, var=1)", "source": "8 Fourier modes",
            "dirichlet": "all boundary nodes", "l2": "flushed (512 MB write) before each step"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank == 0:
            run_reference(args, rank)
        return

    import torch
    import torch.distributed as dist
    from femx_gb300 import _lib as L
    from femx_gb300 import assembly as A
    from femx_gb300 import build as B
    from femx_gb300 import meshes

    if not os.path.exists(B.LIB):
        B.build()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    coords, conn, kappa, f, u, bdofs, g = make_inputs()
    n, e = coords.shape[0], conn.shape[0]
    offs, dofs = meshes.scalar_elem_dofs(conn)

    def d(a, dtype=None):
        t = torch.from_numpy(np.ascontiguousarray(a))
        return (t if dtype is None else t.to(dtype)).cuda()

    amap = A.makeAssemblyMap(n, n, d(offs), d(dofs), d(offs), d(dofs))
    pat = amap.pattern()
    bc = A.makeBoundaryMap(d(bdofs), pat)
    coords_d, kappa_d, f_d, u_d, g_d = d(coords), d(kappa), d(f), d(u), d(g)
    res = torch.zeros(n, dtype=torch.float64, device="cuda")
    rhs = torch.zeros_like(res)
    xa = torch.zeros_like(res)
    xb = torch.zeros_like(res)
    jac = A.CsrMatrix(pat)
    nnz = pat.nnz
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def step(ev=None):
        if ev is not None:
            ev[0].record(stream)
        A.assembleP1Kappa(amap, coords_d, kappa_d, f_d, u_d, res, jac)
        if ev is not None:
            ev[1].record(stream)
        A.axpby(-1.0, res, 0.0, rhs)
        A.prepareForwardSolve(bc, jac, rhs, g_d)
        if ev is not None:
            ev[2].record(stream)
        x, y = rhs, xa
        for i in range(NSPMV):
            A.matvec(jac, x, y, alpha=SPMV_SCALE)
            x, y = y, (xb if y is xa else xa)
        if ev is not None:
            ev[3].record(stream)
        return x

    launches_per_step = 1 + 1 + 1 + NSPMV  # assemble, axpby, lifting, SpMVs

    for _ in range(args.warmup):
        step()
    amap.check()
    torch.cuda.synchronize()

    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(args.steps)]
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        for s in range(args.steps):
            flush.zero_()
            step(evs[s])
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t_asm = sum(ev[0].elapsed_time(ev[1]) for ev in evs) / args.steps * 1e-3
    t_bc = sum(ev[1].elapsed_time(ev[2]) for ev in evs) / args.steps * 1e-3
    t_spmv = sum(ev[2].elapsed_time(ev[3]) for ev in evs) / args.steps * 1e-3
    t_step = t_asm + t_bc + t_spmv
    if world > 1:
        tt = torch.tensor([t_step], dtype=torch.float64, device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_step = float(tt.item())

    # e2e: public API with pinned host buffers, copies inside the timed region
    kappa_h = torch.from_numpy(kappa).pin_memory()
    f_h = torch.from_numpy(f).pin_memory()
    u_h = torch.from_numpy(u).pin_memory()
    rhs_h = torch.empty(n, dtype=torch.float64).pin_memory()
    x_h = torch.empty(n, dtype=torch.float64).pin_memory()
    h2d = 8 * e + 8 * n + 8 * n
    d2h = 8 * n + 8 * n

    def e2e_step():
        kappa_d.copy_(kappa_h, non_blocking=True)
        f_d.copy_(f_h, non_blocking=True)
        u_d.copy_(u_h, non_blocking=True)
        x = step()
        rhs_h.copy_(rhs, non_blocking=True)
        x_h.copy_(x, non_blocking=True)

    for _ in range(2):
        e2e_step()
    torch.cuda.synchronize()
    e2e_t = 0.0
    for s in range(args.steps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        e2e_step()
        e1.record(stream)
        e1.synchronize()
        e2e_t += e0.elapsed_time(e1) * 1e-3
    e2e_t /= args.steps
    if world > 1:
        tt = torch.tensor([e2e_t], dtype=torch.float64, device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_t = float(tt.item())

    hbm, peak_kind = peaks()
    b_asm = 20 * e + 32 * n + 8 * nnz
    b_spmv = 12 * nnz + 20 * n
    t_one_spmv = t_spmv / NSPMV
    traffic = traffic_table()
    kern = {
        "p1_assemble": {"bound": "hbm", "achieved": b_asm / t_asm / 1e9, "peak": hbm,
                        "unit": "GB/s", "frac": b_asm / t_asm / 1e9 / hbm,
                        "traffic": traffic.get("p1_assemble"), "launch_ms": t_asm * 1e3,
                        "algorithmic_bytes": b_asm},
        "spmv": {"bound": "hbm", "achieved": b_spmv / t_one_spmv / 1e9, "peak": hbm,
                 "unit": "GB/s", "frac": b_spmv / t_one_spmv / 1e9 / hbm,
                 "traffic": traffic.get("spmv"), "launch_ms": t_one_spmv * 1e3,
                 "algorithmic_bytes": b_spmv},
    }
    dominant = "p1_assemble" if t_asm >= t_spmv else "spmv"
    roof = dict(kern[dominant])
    roof["kernel"] = dominant
    roof["peak_source"] = f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})"
    fp64 = fp64_peak_tflops(torch, L)

    line = {
        "metric": METRIC, "value": world * e / t_step, "unit": "elements/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded)", "config": config_block(),
        "e2e": {"value": world * e / e2e_t, "unit": "elements/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": e2e_t * 1e3},
        "roofline": roof,
        "kernels": kern,
        "phases_ms": {"assemble": t_asm * 1e3, "rhs_and_lifting": t_bc * 1e3,
                      "spmv_x10": t_spmv * 1e3},
        "nnz_per_s": world * nnz / t_asm,
        "fp64_fma_peak_tflops_measured": fp64,
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clk.summary(),
        "scaling_mode": "replicas" if world > 1 else "single",
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(coords, conn, kappa, f, u, bdofs, g)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def cpu_baseline(coords, conn, kappa, f, u, bdofs, g):
    """Oracle port on one host core, bounded sample of the same workload."""
    from oracle import pyoracle as orc
    from femx_gb300 import meshes
    n, e = coords.shape[0], conn.shape[0]
    offs, dofs = meshes.scalar_elem_dofs(conn)
    om = orc.AssemblyMap(n, n, offs, dofs, offs, dofs)
    q = orc.P1Quad(coords, conn)
    ob = orc.BoundaryMap(bdofs, om.row_ptr, om.col_ind)
    steps, t_total = 0, 0.0
    while t_total < 10.0 and steps < 20:
        t0 = time.perf_counter()
        res, vals = orc.assemble_p1_kappa(om, q, kappa, f, u)
        vals, rhs = ob.prepare_forward_solve(vals, -res, g)
        x = rhs
        for _ in range(NSPMV):
            x = orc.matvec(om.row_ptr, om.col_ind, vals, x, alpha=SPMV_SCALE)
        t_total += time.perf_counter() - t0
        steps += 1
    return {"value": e * steps / t_total, "unit": "elements/s", "cores": 1, "kind": "port",
            "sample": f"{steps} full steps of the same 1024x1024 workload (serial oracle)"}


if __name__ == "__main__":
    main()
