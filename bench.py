"""Benchmark of the femx assembly hot path on GB300.

Headline workload (one GPU): incompressible Navier-Stokes lid-driven cavity,
Taylor-Hood P2/P1 on a structured 256x256 triangulation (131,072 elements,
526,338 velocity + 66,049 pressure DOFs, 17,526,281 nonzeros), Re = 1000
(nu = 1e-3). One step assembles the Newton Jacobian and residual at a
seeded iterate (stream-function velocity, N(0,1) pressure) and applies the
Dirichlet rows (lid u = (1,0), no-slip walls, pressure pinned at vertex 0)
with replaceRes + replaceRows(diag 1), as ConstrainedTimeResidual does.
  value          elements/s of the plain FP64 path (the drop-in; the
                 reference arm computes in FP64 too), its errors against the
                 oracle at full size in rel_err_vs_oracle_full_size
  fp32_quad      the same step with FP32 element quadrature / FP64
                 accumulation, its speed-up over FP64 and its error
  mixed_newton   FP32-quadrature Jacobian, residual to FP64 accuracy
Sub-results in the same line:
  vjp            P1 Poisson 512x512 (524,288 elements): residual VJP w.r.t.
                 the state and the per-element control m = log kappa,
                 grads/s (one gradient = both VJPs once)
  poisson        P1 Poisson 1024x1024 FP64: assembly + rhs = -res +
                 prepareForwardSolve + 10 SpMVs, elements/s
  navier         femx's own GLS Navier-Stokes time operator (CN + AB2) on
                 the 256x256 P1 triangulation: residual + next-state
                 Jacobian, and the history VJP, elements/s, with the oracle
                 (femx's operator restated) on every host core beside it
  batch          256 uneven instances (P1 and Taylor-Hood) in one
                 persistent launch replayed from a CUDA graph, FP32 / MIXED /
                 FP64, autotuned, errors against the FP64 batch
The headline, navier, poisson, vjp and batch entries each carry a CPU
baseline of the oracle timed on this host (cores stated: every core for the
Taylor-Hood and GLS NS loops, as femx's OpenMP NS assembly runs; one core
for the Poisson step, the VJP and the batch, as femx's generic assembly
runs); poisson also reports its full-size errors against the oracle.
Inputs are seeded synthetic fields with the configured shapes (no dataset).
Timing: CUDA events on the launch stream, 512 MB L2 flush before each step
(outside the events), warm-up steps untimed. e2e: the FP64 step through the
public host-state entry (gbfem_newton_system_th_ns_host): the state copied in
from pinned host memory and the final residual copied out, inside the timed
region, the copies overlapping the zero fill and the row replacement (the
FP32-quadrature e2e beside it under fp32_quad).
--impl reference: the CPU oracle (restatement of femx's element loop with the
Taylor-Hood operator) on every host core with atomic adds, the scheme of
femx's OpenMP NS assembly; same headline workload.
Multi-GPU (torchrun): replicas only; value = all ranks' elements / max time.
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
TH_NX, NU = 256, 1.0e-3
# Thread instructions per element of the double-float Taylor-Hood kernel
# (thElemKernelDd), counted by ncu (inst_executed x 32 / elements, 256x256
# cavity): the numerator of its issue roofline.
DF_INSTR_PER_ELEM = 27446
# FP64 instructions per element of the plain FP64 Taylor-Hood kernel
# (thElemKernel64), counted by ncu the same way: DFMA + DMUL + DADD.
FP64_INSTR_PER_ELEM = 1023
VJP_NX = 512
POISSON_NX, NSPMV, SPMV_SCALE = 1024, 10, 0.125
NS_NX = 256


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_table():
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh)
    return {}


# ------------------------------------------------------------------ inputs

def th_inputs(nx):
    from femx_gb300 import meshes
    c3, k3 = meshes.structured_tri(nx)
    cp2, conn6, nv = meshes.p2_mesh(c3, k3)
    offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
    state = meshes.cavity_state(cp2, nv, seed=3)
    bdofs, bvals = meshes.cavity_dirichlet(cp2, cp2.shape[0])
    return dict(coords=cp2, conn6=conn6, nv=nv, offs=offs, dofs=dofs, nd=nd, state=state,
                bdofs=bdofs, bvals=bvals)


def p1_inputs(nx, seed_kappa=2):
    from femx_gb300 import meshes
    coords, conn = meshes.structured_tri(nx)
    kappa = np.exp(meshes.grf_centroids(coords, conn, seed=seed_kappa, ell=0.05, var=1.0,
                                        grid=max(512, nx)))
    f = meshes.fourier_source(coords, 1)
    bdofs = meshes.dirichlet_dofs(coords, meshes.boundary_nodes(coords))
    offs, dofs = meshes.scalar_elem_dofs(conn)
    return dict(coords=coords, conn=conn, kappa=kappa, f=f, bdofs=bdofs, offs=offs, dofs=dofs)


def th_config():
    from femx_gb300 import meshes
    c = meshes.structured_counts(TH_NX)
    return {"workload": f"ns_taylor_hood_p2p1_cavity_{TH_NX}x{TH_NX}_newton_jacobian_residual",
            "elements": c["elems"], "velocity_dofs": 2 * (c["nodes"] + c["edges"]),
            "pressure_dofs": c["nodes"], "nnz": 17526281, "Re": 1000,
            "precision": "fp64 (the plain drop-in path)",
            "bcs": "lid u=(1,0), no-slip walls, pressure pin; replaceRes + replaceRows",
            "l2": "flushed (512 MB write) before each step"}


# ------------------------------------------------------------------ clocks

class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.proc, self.out = index, None, ""

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


# ------------------------------------------------------------------ reference arm

def run_reference(args):
    from oracle import pyoracle as orc
    d = th_inputs(TH_NX)
    nd = d["nd"]
    t0 = time.perf_counter()
    om = orc.AssemblyMap(nd, nd, d["offs"], d["dofs"], d["offs"], d["dofs"])
    th = orc.THQuad(d["coords"], d["conn6"])
    ob = orc.BoundaryMap(d["bdofs"], om.row_ptr, om.col_ind)
    setup_s = time.perf_counter() - t0
    e = d["conn6"].shape[0]
    res = np.zeros(nd)
    vals = np.zeros(om.nnz)

    cores = host_cores()

    def step():
        orc.assemble_th_threads(om, th, NU, d["state"], cores, res, vals)
        orc.lib().orc_replace_res(ob.h, d["state"], d["bvals"], res)
        orc.lib().orc_replace_rows(ob.h, ob.row_ptr, vals, 1.0)

    for _ in range(args.warmup):
        step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    dt = (time.perf_counter() - t0) / args.steps
    value = e / dt
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": value, "unit": "elements/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": th_config(),
        "cpu_baseline": {"value": value, "unit": "elements/s", "cores": cores, "kind": "port",
                         "sample": f"full 256x256 Taylor-Hood mesh, {args.steps} steps after "
                                   f"{args.warmup} warm-up; setup {setup_s:.1f}s excluded"},
        "e2e": {"value": value, "unit": "elements/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "notes": "oracle restatement of femx's element loop with the Taylor-Hood operator, "
                 "run on every host core with atomic adds (the scheme of femx's OpenMP NS "
                 "assembly); Dirichlet rows serial as in femx",
    }), flush=True)


def host_cores():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ------------------------------------------------------------------ GPU arm

class Timer:
    """Per-step CUDA-event timing on the launch stream, L2 flushed before
    every step (outside the events); the timed region is bracketed by a
    barrier + synchronize on both sides (replicas: every rank)."""

    def __init__(self, torch, stream, flush, rep):
        self.torch, self.stream, self.flush, self.rep = torch, stream, flush, rep

    def run(self, fn, steps, warmup):
        torch = self.torch
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        self.rep.barrier()
        torch.cuda.synchronize()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        for a, b in evs:
            self.flush.zero_()
            a.record(self.stream)
            fn()
            b.record(self.stream)
        torch.cuda.synchronize()
        self.rep.barrier()
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in evs) / steps * 1e-3


_FP64_PEAK = []


def fp64_peak_tflops(torch, L):
    """Measured FP64 FMA rate of this GPU (TFLOP/s), probed once per run."""
    if _FP64_PEAK:
        return _FP64_PEAK[0]
    import ctypes as C
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    blocks, threads, iters = props.multi_processor_count * 16, 256, 4096
    out = torch.empty(blocks * threads, dtype=torch.float64, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    f = L.lib().gbfem_probe_fp64_fma
    for _ in range(2):
        L.check(f(blocks, threads, iters, C.c_void_p(out.data_ptr()), s))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    L.check(f(blocks, threads, iters, C.c_void_p(out.data_ptr()), s))
    e1.record()
    torch.cuda.synchronize()
    _FP64_PEAK.append(16.0 * iters * blocks * threads / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return _FP64_PEAK[0]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--only", default="",
                    help="run one workload: th, th64, vjp, poisson, navier, batch")
    ap.add_argument("--batch-instances", type=int, default=256,
                    help="instances in the batched workload (smaller only to profile it)")
    ap.add_argument("--soak", type=float, default=1.0,
                    help="seconds of untimed headline steps before timing (clock sampling)")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    args.warmup = max(args.warmup, 3)

    import torch
    import torch.distributed as dist
    from femx_gb300 import _lib as L
    from femx_gb300 import assembly as A
    from femx_gb300 import build as B

    if not os.path.exists(B.LIB):
        B.build()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    stream = torch.cuda.current_stream()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    from femx_gb300.replicas import Replicas
    rep = Replicas(dist)
    timer = Timer(torch, stream, flush, rep)
    hbm, peak_kind = peaks()
    traffic = traffic_table()

    def d(a, dtype=None):
        t = torch.from_numpy(np.ascontiguousarray(a))
        return (t if dtype is None else t.to(dtype)).cuda()

    def maxrank(x):
        return rep.max_time(x)

    only = args.only
    line = {}
    launches = 0

    # ---------------- headline: Taylor-Hood Newton J + R ----------------
    if only in ("", "th", "th64"):
        nx = 64 if only == "th64" else TH_NX
        t = th_inputs(nx)
        nd, e = t["nd"], t["conn6"].shape[0]
        amap = A.makeAssemblyMap(nd, nd, d(t["offs"]), d(t["dofs"]), d(t["offs"]), d(t["dofs"]))
        pat = amap.pattern()
        bc = A.makeBoundaryMap(d(t["bdofs"]), pat)
        coords, conn6, state = d(t["coords"]), d(t["conn6"]), d(t["state"])
        bvals = d(t["bvals"])
        res = torch.zeros(nd, dtype=torch.float64, device="cuda")
        jac = A.CsrMatrix(pat)

        def th_step(prec, det=False):
            def fn():
                A.assembleTaylorHood(amap, coords, conn6, NU, state, res, jac, precision=prec,
                                     deterministic=det)
                A.replaceRes(bc, state, bvals, res)
                A.replaceRows(bc, jac, 1.0)
            return fn

        # clock soak (~1 s of the headline step) then the timed region
        with Clocks(local) as clk:
            t_end = time.perf_counter() + args.soak
            while time.perf_counter() < t_end:
                th_step("fp32_quad")()
                torch.cuda.synchronize()
            if world > 1:
                dist.barrier()
            torch.cuda.synchronize()
            t_fast = maxrank(timer.run(th_step("fp32_quad"), args.steps, args.warmup))
            if world > 1:
                dist.barrier()
            t_plain = maxrank(timer.run(th_step("fp64"), args.steps, args.warmup))
            t_mixed = maxrank(timer.run(th_step("mixed"), args.steps, args.warmup))
            t_df = maxrank(timer.run(th_step("double_float"), args.steps, args.warmup))
        launches += 4 * args.steps
        amap.check()
        # deterministic mode (row-gather, no atomics): time and bitwise check
        t_det = timer.run(th_step("fp32_quad", det=True), args.steps, args.warmup)
        det_runs = []
        for _ in range(2):
            th_step("fp32_quad", det=True)()
            det_runs.append((res.clone(), jac.vals.clone()))
        det_bitwise = bool(torch.equal(det_runs[0][0], det_runs[1][0])
                           and torch.equal(det_runs[0][1], det_runs[1][1]))
        launches += 4 * args.steps
        # kernel-only time of the fast assembly (no BC kernels)
        t_kern = timer.run(lambda: A.assembleTaylorHood(amap, coords, conn6, NU, state, res, jac,
                                                        precision="fp32_quad"),
                           args.steps, args.warmup)
        t_kern64 = timer.run(lambda: A.assembleTaylorHood(amap, coords, conn6, NU, state, res,
                                                          jac, precision="fp64"),
                             max(3, args.steps // 4), 2)
        t_kern_df = timer.run(lambda: A.assembleTaylorHood(amap, coords, conn6, NU, state, res,
                                                           jac, precision="double_float"),
                              args.steps, args.warmup)
        # accuracy of the fast path against the plain FP64 path at full size
        A.assembleTaylorHood(amap, coords, conn6, NU, state, res, jac, precision="fp64")
        j64, r64 = jac.vals.clone(), res.clone()
        # the Taylor-Hood state VJP g = J(u)^T lam without forming J (the
        # transpose action behind the autograd wrapper), against J^T lam of
        # the FP64 Jacobian just assembled (gbfem_spmv_t)
        lam_th = torch.from_numpy(np.random.default_rng(7).standard_normal(nd)).cuda()
        g_ref = torch.zeros(nd, dtype=torch.float64, device="cuda")
        A.matvecT(jac, lam_th, g_ref)
        g_th = torch.zeros(nd, dtype=torch.float64, device="cuda")
        th_vjp = {"workload": f"J(u)^T lam, Taylor-Hood {nx}x{nx} cavity, {e} elements",
                  "check": "against J^T lam of the assembled FP64 Jacobian (CSR SpMV-T)"}
        for prec in ("fp64", "double_float", "fp32_quad"):
            tv = maxrank(timer.run(lambda: A.vjpTaylorHood(amap, coords, conn6, NU, state, lam_th,
                                                           g_th, precision=prec),
                                   args.steps, args.warmup))
            th_vjp[prec] = {"ms_per_grad": tv * 1e3, "grads_per_s": 1.0 / tv,
                            "elements_per_s": world * e / tv,
                            "rel_err_vs_fp64_jt_lam":
                                float((g_th - g_ref).abs().max() / g_ref.abs().max())}
        launches += 6 * args.steps
        A.assembleTaylorHood(amap, coords, conn6, NU, state, res, jac, precision="fp32_quad")
        err_j = float((jac.vals - j64).abs().max() / j64.abs().max())
        err_r = float((res - r64).abs().max() / r64.abs().max())
        A.assembleTaylorHood(amap, coords, conn6, NU, state, res, jac, precision="mixed")
        err_jm = float((jac.vals - j64).abs().max() / j64.abs().max())
        err_rm = float((res - r64).abs().max() / r64.abs().max())

        # e2e: state in from pinned host memory, residual out, inside the timing
        state_h = torch.from_numpy(t["state"]).pin_memory()
        res_h = torch.empty(nd, dtype=torch.float64).pin_memory()

        def e2e(prec):
            def fn():
                # one call: state upload, assembly, Dirichlet rows, residual download
                A.newtonSystemTaylorHoodHost(amap, bc, coords, conn6, NU, state_h, state, bvals,
                                             res, jac, res_h, 1.0, precision=prec)
            return fn
        t_e2e = maxrank(timer.run(e2e("fp64"), args.steps, args.warmup))
        t_e2e32 = maxrank(timer.run(e2e("fp32_quad"), args.steps, args.warmup))
        t_e2e_df = maxrank(timer.run(e2e("double_float"), args.steps, args.warmup))
        launches += 9 * args.steps
        # the plain FP64 step against the oracle at full size (what the
        # headline computes; bench parity, the tests hold the same gate)
        from oracle import pyoracle as orc
        om = orc.AssemblyMap(nd, nd, t["offs"], t["dofs"], t["offs"], t["dofs"])
        oth = orc.THQuad(t["coords"], t["conn6"])
        o_r, o_v = orc.assemble_th_threads(om, oth, NU, t["state"], host_cores())
        th_step("fp64")()
        torch.cuda.synchronize()
        ob = orc.BoundaryMap(t["bdofs"], om.row_ptr, om.col_ind)
        o_r = ob.replace_res(t["state"], t["bvals"], o_r)
        o_v = ob.replace_rows(o_v, 1.0)
        err_or = float(np.abs(res.cpu().numpy() - o_r).max() / np.abs(o_r).max())
        err_ov = float(np.abs(jac.vals.cpu().numpy() - o_v).max() / np.abs(o_v).max())
        th_step("double_float")()
        torch.cuda.synchronize()
        err_df_r = float(np.abs(res.cpu().numpy() - o_r).max() / np.abs(o_r).max())
        err_df_v = float(np.abs(jac.vals.cpu().numpy() - o_v).max() / np.abs(o_v).max())
        del om, oth, ob, o_r, o_v

        nnz = pat.nnz
        np2 = t["coords"].shape[0]
        b_th = 8 * nnz + 16 * nd + 60 * e + 24 * e + 16 * np2
        clk_sum = clk.summary()
        sm_mhz = clk_sum["sm_mhz"] or clk_sum["sm_max_mhz"] or 2070.0
        issue_peak = torch.cuda.get_device_properties(local).multi_processor_count * 128 \
            * sm_mhz * 1e6
        # FP64 instructions of the plain kernel per element, counted by ncu
        # on the 256x256 cavity (DFMA + DMUL + DADD thread instructions per
        # element), set against the measured FMA issue rate (fp64 = TFLOP/s
        # with FMA = 2).
        fp64 = fp64_peak_tflops(torch, L)
        i64 = FP64_INSTR_PER_ELEM * e  # FP64 instructions per launch of the plain kernel
        line.update({
            "metric": METRIC, "value": world * e / t_plain, "unit": "elements/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_plain * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)", "config": th_config() if nx == TH_NX else
            {"workload": f"ns_taylor_hood_p2p1_cavity_{nx}x{nx}"},
            "e2e": {"value": world * e / t_e2e, "unit": "elements/s",
                    "h2d_bytes_per_step": 8 * nd, "d2h_bytes_per_step": 8 * nd,
                    "ms_per_step": t_e2e * 1e3, "precision": "fp64",
                    "entry": "gbfem_newton_system_th_ns_host"},
            "rel_err_vs_oracle_full_size": {"jacobian": err_ov, "residual": err_or,
                                            "gate": 1e-12, "norm": "inf, relative",
                                            "after": "replaceRes + replaceRows"},
            "fp32_quad": {"value": world * e / t_fast, "unit": "elements/s",
                          "ms_per_step": t_fast * 1e3,
                          "speedup_vs_plain_fp64": t_plain / t_fast,
                          "e2e": {"value": world * e / t_e2e32, "ms_per_step": t_e2e32 * 1e3},
                          "rel_err_vs_fp64": {"jacobian": err_j, "residual": err_r,
                                              "gate": 1e-6, "norm": "inf, relative"},
                          "precision": "element quadrature fp32, accumulation/scatter/"
                                       "vectors fp64"},
            "fp64_double_float": {
                "value": world * e / t_df, "unit": "elements/s", "ms_per_step": t_df * 1e3,
                "speedup_vs_plain_fp64": t_plain / t_df,
                "e2e": {"value": world * e / t_e2e_df, "ms_per_step": t_e2e_df * 1e3},
                "rel_err_vs_oracle_full_size": {"jacobian": err_df_v, "residual": err_df_r,
                                                "gate": 1e-12},
                "kernel": "thElemKernelDd<false>", "launch_ms": t_kern_df * 1e3,
                "roofline": {"bound": "hbm", "achieved": b_th / t_kern_df / 1e9, "peak": hbm,
                             "unit": "GB/s", "frac": b_th / t_kern_df / 1e9 / hbm,
                             "traffic": traffic.get("th_double_float")},
                "issue": {"binding_resource": "instruction issue (all pipes), not HBM",
                          "thread_instructions_per_element": DF_INSTR_PER_ELEM,
                          "achieved_tinstr_per_s": DF_INSTR_PER_ELEM * e / t_kern_df,
                          "peak_tinstr_per_s": issue_peak,
                          "frac": DF_INSTR_PER_ELEM * e / t_kern_df / issue_peak,
                          "peak_source": "one warp instruction per SM sub-partition per clock "
                                         "(4 x 32 lanes per SM) at the median SM clock sampled "
                                         "in the timed region",
                          "count_source": "ncu inst_executed of the kernel x 32 / elements"},
                "precision": "FP64-accurate: element arithmetic in double-float (float "
                             "pairs, ~48 significant bits) on the FP32 pipe; accumulation, "
                             "scatter and vectors FP64"},
            "deterministic_fp32": {"value": world * e / t_det, "unit": "elements/s",
                                   "ms_per_step": t_det * 1e3,
                                   "bitwise_equal_over_runs": det_bitwise,
                                   "scheme": "element rows as records, CSR rows summed in "
                                             "element order, no atomics"},
            "mixed_newton": {"value": world * e / t_mixed, "unit": "elements/s",
                             "ms_per_step": t_mixed * 1e3,
                             "speedup_vs_plain_fp64": t_plain / t_mixed,
                             "precision": "Jacobian fp32 quadrature, residual to fp64 "
                                          "accuracy (double-float arithmetic on the FP32 pipe)",
                             "rel_err_vs_fp64": {"jacobian": err_jm, "residual": err_rm}},
            "roofline": {"bound": "hbm", "achieved": b_th / t_kern64 / 1e9, "peak": hbm,
                         "unit": "GB/s", "frac": b_th / t_kern64 / 1e9 / hbm,
                         "traffic": traffic.get("th_fp64"), "kernel": "thElemKernel64",
                         "launch_ms": t_kern64 * 1e3, "algorithmic_bytes": b_th,
                         "peak_source": f"MEASURED_PEAKS.json hbm_gbs ({peak_kind})",
                         "binding_resource": "FP64 issue (see fp64_issue)"},
            "fp64_issue": {"kernel": "thElemKernel64 (thread per element)",
                           "instructions_per_element": FP64_INSTR_PER_ELEM,
                           "achieved_ginstr_per_s": i64 / t_kern64 / 1e9,
                           "peak_ginstr_per_s": fp64 / 2 * 1e3,
                           "frac": i64 / t_kern64 / 1e12 / (fp64 / 2),
                           "peak_source": "FP64 FMA rate measured by gbfem_probe_fp64_fma",
                           "note": "FP64 instructions issued per second against the measured "
                                   "FMA issue rate (an instruction-issue fraction, not FLOP)"},
            "roofline_fp32_quad": {"bound": "hbm", "achieved": b_th / t_kern / 1e9, "peak": hbm,
                                   "unit": "GB/s", "frac": b_th / t_kern / 1e9 / hbm,
                                   "traffic": traffic.get("th_fp32"),
                                   "kernel": "thKernel<float,true>",
                                   "launch_ms": t_kern * 1e3, "algorithmic_bytes": b_th},
            "fp64_fma_peak_tflops_measured": fp64,
            "th_state_vjp": th_vjp,
            "clocks": clk_sum,
        })
        del amap, bc, jac, res, j64, r64

    # ---------------- VJP (config 4) ----------------
    if only in ("", "vjp"):
        p = p1_inputs(VJP_NX, seed_kappa=4)
        n, e = p["coords"].shape[0], p["conn"].shape[0]
        amap = A.makeAssemblyMap(n, n, d(p["offs"]), d(p["dofs"]), d(p["offs"]), d(p["dofs"]))
        coords, kappa = d(p["coords"]), d(p["kappa"])
        rng = np.random.default_rng(4)
        u, lam = d(rng.standard_normal(n)), d(rng.standard_normal(n))
        g_u = torch.zeros(n, dtype=torch.float64, device="cuda")
        g_m = torch.zeros(e, dtype=torch.float64, device="cuda")
        res_v = {}
        for prec in ("fp32_quad", "fp64"):
            tt = maxrank(timer.run(lambda: A.vjpP1Kappa(amap, coords, kappa, u, lam, g_u, g_m,
                                                         precision=prec), args.steps,
                                   args.warmup))
            res_v[prec] = (tt, g_u.clone(), g_m.clone())
        launches += 2 * args.steps
        t64, gu64, gm64 = res_v["fp64"]
        t32, gu32, gm32 = res_v["fp32_quad"]
        b_vjp = 28 * e + 40 * n
        # the tiled residual VJPs (g_u row by row, g_m by each element's owner
        # tile: no atomics, no zero fill), FP64-accurate
        amap.enableTiles(coords)
        vjp_tiled = {}
        for prec in ("double_float", "fp64"):
            tt = maxrank(timer.run(lambda: A.vjpP1Kappa(amap, coords, kappa, u, lam, g_u, g_m,
                                                         precision=prec, tiled=True),
                                   args.steps, args.warmup))
            vjp_tiled[prec] = {
                "ms_per_grad": tt * 1e3, "grads_per_s": 1.0 / tt,
                "roofline": {"bound": "hbm", "achieved": b_vjp / tt / 1e9, "peak": hbm,
                             "unit": "GB/s", "frac": b_vjp / tt / 1e9 / hbm},
                "rel_err_vs_fp64_vjp": {
                    "g_u": float((g_u - gu64).abs().max() / gu64.abs().max()),
                    "g_m": float((g_m - gm64).abs().max() / gm64.abs().max())}}
        launches += 2 * args.steps
        # Central differences of the FP64 residual (h = 1e-6) against the
        # FP32-quadrature VJP along 32 seeded unit directions in m and in u.
        from femx_gb300.autograd import p1_kappa_residual
        f_d = d(p["f"])
        bdofs = d(p["bdofs"])
        bcv = A.makeBoundaryMap(bdofs, amap.pattern())
        gz = torch.zeros(bdofs.numel(), dtype=torch.float64, device="cuda")
        m0 = torch.log(kappa)
        grads = {}
        for prec in ("mixed", "fp32_quad"):
            u_r, m_r = u.clone().requires_grad_(), m0.clone().requires_grad_()
            rr = p1_kappa_residual(u_r, m_r, amap, coords, f_d, bcv, gz, precision=prec)
            (rr * lam).sum().backward()
            grads[prec] = (u_r.grad, m_r.grad)
        # Central differences from the serial CPU oracle residual (fixed
        # summation order, so the two evaluations' rounding is correlated).
        from oracle import pyoracle as orc
        om = orc.AssemblyMap(n, n, p["offs"], p["dofs"], p["offs"], p["dofs"])
        oq = orc.P1Quad(p["coords"], p["conn"])
        ob = orc.BoundaryMap(p["bdofs"], om.row_ptr, om.col_ind)
        u_h, m_h, lam_h = u.cpu().numpy(), m0.cpu().numpy(), lam.cpu().numpy()
        g_h = np.zeros(len(p["bdofs"]))

        def R(uu, mm):
            r_, _ = orc.assemble_p1_kappa(om, oq, np.exp(mm), p["f"], uu)
            return ob.replace_res(uu, g_h, r_)

        hg = {k: (gu_.cpu().numpy(), gm_.cpu().numpy()) for k, (gu_, gm_) in grads.items()}
        # the oracle's own analytic gradient: its disagreement with the same
        # finite differences is the noise floor of the FD check itself
        lt = lam_h.copy()
        lt[p["bdofs"]] = 0.0
        ogu, ogm = orc.vjp_p1_kappa(om, oq, np.exp(m_h), u_h, lt)
        # the serial oracle VJP timed on one host core (bounded sample)
        kap_h = np.exp(m_h)
        n_v, t_v = 0, 0.0
        while (rank == 0 and world == 1 and not args.no_cpu_baseline
               and n_v < 20 and (n_v < 1 or t_v < 4.0)):
            t0 = time.perf_counter()
            orc.vjp_p1_kappa(om, oq, kap_h, u_h, lt)
            t_v += time.perf_counter() - t0
            n_v += 1
        ogu[p["bdofs"]] += lam_h[p["bdofs"]]
        hg["oracle"] = (ogu, ogm)
        direct = {"g_u": float(np.abs(hg["mixed"][0] - ogu).max() / np.abs(ogu).max()),
                  "g_m": float(np.abs(hg["mixed"][1] - ogm).max() / np.abs(ogm).max())}
        # Two FD schemes along the same 32 + 32 unit directions: plain central
        # differences at h = 1e-6 (the step the configuration names), whose
        # own rounding floor at this size is above 1e-6, and a resolved
        # scheme whose error is far below the gate: h = 1 in u (R is affine
        # in u, so the central difference is exact up to rounding) and
        # Richardson-extrapolated central differences (h = 1e-2, 5e-3) in m.
        # The oracle's exact gradient against the same differences gives
        # each scheme's noise floor.
        def fd_dir(which, dv, scheme):
            if which == "u":
                hh = 1e-6 if scheme == "h1e-6" else 1.0
                return float((R(u_h + hh * dv, m_h) - R(u_h - hh * dv, m_h)) @ lam_h) / (2 * hh)

            def central(hh):
                return float((R(u_h, m_h + hh * dv) - R(u_h, m_h - hh * dv)) @ lam_h) / (2 * hh)
            if scheme == "h1e-6":
                return central(1e-6)
            return (4.0 * central(5e-3) - central(1e-2)) / 3.0

        schemes = ("h1e-6", "resolved")
        fd_err = {sc: {k: 0.0 for k in hg} for sc in schemes}
        exact_err = {k: 0.0 for k in hg}
        for _ in range(32):
            for which in ("m", "u"):
                dv = rng.standard_normal(e if which == "m" else n)
                dv /= np.linalg.norm(dv)
                ex = float((ogm if which == "m" else ogu) @ dv)
                for sc in schemes:
                    fd = fd_dir(which, dv, sc)
                    for prec, (gu_, gm_) in hg.items():
                        an = float((gm_ if which == "m" else gu_) @ dv)
                        fd_err[sc][prec] = max(fd_err[sc][prec],
                                               abs(fd - an) / max(abs(fd), 1e-300))
                for prec, (gu_, gm_) in hg.items():
                    an = float((gm_ if which == "m" else gu_) @ dv)
                    exact_err[prec] = max(exact_err[prec], abs(an - ex) / max(abs(ex), 1e-300))
        line["vjp"] = {
            "workload": f"poisson_p1_{VJP_NX}x{VJP_NX}_vjp_state_and_control",
            "grads_per_s": world / t32, "grads_per_s_fp64": world / t64,
            "ms_per_grad": t32 * 1e3, "ms_per_grad_fp64": t64 * 1e3,
            "elements": e,
            "tiled": vjp_tiled,
            "rel_err_fp32_vs_fp64": {
                "g_u": float((gu32 - gu64).abs().max() / gu64.abs().max()),
                "g_m": float((gm32 - gm64).abs().max() / gm64.abs().max())},
            "fd_check": {
                "directions": "32 in m and 32 in u (unit, seeded)", "gate": 1e-6,
                "fd_of": "fp64 residual with Dirichlet rows (serial CPU oracle)",
                "resolved": {"scheme": "u: central h=1 (R affine in u); m: Richardson "
                                       "extrapolation of central h=1e-2 and 5e-3",
                             "fp64_gradient": fd_err["resolved"]["mixed"],
                             "fp32_quadrature_gradient": fd_err["resolved"]["fp32_quad"],
                             "oracle_exact_gradient_noise_floor": fd_err["resolved"]["oracle"]},
                "h=1e-6": {"fp64_gradient": fd_err["h1e-6"]["mixed"],
                           "fp32_quadrature_gradient": fd_err["h1e-6"]["fp32_quad"],
                           "oracle_exact_gradient_noise_floor": fd_err["h1e-6"]["oracle"]},
                "vs_oracle_exact_gradient": {"fp64_gradient": exact_err["mixed"],
                                             "fp32_quadrature_gradient": exact_err["fp32_quad"]},
                "gpu_fp64_gradient_vs_oracle_gradient": direct,
                "note": "max over directions of |d - d_ref| / |d_ref|; at h=1e-6 the "
                        "differences carry their own rounding (the oracle's exact "
                        "gradient shows that floor); the FP32-quadrature VJP forms the "
                        "element geometry in FP32 and the gradient reduction in FP64"},
            "roofline": {"bound": "hbm", "achieved": b_vjp / t32 / 1e9, "peak": hbm,
                         "unit": "GB/s", "frac": b_vjp / t32 / 1e9 / hbm,
                         "algorithmic_bytes": b_vjp},
        }
        if n_v:
            line["vjp"]["cpu_baseline"] = {
                "grads_per_s": n_v / t_v, "ms_per_grad": t_v / n_v * 1e3, "cores": 1,
                "kind": "port",
                "sample": f"{n_v} state + control VJPs of the same {VJP_NX}x{VJP_NX} "
                          f"system (serial oracle, FP64)"}
        del bcv
        del amap

    # ---------------- Poisson forward + SpMV (config 2) ----------------
    if only in ("", "poisson"):
        p = p1_inputs(POISSON_NX)
        n, e = p["coords"].shape[0], p["conn"].shape[0]
        amap = A.makeAssemblyMap(n, n, d(p["offs"]), d(p["dofs"]), d(p["offs"]), d(p["dofs"]))
        pat = amap.pattern()
        b_p1 = 20 * e + 32 * n + 8 * pat.nnz   # algorithmic bytes of one assembly
        bc = A.makeBoundaryMap(d(p["bdofs"]), pat)
        coords, kappa, f = d(p["coords"]), d(p["kappa"]), d(p["f"])
        u = torch.zeros(n, dtype=torch.float64, device="cuda")
        g = torch.zeros(len(p["bdofs"]), dtype=torch.float64, device="cuda")
        res = torch.zeros(n, dtype=torch.float64, device="cuda")
        rhs, xa, xb = torch.zeros_like(res), torch.zeros_like(res), torch.zeros_like(res)
        jac = A.CsrMatrix(pat)

        def asm():
            A.assembleP1Kappa(amap, coords, kappa, f, u, res, jac)

        def bcs():
            A.axpby(-1.0, res, 0.0, rhs)
            A.prepareForwardSolve(bc, jac, rhs, g)

        def spmvs():
            x, y = rhs, xa
            for _ in range(NSPMV):
                A.matvec(jac, x, y, alpha=SPMV_SCALE)
                x, y = y, (xb if y is xa else xa)

        def full():
            asm()
            bcs()
            spmvs()

        t_full = maxrank(timer.run(full, args.steps, args.warmup))
        amap.enableTiles(coords)

        def full_tiled():
            A.assembleP1Kappa(amap, coords, kappa, f, u, res, jac, precision="double_float",
                              tiled=True)
            bcs()
            spmvs()

        t_full_tiled = maxrank(timer.run(full_tiled, args.steps, args.warmup))
        t_asm = timer.run(asm, args.steps, args.warmup)
        # the FP32-quadrature assembly of the same system (FP64 accumulation)
        t_asm32 = timer.run(lambda: A.assembleP1Kappa(amap, coords, kappa, f, u, res, jac,
                                                      precision="fp32_quad"),
                            args.steps, args.warmup)
        # the FP64-accurate double-float assembly, and its distance to FP64
        t_asm_df = timer.run(lambda: A.assembleP1Kappa(amap, coords, kappa, f, u, res, jac,
                                                       precision="double_float"),
                             args.steps, args.warmup)
        A.assembleP1Kappa(amap, coords, kappa, f, u, res, jac, precision="double_float")
        v_df, r_df = jac.vals.clone(), res.clone()
        A.assembleP1Kappa(amap, coords, kappa, f, u, res, jac, precision="fp64")
        err_df = {"jacobian": float((v_df - jac.vals).abs().max() / jac.vals.abs().max()),
                  "residual": float((r_df - res).abs().max() / res.abs().max())}
        del v_df, r_df
        # the owner-computes tiled assembly (each CSR row written once, no
        # atomics, no zero fill) in double-float (FP64-accurate), FP64 and FP32
        ntiles = amap.numTiles()
        tiled = {}
        A.assembleP1Kappa(amap, coords, kappa, f, u, res, jac, precision="fp64")
        v64, r64 = jac.vals.clone(), res.clone()
        for prec in ("double_float", "fp64", "fp32_quad"):
            def fn(prec=prec):
                A.assembleP1Kappa(amap, coords, kappa, f, u, res, jac, precision=prec,
                                  tiled=True)
            t_t = timer.run(fn, args.steps, args.warmup)
            fn()
            v1, r1 = jac.vals.clone(), res.clone()
            fn()
            tiled[prec] = {
                "bound": "hbm", "achieved": b_p1 / t_t / 1e9, "peak": hbm, "unit": "GB/s",
                "frac": b_p1 / t_t / 1e9 / hbm, "launch_ms": t_t * 1e3,
                "elements_per_s": e / t_t, "nnz_per_s": pat.nnz / t_t,
                "rel_err_vs_fp64": {
                    "jacobian": float((v1 - v64).abs().max() / v64.abs().max()),
                    "residual": float((r1 - r64).abs().max() / r64.abs().max())},
                "bitwise_equal_over_runs": bool(torch.equal(v1, jac.vals)
                                                and torch.equal(r1, res))}
            del v1, r1
        # the reference's own CUDA assembly (femx's assembleKernel with the same
        # operator in femx's plug-in form), timed on the same GPU
        ref_bar = reference_gpu_bar(torch, timer, args, p, coords, kappa, f, u, amap, pat,
                                    v64, r64)
        del v64, r64
        asm()
        bcs()
        t_spmv = timer.run(spmvs, args.steps, args.warmup) / NSPMV
        # the library bar: cuSPARSE CSR SpMV, which femx's
        # MatrixHandler<CudaCsrBackend>::matvec calls (MatrixHandler.cu:285-398),
        # reached through torch's sparse CSR mv on the same matrix and vectors
        a_csr = torch.sparse_csr_tensor(pat.row_ptr, pat.col_ind, jac.vals, size=(n, n))

        def spmvs_lib():
            x = rhs
            for _ in range(NSPMV):
                x = torch.mv(a_csr, x)

        try:
            spmvs_lib()
            torch.cuda.synchronize()
            t_lib = timer.run(spmvs_lib, args.steps, args.warmup) / NSPMV
        except RuntimeError as exc:  # sparse CSR mv unavailable in this torch build
            t_lib, lib_err = None, str(exc).splitlines()[0]
        launches += (3 + NSPMV) * args.steps
        nnz = pat.nnz
        b_asm = 20 * e + 32 * n + 8 * nnz
        b_spmv = 12 * nnz + 20 * n
        fp64_p1 = fp64_peak_tflops(torch, L)
        line["poisson"] = {
            "workload": f"poisson_p1_kappa_{POISSON_NX}x{POISSON_NX}_assemble_bc_{NSPMV}spmv",
            "elements_per_s": world * e / t_full, "ms_per_step": t_full * 1e3,
            "step_tiled_double_float": {
                "ms_per_step": t_full_tiled * 1e3, "elements_per_s": world * e / t_full_tiled,
                "what": "the same step with the FP64-accurate tiled assembly"},
            "nnz_per_s_assembly": nnz / t_asm,
            "assembly": {"bound": "hbm", "achieved": b_asm / t_asm / 1e9, "peak": hbm,
                         "unit": "GB/s", "frac": b_asm / t_asm / 1e9 / hbm,
                         "launch_ms": t_asm * 1e3, "traffic": traffic.get("p1_assemble"),
                         "note": "plain FP64: FP64-pipe bound on GB300"},
            # the bound that applies: 45 FP64 instructions per element (edges 4,
            # determinant 3, reciprocal 4, scale 2, gradient sums 2, stiffness
            # 12, residual 9, load 9; counted from the kernel), each the issue
            # cost of one FMA: expressed as FLOP with FMA = 2
            "assembly_fp64_pipe": {"bound": "fp64",
                                   "achieved": 2 * 45 * e / t_asm / 1e12,
                                   "peak": fp64_p1, "unit": "TFLOP/s",
                                   "frac": 2 * 45 * e / t_asm / 1e12 / fp64_p1,
                                   "launch_ms": t_asm * 1e3,
                                   "peak_source": "measured by gbfem_probe_fp64_fma"},
            "assembly_fp32_quad": {"bound": "hbm", "achieved": b_asm / t_asm32 / 1e9,
                                   "peak": hbm, "unit": "GB/s",
                                   "frac": b_asm / t_asm32 / 1e9 / hbm,
                                   "launch_ms": t_asm32 * 1e3},
            "assembly_double_float": {"bound": "hbm", "achieved": b_asm / t_asm_df / 1e9,
                                      "peak": hbm, "unit": "GB/s",
                                      "frac": b_asm / t_asm_df / 1e9 / hbm,
                                      "launch_ms": t_asm_df * 1e3,
                                      "rel_err_vs_fp64": err_df,
                                      "precision": "FP64-accurate: element arithmetic in "
                                                   "double-float on the FP32 pipe"},
            "assembly_tiled": dict(tiled, tiles=ntiles,
                                   scheme="owner-computes tiles: each CSR row written once, "
                                          "no atomics, no zero fill",
                                   precision={"double_float": "FP64-accurate: double-float "
                                              "element arithmetic, integer-pipe conversions",
                                              "fp64": "IEEE FP64 element arithmetic",
                                              "fp32_quad": "FP32 element arithmetic"}),
            "generic_user_operator": generic_user_operator(POISSON_NX),
            "reference_gpu_assembly": dict(ref_bar, **({"speedup": {
                "plain_fp64": ref_bar["launch_ms"] / (t_asm * 1e3),
                "tiled_double_float": ref_bar["launch_ms"] / tiled["double_float"]["launch_ms"],
                "tiled_fp32": ref_bar["launch_ms"] / tiled["fp32_quad"]["launch_ms"]}}
                if "launch_ms" in ref_bar else {})),
            "spmv": {"bound": "hbm", "achieved": b_spmv / t_spmv / 1e9, "peak": hbm,
                     "unit": "GB/s", "frac": b_spmv / t_spmv / 1e9 / hbm,
                     "launch_ms": t_spmv * 1e3, "traffic": traffic.get("spmv"),
                     # the co-bound on GB300: one FP64 FMA per nonzero
                     "fp64_pipe": {"achieved": 2 * nnz / t_spmv / 1e12, "peak": fp64_p1,
                                   "unit": "TFLOP/s",
                                   "frac": 2 * nnz / t_spmv / 1e12 / fp64_p1}},
            "spmv_cusparse": ({"launch_ms": t_lib * 1e3,
                               "achieved": b_spmv / t_lib / 1e9, "unit": "GB/s",
                               "ours_speedup": t_lib / t_spmv,
                               "via": "torch.mv on a sparse CSR tensor (cuSPARSE SpMV)"}
                              if t_lib is not None else {"unavailable": lib_err}),
        }
        if rank == 0 and world == 1 and not args.no_cpu_baseline:
            line["poisson"].update(poisson_cpu(p, n, A, asm, bcs, rhs, jac, torch))
        del amap, bc, jac

    # ---------------- femx's GLS NS time operator (P1/P1, 256x256) ----------
    if only in ("", "navier"):
        from femx_gb300 import meshes
        c2, k2 = meshes.structured_tri(NS_NX)
        nn, e = c2.shape[0], k2.shape[0]
        offs, dofs, nd = meshes.navier_elem_dofs(k2, nn)
        rng = np.random.default_rng(6)
        hist_h = np.concatenate([meshes.stream_velocity(c2, seed=6).reshape(-1),
                                 rng.standard_normal(nn),
                                 meshes.stream_velocity(c2, seed=7).reshape(-1),
                                 rng.standard_normal(nn)])
        nxt_h = hist_h[:nd] + 1e-2 * rng.standard_normal(nd)
        adj_h = rng.standard_normal(nd)
        prm = (1.0, 1.0e-3, 1.0e-2, 2)  # rho, mu (Re 1000), dt, step (AB2 on)
        amap = A.makeAssemblyMap(nd, nd, d(offs), d(dofs), d(offs), d(dofs))
        coords, conn = d(c2), d(k2)
        hist, nxt, adj = d(hist_h), d(nxt_h), d(adj_h)
        res = torch.zeros(nd, dtype=torch.float64, device="cuda")
        jac = A.CsrMatrix(amap.pattern())
        g_hist = torch.zeros(2 * nd, dtype=torch.float64, device="cuda")

        def ns_asm():
            A.assembleNavier(amap, coords, conn, *prm, hist, nxt, res, jac)

        def ns_vjp():
            A.vjpNavierHist(amap, coords, conn, *prm, hist, nxt, adj, g_hist)

        t_asm = maxrank(timer.run(ns_asm, args.steps, args.warmup))
        t_vjp = maxrank(timer.run(ns_vjp, args.steps, args.warmup))
        launches += 2 * args.steps
        ns_asm()
        amap.check()
        entry = {
            "workload": f"femx_gls_navier_stokes_p1p1_{NS_NX}x{NS_NX}_cn_ab2_step",
            "elements": e, "dofs": nd, "nnz": amap.pattern().nnz,
            "operator": "femx NavierOperator (equal-order GLS, CN + AB2), FP64",
            "assemble_next": {"elements_per_s": world * e / t_asm, "ms": t_asm * 1e3},
            "history_vjp": {"elements_per_s": world * e / t_vjp, "ms": t_vjp * 1e3,
                            "note": "femx computes this with Enzyme; reverse mode by hand here"},
        }
        entry["reference_gpu_assembly"] = reference_gpu_ns_bar(
            torch, timer, args, c2, k2, amap, prm, hist, nxt, jac.vals, res, t_asm)
        if rank == 0 and world == 1 and not args.no_cpu_baseline:
            from oracle import pyoracle as orc
            om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
            q = orc.P1Quad(c2, k2, order=2)
            cores = host_cores()
            r_o, v_o = np.zeros(nd), np.zeros(om.nnz)
            n_s, tot = 0, 0.0
            while tot < 6.0 and n_s < 10:
                t0 = time.perf_counter()
                orc.assemble_navier_threads(om, q, *prm, hist_h, nxt_h, cores, res=r_o, vals=v_o)
                tot += time.perf_counter() - t0
                n_s += 1
            entry["cpu_baseline"] = {
                "elements_per_s": e * n_s / tot, "cores": cores, "kind": "port",
                "sample": f"{n_s} full assemblies (oracle restatement of femx's NavierOperator, "
                          f"bit-identical to the reference on the golden cases; atomic adds)"}
            entry["rel_err_vs_oracle_full_size"] = {
                "residual": float(np.abs(res.cpu().numpy() - r_o).max() / np.abs(r_o).max()),
                "jacobian": float(np.abs(jac.vals.cpu().numpy() - v_o).max() / np.abs(v_o).max())}
        line["navier"] = entry
        del amap, jac

    # ---------------- batched uneven instances (config 5) ----------------
    if only in ("", "batch"):
        from femx_gb300 import meshes
        from femx_gb300.batch import Batch, P1Instance, THInstance, autotune
        rng = np.random.default_rng(5)
        insts, cpu_sample = [], []
        n_p1 = n_th = 0
        for k in range(args.batch_instances):
            if rng.random() < 0.5:
                nx = int(rng.integers(32, 513))
                coords, conn = meshes.jittered_tri(nx, seed=1000 + k)
                nn, ne = coords.shape[0], conn.shape[0]
                offs, dofs = meshes.scalar_elem_dofs(conn)
                amap = A.makeAssemblyMap(nn, nn, d(offs), d(dofs), d(offs), d(dofs))
                kappa = np.exp(meshes.grf_centroids(coords, conn, seed=2000 + k, ell=0.05,
                                                    grid=256))
                u_k, f_k = rng.standard_normal(nn), meshes.fourier_source(coords, k)
                lam_k = rng.standard_normal(nn)
                insts.append(P1Instance(amap, d(coords), d(kappa), d(u_k), d(f_k), d(lam_k)))
                if sum(1 for c in cpu_sample if c[0] == "p1") < 4:
                    cpu_sample.append(("p1", ne, coords, conn, offs, dofs, kappa, u_k, f_k,
                                       lam_k))
                n_p1 += 1
            else:
                nx = int(rng.integers(32, 129))
                re = float(rng.uniform(100.0, 1000.0))
                c3, k3 = meshes.jittered_tri(nx, seed=3000 + k)
                cp2, conn6, nv = meshes.p2_mesh(c3, k3)
                offs, dofs, nd = meshes.th_elem_dofs(conn6, cp2.shape[0])
                amap = A.makeAssemblyMap(nd, nd, d(offs), d(dofs), d(offs), d(dofs))
                st_k, lam_k = meshes.cavity_state(cp2, nv, seed=k), rng.standard_normal(nd)
                insts.append(THInstance(amap, d(cp2), d(conn6), 1.0 / re, d(st_k), d(lam_k)))
                if sum(1 for c in cpu_sample if c[0] == "th") < 4:
                    cpu_sample.append(("th", conn6.shape[0], cp2, conn6, offs, dofs, nd,
                                       1.0 / re, st_k, lam_k))
                n_th += 1
        batch = Batch(insts, coloured=True)
        runs, tuned = {}, {}
        for prec in ("fp64", "mixed", "fp32_quad"):
            params, tune = autotune(batch, prec, reps=2, use_cache=False)
            gr = batch.graph(prec, **params)
            runs[prec] = maxrank(timer.run(gr.replay, args.steps, args.warmup))
            tuned[prec] = params
            if prec == "fp64":
                ref = [(x.res.clone(), x.vals.clone(), x.g_u.clone(),
                        None if getattr(x, "g_m", None) is None else x.g_m.clone())
                       for x in insts]
            else:
                err = {"jacobian": 0.0, "residual": 0.0, "vjp_state": 0.0, "vjp_control": 0.0}
                for x, (r64, v64, gu64, gm64) in zip(insts, ref):
                    def rel(a, b):
                        return float((a - b).abs().max() / b.abs().max())
                    err["residual"] = max(err["residual"], rel(x.res, r64))
                    err["jacobian"] = max(err["jacobian"], rel(x.vals, v64))
                    err["vjp_state"] = max(err["vjp_state"], rel(x.g_u, gu64))
                    if gm64 is not None:
                        err["vjp_control"] = max(err["vjp_control"], rel(x.g_m, gm64))
                tuned[prec + "_err"] = err
            del gr
            batch.check()
        t_b32, t_b64, t_bmx = runs["fp32_quad"], runs["fp64"], runs["mixed"]
        launches += 6 * args.steps
        # deterministic runs: the colouring scheme (colour rounds, plain adds)
        det_runs = {}
        for prec in ("fp64", "fp32_quad"):
            params, _ = autotune(batch, prec, reps=2, use_cache=False, deterministic=True)
            gr = batch.graph(prec, **params)
            det_runs[prec] = {"ms_per_step": maxrank(timer.run(gr.replay, args.steps,
                                                               args.warmup)) * 1e3,
                              "params": params}
            gr.replay()
            torch.cuda.synchronize()
            first = [x.vals.clone() for x in insts]
            gr.replay()
            torch.cuda.synchronize()
            det_runs[prec]["bitwise_equal_over_runs"] = all(
                torch.equal(a, x.vals) for a, x in zip(first, insts))
            del gr, first
            launches += args.steps * (2 + max(x.amap.numColours() for x in insts))
        # Baseline of the same kind: one CUDA graph of per-instance calls of
        # the standalone kernels (assemble + VJP per instance, each with its
        # own zero fill), replayed like the persistent launch's graph.
        per_inst, per_inst_err = {}, {}
        jacs = [A.CsrMatrix(x.amap.pattern(), x.vals) for x in insts]

        def per_instance(prec):
            for x, jm in zip(insts, jacs):
                if isinstance(x, P1Instance):
                    A.assembleP1Kappa(x.amap, x.coords, x.kappa, x.f, x.u, x.res, jm,
                                      precision=prec)
                    A.vjpP1Kappa(x.amap, x.coords, x.kappa, x.u, x.lam, x.g_u, x.g_m,
                                 precision=prec)
                else:
                    A.assembleTaylorHood(x.amap, x.coords, x.conn6, x.nu, x.state, x.res, jm,
                                         precision=prec)
                    A.vjpTaylorHood(x.amap, x.coords, x.conn6, x.nu, x.state, x.lam, x.g_u,
                                    precision=prec)
        for prec in ("fp64", "mixed", "fp32_quad"):
            per_instance(prec)
            torch.cuda.synchronize()
            g_pi = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g_pi):
                per_instance(prec)
            per_inst[prec] = maxrank(timer.run(g_pi.replay, args.steps, args.warmup))
            if prec == "fp64":
                # same results as the persistent FP64 launch (atomic order only)
                e_pi = 0.0
                for x, (r64, v64, gu64, gm64) in zip(insts, ref):
                    for a_, b_ in ((x.res, r64), (x.vals, v64), (x.g_u, gu64),
                                   (getattr(x, "g_m", None), gm64)):
                        if b_ is not None:
                            e_pi = max(e_pi, float((a_ - b_).abs().max() / b_.abs().max()))
                per_inst_err["fp64_vs_persistent_fp64"] = e_pi
            del g_pi
        # zero fill + element kernel for the assembly and for the VJP
        launches += 3 * args.steps * 4 * len(insts)
        line["batch"] = {
            "workload": f"{args.batch_instances} uneven instances (P1 Poisson "
                        "jittered/permuted nx in 32..512, "
                        "Taylor-Hood cavity nx in 32..128, Re in 100..1000), residual + "
                        "Jacobian + VJP, one persistent launch replayed from a CUDA graph",
            "instances": {"p1": n_p1, "taylor_hood": n_th}, "elements": batch.num_elems,
            "elements_per_s_fp32_quad": world * batch.num_elems / t_b32,
            "elements_per_s_mixed": world * batch.num_elems / t_bmx,
            "elements_per_s_fp64": world * batch.num_elems / t_b64,
            "ms_per_step": {"fp32_quad": t_b32 * 1e3, "mixed": t_bmx * 1e3,
                            "fp64": t_b64 * 1e3},
            "speedup_vs_plain_fp64": {"fp32_quad": t_b64 / t_b32, "mixed": t_b64 / t_bmx},
            "max_rel_err_vs_fp64": {"fp32_quad": tuned.pop("fp32_quad_err"),
                                    "mixed": tuned.pop("mixed_err")},
            "gate": 1e-6,
            "precision_modes": {"fp32_quad": "all element quadrature fp32, fp64 accumulation",
                                "mixed": "Jacobian fp32 quadrature; residual to fp64 accuracy "
                                         "(Taylor-Hood: double-float, P1: fp64) and P1 "
                                         "gradients fp64; Taylor-Hood J^T lam from the fp32 J"},
            "autotuned": tuned,
            "deterministic_colouring": det_runs,
            "per_instance_graph": {
                "what": "one CUDA graph of per-instance standalone calls (assemble with its "
                        "zero fill + VJP per instance) on the same instances and outputs",
                "ms_per_step": {k: v * 1e3 for k, v in per_inst.items()},
                "elements_per_s": {k: world * batch.num_elems / v for k, v in per_inst.items()},
                "persistent_speedup": {k: per_inst[k] / runs[k] for k in per_inst},
                "max_rel_err": per_inst_err},
        }
        if rank == 0 and world == 1 and not args.no_cpu_baseline:
            e_p1 = sum(x.kappa.numel() for x in insts if isinstance(x, P1Instance))
            line["batch"]["cpu_baseline"] = batch_cpu(cpu_sample, e_p1,
                                                      batch.num_elems - e_p1)
        del insts, batch

    line["gpu_launches"] = launches
    line["scaling_mode"] = "replicas" if world > 1 else "single"
    if rank == 0 and world == 1 and not args.no_cpu_baseline and only in ("", "th"):
        line["cpu_baseline"] = cpu_baseline()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def batch_cpu(sample, e_p1, e_th):
    """Serial oracle time of the batch's work (residual + Jacobian + VJP),
    from a sample of its own instances: per-element rates of each physics,
    applied to the batch's element counts."""
    from oracle import pyoracle as orc
    t = {"p1": 0.0, "th": 0.0}
    n = {"p1": 0, "th": 0}
    for rec in sample:
        if rec[0] == "p1":
            _, ne, coords, conn, offs, dofs, kappa, u, f, lam = rec
            nn = coords.shape[0]
            om = orc.AssemblyMap(nn, nn, offs, dofs, offs, dofs)
            oq = orc.P1Quad(coords, conn)
            t0 = time.perf_counter()
            orc.assemble_p1_kappa(om, oq, kappa, f, u)
            orc.vjp_p1_kappa(om, oq, kappa, u, lam)
        else:
            _, ne, cp2, conn6, offs, dofs, nd, nu, st, lam = rec
            om = orc.AssemblyMap(nd, nd, offs, dofs, offs, dofs)
            th = orc.THQuad(cp2, conn6)
            res, vals = np.zeros(nd), np.zeros(om.nnz)
            t0 = time.perf_counter()
            orc.assemble_th_threads(om, th, nu, st, 1, res, vals)
            orc.matvec_t(om.row_ptr, om.col_ind, vals, lam, nd)
        t[rec[0]] += time.perf_counter() - t0
        n[rec[0]] += ne
    total = (e_p1 * t["p1"] / max(n["p1"], 1)) + (e_th * t["th"] / max(n["th"], 1))
    return {"elements_per_s": (e_p1 + e_th) / total, "seconds_per_batch": total, "cores": 1,
            "kind": "port",
            "sample": f"serial oracle on {sum(1 for r in sample if r[0] == 'p1')} P1 "
                      f"({n['p1']} elements) and {sum(1 for r in sample if r[0] == 'th')} "
                      f"Taylor-Hood ({n['th']} elements) instances of the batch, residual + "
                      f"Jacobian + VJP (Taylor-Hood VJP as J^T lam), per-element rates "
                      f"applied to the batch's {e_p1} P1 and {e_th} Taylor-Hood elements"}


def generic_user_operator(nx):
    """The header-only user-operator path (include/gbfem/generic_assembly.cuh,
    femx's evalRow contract) for a P1 Laplacian written as a user functor,
    against the KappaPoissonP1 tag on the same structured nx x nx mesh: both
    timed inside one CUDA program (tests/cpp/generic_assembly_test.cu, compiled
    here with nvcc against libgbfem), zero fill included."""
    import subprocess
    import tempfile
    root = os.path.dirname(os.path.abspath(__file__))
    try:
        exe = os.path.join(tempfile.mkdtemp(), "generic_time")
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-O2",
                        "-std=c++17", "-I" + os.path.join(root, "include"),
                        os.path.join(root, "tests", "cpp", "generic_assembly_test.cu"),
                        "-L" + os.path.join(root, "femx_gb300"), "-lgbfem",
                        "-Xlinker", "-rpath," + os.path.join(root, "femx_gb300"), "-o", exe],
                       check=True, capture_output=True, text=True, timeout=600)
        out = subprocess.run([exe, "time", str(nx), "20"], check=True, capture_output=True,
                             text=True, timeout=600).stdout
        f = out.split("TIME", 1)[1].split()
        gen, tag, ne = float(f[1]), float(f[3]), int(f[5])
    except Exception as exc:  # no nvcc, or the program failed
        return {"unavailable": str(exc).splitlines()[0][:200]}
    return {"what": "user evalRow functor (P1 Laplacian) through generic_assembly.cuh vs the "
                    "KappaPoissonP1 tag, FP64, zero fill included",
            "mesh": f"structured {nx}x{nx}", "elements": ne,
            "generic_ms": gen, "tag_ms": tag, "generic_elements_per_s": ne / (gen * 1e-3),
            "tag_speedup": gen / tag}


def reference_gpu_bar(torch, timer, args, p, coords, kappa, f, u, amap, pat, v64, r64):
    """femx's own CUDA assembly (CudaAssembly.hpp:100-169, one block of 128
    threads per element, FP64 atomics, quadrature from ElementQuadratureData
    tables) for the kappa-weighted P1 operator, compiled from femx's sources
    into oracle/_ref/gpu_bar.cubin, on this GPU: its time per assembly (zero
    fill included, as femx's assemble does it) and its distance to the FP64
    product kernel."""
    from oracle import gpu_bar
    reason = gpu_bar.unavailable_reason()
    if reason is not None:
        return {"unavailable": reason}
    from oracle import pyoracle as orc
    conn = torch.from_numpy(np.ascontiguousarray(p["conn"], dtype=np.int32)).cuda()
    tables = orc.P1Quad(p["coords"], p["conn"]).tables()
    view = {k: v.data_ptr() for k, v in amap.view().items()}
    view.update(num_res=amap.numRes(), num_states=amap.numStates())
    bar = gpu_bar.RefP1Assembly(torch, coords, conn, kappa, f, tables, view)
    res = torch.zeros_like(r64)
    vals = torch.zeros_like(v64)
    stream = torch.cuda.current_stream().cuda_stream
    t = timer.run(lambda: bar.assemble(u, res, vals, stream), args.steps, args.warmup)
    bar.assemble(u, res, vals, stream)
    torch.cuda.synchronize()
    return {"what": "femx assembleKernel<KappaPoissonP1> (the reference's CUDA assembly), "
                    "with its zero fill, on this GPU",
            "kernel": bar.kernel[:120], "launch_ms": t * 1e3,
            "elements_per_s": amap.numElems() / t,
            "rel_err_vs_fp64_product": {
                "jacobian": float((vals - v64).abs().max() / v64.abs().max()),
                "residual": float((res - r64).abs().max() / r64.abs().max())}}


def reference_gpu_ns_bar(torch, timer, args, c2, k2, amap, prm, hist, nxt, v_ours, r_ours,
                         t_ours):
    """femx's own GPU time assembly of its NS model (assembleTimeKernel with
    femx's NavierOperator, CudaAssembly.hpp:171-236 and
    femx/model/ns/Components.hpp:400-577, compiled from femx's sources into
    oracle/_ref/gpu_bar.cubin), next-state block with its zero fill, on this
    GPU, against the product's gbfem_assemble_navier on the same data."""
    from oracle import gpu_bar
    reason = gpu_bar.unavailable_reason()
    if reason is not None:
        return {"unavailable": reason}
    from oracle import pyoracle as orc
    view = {k: v.data_ptr() for k, v in amap.view().items()}
    view.update(num_res=amap.numRes(), num_states=amap.numStates())
    tables = orc.P1Quad(c2, k2, order=2).tables()
    rho, mu, dt, step = prm
    bar = gpu_bar.RefNavierAssembly(torch, tables, view, c2.shape[0], rho, mu, dt)
    res, vals = torch.zeros_like(r_ours), torch.zeros_like(v_ours)
    stream = torch.cuda.current_stream().cuda_stream
    t = timer.run(lambda: bar.assemble(step, hist, nxt, res, vals, stream), args.steps,
                  args.warmup)
    bar.assemble(step, hist, nxt, res, vals, stream)
    torch.cuda.synchronize()
    return {"what": "femx assembleTimeKernel<NavierOperator> (the reference's CUDA NS "
                    "assembly), next-state block with its zero fill, on this GPU",
            "kernel": bar.kernel[:120], "ms": t * 1e3,
            "elements_per_s": amap.numElems() / t, "ours_speedup": t / t_ours,
            "rel_err_vs_product": {
                "jacobian": float((vals - v_ours).abs().max() / v_ours.abs().max()),
                "residual": float((res - r_ours).abs().max() / r_ours.abs().max())}}


def poisson_cpu(p, n, A, asm, bcs, rhs, jac, torch):
    """The same Poisson step on one host core with the oracle (femx's generic
    assembly has no OpenMP): assembly, prepareForwardSolve and the ten
    products, timed in place on preallocated arrays; plus the GPU results'
    errors against it at full size. Each GPU product is checked against the
    oracle's product of the same input vector: along the chain itself the
    rounding of every product is amplified by the next (interior rows of the
    stiffness sum to zero, so each product cancels)."""
    from oracle import pyoracle as orc
    om = orc.AssemblyMap(n, n, p["offs"], p["dofs"], p["offs"], p["dofs"])
    oq = orc.P1Quad(p["coords"], p["conn"])
    ob = orc.BoundaryMap(p["bdofs"], om.row_ptr, om.col_ind)
    lib = orc.lib()
    kap, f = np.ascontiguousarray(p["kappa"]), np.ascontiguousarray(p["f"])
    u0, g = np.zeros(n), np.zeros(len(p["bdofs"]))
    r_o, v_o, ya, yb = np.zeros(n), np.zeros(om.nnz), np.zeros(n), np.zeros(n)
    rp, ci = om.row_ptr, om.col_ind

    f_p = orc._ptr(f)

    def step():
        orc._check(lib.orc_assemble_p1_kappa(om.h, oq.h, oq.conn, kap, f_p, u0, r_o, v_o))
        np.negative(r_o, out=r_o)  # rhs = -res at u = 0
        orc._check(lib.orc_prepare_forward_solve(ob.h, rp, v_o, r_o, g))
        x, y = r_o, ya
        for _ in range(NSPMV):
            lib.orc_matvec(n, rp, ci, v_o, x, y, SPMV_SCALE, 0.0)
            x, y = y, (yb if y is ya else ya)
        return x

    step()
    n_s, tot = 0, 0.0
    while n_s < 5 and (n_s < 1 or tot < 8.0):
        t0 = time.perf_counter()
        step()
        tot += time.perf_counter() - t0
        n_s += 1
    e = p["conn"].shape[0]
    # the GPU step once more, then its outputs against the oracle's
    asm()
    bcs()
    rhs_g = rhs.cpu().numpy()
    vals_g = jac.vals.cpu().numpy()
    r_chk, v_chk = np.zeros(n), np.zeros(om.nnz)
    orc._check(lib.orc_assemble_p1_kappa(om.h, oq.h, oq.conn, kap, f_p, u0, r_chk, v_chk))
    np.negative(r_chk, out=r_chk)
    orc._check(lib.orc_prepare_forward_solve(ob.h, rp, v_chk, r_chk, g))

    def rel(a, b):
        return float(np.abs(a - b).max() / np.abs(b).max())

    # each product against the oracle's product of the same matrix and vector;
    # also scaled by (|A||x|)_i, the bound of a dot product's rounding
    x_g, spmv_err, spmv_abs = rhs.clone(), 0.0, 0.0
    y_ref, y_abs, a_abs = np.zeros(n), np.zeros(n), np.abs(vals_g)
    for _ in range(NSPMV):
        y_g = torch.empty_like(x_g)
        A.matvec(jac, x_g, y_g, alpha=SPMV_SCALE)
        x_h = x_g.cpu().numpy()
        lib.orc_matvec(n, rp, ci, vals_g, x_h, y_ref, SPMV_SCALE, 0.0)
        lib.orc_matvec(n, rp, ci, a_abs, np.abs(x_h), y_abs, SPMV_SCALE, 0.0)
        d_y = np.abs(y_g.cpu().numpy() - y_ref)
        spmv_err = max(spmv_err, float(d_y.max() / np.abs(y_ref).max()))
        spmv_abs = max(spmv_abs, float(d_y.max() / y_abs.max()))
        x_g = y_g
    torch.cuda.synchronize()

    return {
        "cpu_baseline": {"elements_per_s": e * n_s / tot, "ms_per_step": tot / n_s * 1e3,
                         "cores": 1, "kind": "port",
                         "sample": f"{n_s} full steps (assembly, prepareForwardSolve, "
                                   f"{NSPMV} SpMV) of the same 1024x1024 system, serial "
                                   f"oracle in place"},
        "rel_err_vs_oracle_full_size": {"csr_vals_after_bc": rel(vals_g, v_chk),
                                        "rhs_after_lifting": rel(rhs_g, r_chk),
                                        "spmv_each_product_max": spmv_err,
                                        "spmv_each_product_max_vs_abs_products": spmv_abs},
    }


def cpu_baseline():
    """Oracle port on every host core: bounded sample of the headline workload."""
    from oracle import pyoracle as orc
    t = th_inputs(TH_NX)
    nd = t["nd"]
    om = orc.AssemblyMap(nd, nd, t["offs"], t["dofs"], t["offs"], t["dofs"])
    th = orc.THQuad(t["coords"], t["conn6"])
    res, vals = np.zeros(nd), np.zeros(om.nnz)
    e = t["conn6"].shape[0]
    cores = host_cores()
    steps, total = 0, 0.0
    while total < 8.0 and steps < 20:
        t0 = time.perf_counter()
        orc.assemble_th_threads(om, th, NU, t["state"], cores, res, vals)
        total += time.perf_counter() - t0
        steps += 1
    return {"value": e * steps / total, "unit": "elements/s", "cores": cores, "kind": "port",
            "sample": f"{steps} full assemblies of the 256x256 Taylor-Hood mesh (oracle, "
                      f"{cores} threads, atomic adds)"}


if __name__ == "__main__":
    main()
