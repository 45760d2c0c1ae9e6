"""Benchmark: EbE-PCG solve time to 1e-8 relative displacement error on the
1.39M-DOF jittered tet cantilever, FP32 + FP64 iterative refinement vs plain
FP64 on the same GPU, plus the EbE matvec's HBM roofline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Workload (one step = one full static solve, inputs resident in HBM): box
1x1x4, 48x48x192 hexes x 6 Kuhn tets (2,654,208 tets, 463,393 nodes,
1,390,179 DOF), interior nodes jittered +-0.2h (seed 0), E=2e7, nu=0.25, z=0
clamped, traction 1e3 in -y on z=4, textbook (consistent) traction loads.
The target error is measured against an FP64 solution converged to relative
residual 1e-13 before timing; each method's stopping tolerance is calibrated (untimed) to the
loosest value that reaches the target. L2 is flushed (512 MB write) before every step.
The path does not shard (one mesh, one GPU): with N > 1 every rank solves its
own replica and `value` is the max-over-ranks time of a replica's solve.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "EbE-PCG solve time to 1e-8 rel err, FP32+refine vs FP64; matvec HBM GB/s"
WORKLOAD = ("3D linear-tet cantilever 1x1x4, 48x48x192 hexes x 6 tets (2,654,208 tets, 463,393 nodes, "
            "1,390,179 DOF), jitter 0.2h seed 0, E=2e7 nu=0.25, z=0 clamped, traction 1e3 -y on z=4")
TARGET_ERR = 1e-8


def _peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([v.strip() for v in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if len(s) > 5 + i and s[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def _dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_baseline(problem, k_iters: int, iterations: int):
    """The oracle's FP32 element-local restatement of the reference's PCG
    (single thread, as the reference), timed on a bounded sample: its setup and
    k_iters PCG iterations at full size; the solve time is extrapolated with
    the iteration count the reference's own stopping rule needs."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle  # the checker / CPU baseline only
    setup_s, iter_s = oracle.ebe_time(problem, k_iters)
    total_ms = (setup_s + iterations * iter_s) * 1e3
    return {"value": round(total_ms, 1), "unit": "ms", "cores": 1, "kind": "port",
            "sample": (f"oracle FP32 element-local restatement of gpuPCG_EbE_vec (sort-based assembly), "
                       f"setup + {k_iters} PCG iterations on the full mesh ({setup_s:.2f} s + {iter_s:.3f} s/it), "
                       f"extrapolated to {iterations} iterations (reference stopping rule gamma < 1e-8 gamma0, "
                       f"count taken from the GPU FP32 run of the same rule)"),
            "setup_s": round(setup_s, 3), "iter_s": round(iter_s, 4), "extrapolated": True}


def run_reference(args):
    world, rank, _ = _dist_env()
    if rank != 0:
        return 0
    from cudafemproject_gb300 import meshgen
    p = meshgen.cantilever_1p39m()
    p_cfg = {"workload": WORKLOAD, "precision": "fp32 (reference algorithm)", "target": "gamma < 1e-8 gamma0"}
    # iteration count of the reference's rule at this size (measured on the GPU FP32 path when available)
    iters = int(os.environ.get("CFEM_REF_ITERS", "0")) or 2600
    k = 3
    for _ in range(args.warmup):
        pass  # the CPU sample has no warm-up state worth keeping
    vals = []
    t0 = time.time()
    for _ in range(args.steps):
        cb = cpu_baseline(p, k, iters)
        vals.append(cb["value"])
    v = float(np.max(vals))
    cb["value"] = v
    line = {"metric": METRIC, "value": v, "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded mesh generator)", "config": p_cfg,
            "impl": "reference", "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": round(time.time() - t0, 1)}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--small", action="store_true", help="a 24x24x96 box (profiling runs)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)

    import torch
    world, rank, local = _dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from cudafemproject_gb300 import capi, meshgen
    from cudafemproject_gb300.solver import FemContext
    import ctypes as C

    if args.small:
        p = meshgen.box_3d(24, 24, 96, jitter=0.2, seed=0, traction=(0.0, -1e3, 0.0))
        workload = WORKLOAD.replace("48x48x192", "24x24x96").replace("(2,654,208 tets, 463,393 nodes, 1,390,179 DOF)",
                                                                    "(331,776 tets)")
    else:
        p = meshgen.cantilever_1p39m()
        workload = WORKLOAD
    t0 = time.time()
    ctx = FemContext(p, semantics="consistent")
    setup_ms = (time.time() - t0) * 1e3
    L = capi.lib()
    nd = p.n_dof
    f_host = ctx.rhs()
    # FP64 reference solution (untimed): plain FP64 PCG to rel. residual 1e-15
    x_ref, inf_ref = ctx.pcg(f_host, "fp64", tol=1e-13, stop_rule="residual", max_iter=30000,
                             allow_not_converged=True)
    xr = np.asarray(x_ref)
    nref = np.linalg.norm(xr)

    def err(u):
        return float(np.linalg.norm(np.asarray(u).ravel() - xr) / nref)

    # resident inputs for the device-side timing
    f_dev = torch.tensor(f_host, device="cuda")
    u_dev = torch.zeros(nd, dtype=torch.float64, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def solve(kw, f=f_dev, out=u_dev):
        return ctx.pcg(f, out=out, allow_not_converged=True, **kw)

    # Calibration (untimed): for each method the loosest stopping tolerance
    # whose answer is within TARGET_ERR of the FP64 reference solution.
    plain64 = None
    for tol in (1e-7, 1e-8, 1e-9, 1e-10, 1e-11, 1e-12):
        kw = dict(precision="fp64", tol=tol, stop_rule="residual", max_iter=30000)
        _, i64 = solve(kw)
        e64 = err(u_dev.cpu().numpy())
        if e64 <= TARGET_ERR:
            plain64 = kw
            break
    refine, best = None, None
    for inner in (1e-3, 1e-4):
        for outer in (1e-6, 1e-7, 1e-8, 1e-9, 1e-10):
            kw = dict(precision="fp32_refine", tol=inner, stop_rule="residual", outer_tol=outer, max_outer=30,
                      max_iter=30000)
            _, i32 = solve(kw)
            e32 = err(u_dev.cpu().numpy())
            if e32 <= TARGET_ERR:
                if best is None or i32["solve_ms"] < best:
                    refine, best = kw, i32["solve_ms"]
                break
    if refine is None or plain64 is None:
        raise SystemExit(f"calibration failed to reach {TARGET_ERR}: refine={refine} fp64={plain64}")
    for _ in range(args.warmup):
        solve(refine)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    times, launches, infos = [], [], []
    # NVTX range "timed" marks the timed solves (lets a profiler select them)
    torch.cuda.nvtx.range_push("timed")
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            if world > 1:
                torch.distributed.barrier()
            _, inf = solve(refine)
            times.append(inf["solve_ms"])
            infos.append(inf)
        torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    clocks = clk.summary()
    ms = float(np.mean(times))
    err_timed = err(u_dev.cpu().numpy())
    if world > 1:
        t = torch.tensor([ms], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    # plain FP64 timed the same way (fewer steps: it is the slow arm)
    t64 = []
    for _ in range(max(1, min(args.steps, 3))):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        _, i64 = solve(plain64)
        t64.append(i64["solve_ms"])
    ms64 = float(np.mean(t64))
    e64_timed = err(u_dev.cpu().numpy())
    # e2e through the C-ABI with host buffers (h2d of f, d2h of u inside the timed region)
    u_host = np.zeros(nd)
    e2e = []
    for _ in range(max(1, min(args.steps, 3))):
        flush.fill_(1.0)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        ctx.pcg(f_host, out=u_host, **refine)
        e2e.append((time.perf_counter() - t1) * 1e3)
    e2e_ms = float(np.mean(e2e))
    # matvec roofline (FP32 PCG-form kernel, back-to-back launches, CUDA events on its stream)
    hbm, peak_kind = _peaks()
    msl, byt = C.c_double(0), C.c_double(0)
    capi.check(L.cfem_profile_matvec(ctx._h, capi.FP32, 200, C.byref(msl), C.byref(byt)), "profile")
    achieved = byt.value / (msl.value * 1e-3) / 1e9
    msl64, byt64 = C.c_double(0), C.c_double(0)
    capi.check(L.cfem_profile_matvec(ctx._h, capi.FP64, 50, C.byref(msl64), C.byref(byt64)), "profile64")
    traffic = None  # DRAM bytes per launch of the same kernel on this workload, from a committed ncu summary
    tfile = os.path.join(REPO, "profiles", "matvec_fp32_traffic.txt")
    if os.path.exists(tfile) and not args.small:
        for ln in open(tfile):
            if ln.startswith("dram_bytes_per_launch"):
                traffic = float(ln.split("=")[1])
    its = infos[-1]["iterations"]
    kernel_name = ("k_matvec_fan_tma<float,MV_PCG>" if ctx.counts()["matvec_form"] == capi.FORM_GRADIENT_FAN
                   else "k_matvec<float,3,MV_PCG>")
    line = {
        "metric": METRIC, "value": round(ms, 3), "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded mesh generator, see config)",
        "config": {"workload": workload, "precision": (f"FP32 inner PCG (rel. residual {refine['tol']:g}) + FP64 "
                   f"refinement (true rel. residual {refine['outer_tol']:g})"),
                   "fp64_stop": f"recursive rel. residual {plain64['tol']:g}",
                   "target_rel_err": TARGET_ERR, "rel_err_fp32_refine": err_timed,
                   "rel_err_fp64": e64_timed, "l2": "flushed before every step (512 MB write)",
                   "parallelism": "replicas" if world > 1 else "single GPU", "semantics": "consistent"},
        "fp64_ms": round(ms64, 3), "speedup_vs_fp64": round(ms64 / ms, 3),
        "pcg_iterations": its, "outer_iterations": infos[-1]["outer_iterations"],
        "fp64_iterations": i64["iterations"],
        "dof_iterations_per_s": round(nd * its / (ms * 1e-3), 1),
        "setup_ms": round(setup_ms, 1),
        "gpu_launches": int(infos[-1]["kernel_launches"]),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm, "unit": "GB/s",
                     "frac": round(achieved / hbm, 4), "traffic": traffic,
                     "kernel": kernel_name, "ms_per_launch": round(msl.value, 5),
                     "bytes_per_launch": byt.value, "peak_kind": peak_kind},
        "matvec_fp64": {"ms_per_launch": round(msl64.value, 5), "bytes_per_launch": byt64.value,
                        "achieved_gbs": round(byt64.value / (msl64.value * 1e-3) / 1e9, 1)},
        "clocks": clocks,
        "e2e": {"value": round(e2e_ms, 3), "unit": "ms", "h2d_bytes_per_step": nd * 8, "d2h_bytes_per_step": nd * 8},
    }
    if rank == 0 and world == 1 and not args.no_cpu:
        # reference rule iteration count on the GPU (FP32, gamma < 1e-8 gamma0) for the extrapolation
        _, ir = ctx.pcg(f_dev, out=u_dev, precision="fp32", tol=1e-8, stop_rule="reference",
                        allow_not_converged=True)
        line["cpu_baseline"] = cpu_baseline(p, 2, ir["iterations"])
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
