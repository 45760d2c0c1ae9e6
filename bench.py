"""Benchmark: EbE-PCG solve time to 1e-8 relative displacement error on the
1.39M-DOF jittered tet cantilever, FP32 + FP64 iterative refinement vs plain
FP64 on the same GPU, plus the EbE matvec's HBM roofline.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Workload (one step = one full static solve, inputs resident in HBM): box
1x1x4, 48x48x192 hexes x 6 Kuhn tets (2,654,208 tets, 463,393 nodes,
1,390,179 DOF), interior nodes jittered +-0.2h (seed 0), E=2e7, nu=0.25, z=0
clamped, traction 1e3 in -y on z=4, textbook (consistent) traction loads.
The target error is measured against the FP64 oracle's solution of the same
mesh and loads (oracle/fem_oracle.c on all host cores, relative residual
1e-12, computed before any GPU work); each method's stopping tolerance is
calibrated (untimed) to the loosest value that reaches the target. L2 is
flushed (512 MB write) before every step. The same line carries the FP64
oracle's own solve time (multi-threaded CPU figure), the FP32 port of the
reference's PCG timed on one core (CPU baseline) and a 64-case multi-RHS leg
on a 24x24x96 box. The path does not shard (one mesh, one GPU): with N > 1
every rank solves its own replica (errors then against the GPU FP64 solution)
and `value` is the max-over-ranks time of a replica's solve.
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
WORKLOAD_SMALL = ("3D linear-tet box 1x1x4, 24x24x96 hexes x 6 tets (331,776 tets, 181,875 DOF), jitter 0.2h seed 0, "
                  "E=2e7 nu=0.25, z=0 clamped, traction 1e3 -y on z=4")
TARGET_ERR = 1e-8
K_REF = 5  # PCG iterations per CPU sample
DATA = "synthetic (seeded mesh generator, see config)"
# identical on both arms of the benchmark
CONFIG = {"workload": WORKLOAD,
          "loads": ("uniform traction on the unjittered face z=4; the reference's own face-load formula gives loads "
                    "proportional to the textbook ones used here, so both solve the same system up to scale"),
          "l2": "flushed before every GPU step (512 MB write)",
          "parallelism": "single GPU (the path does not shard; --gpus N runs N replicas)"}


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


def _host_cores() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def _oracle():
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle  # the oracle: accuracy reference and CPU baseline only
    return oracle


def cpu_baseline(problem, k_iters: int, iterations: int, source: str):
    """The oracle's FP32 element-local restatement of the reference's PCG
    (femfunc.cpp:25-128 with cpu_fem_utils.cpp's sort-based assembly; single
    thread, as the reference), timed on a bounded sample: its setup and
    k_iters PCG iterations at full size. The solve time is extrapolated to
    the iteration count the reference's stopping rule needs (``source`` says
    where that count was measured)."""
    oracle = _oracle()
    t = oracle.EbeTimer(problem)
    t.iters(1)  # first touch of the work vectors
    iter_s = t.iters(k_iters) / k_iters
    t.close()
    total_ms = (t.init_s + iterations * iter_s) * 1e3
    return {"value": round(total_ms, 1), "unit": "ms", "cores": 1, "host_cores": _host_cores(), "kind": "port",
            "sample": (f"oracle FP32 element-local restatement of gpuPCG_EbE_vec (sort-based assembly, 1 thread): "
                       f"{k_iters} PCG iterations timed on the full mesh ({iter_s:.3f} s/it), extrapolated to "
                       f"{iterations} iterations (reference stopping rule gamma < 1e-8 gamma0; count {source}); "
                       f"setup {t.setup_s:.2f} s reported apart, not in the value"),
            "setup_s": round(t.setup_s, 3), "pcg_init_s": round(t.init_s, 4), "iter_s": round(iter_s, 4),
            "iterations": int(iterations), "extrapolated": True}


def oracle_solution(p, baseline_tol: float = 1e-7, pin_tol: float = 1e-12):
    """FP64 oracle on all host cores (oracle/fem_oracle.c: the reference's
    element matrices in FP64, assembled per node pair, Jacobi PCG of
    femfunc.cpp:25-128 in global form): a cold solve to relative residual
    ``baseline_tol`` (timed: the multi-threaded CPU figure), continued from
    that iterate to ``pin_tol`` (the solution every GPU answer is measured
    against). Runs before any GPU work."""
    oracle = _oracle()
    t0 = time.perf_counter()
    o = oracle.Oracle(p, consistent=True).assemble()
    t_setup = time.perf_counter() - t0
    f = o.rhs()
    t1 = time.perf_counter()
    x_b, it_b = o.pcg(f, tol=baseline_tol, rule=1)
    t_solve = time.perf_counter() - t1
    x, it_pin = o.pcg_warm(f, x_b, tol=pin_tol, rule=1)
    nx = np.linalg.norm(x)
    err_b = float(np.linalg.norm(x_b - x) / nx)
    thr = oracle.num_threads()
    fig = {"value": round(t_solve * 1e3, 1), "unit": "ms", "cores": thr, "host_cores": _host_cores(), "kind": "port",
           "sample": (f"FP64 oracle (reference element matrices in FP64, assembled per node pair, Jacobi PCG, "
                      f"OpenMP {thr} threads): full cold solve of this mesh to relative residual {baseline_tol:g} "
                      f"({it_b} iterations), rel. error {err_b:.2e} against the pinned solution; not the reference"),
           "setup_s": round(t_setup, 2), "iterations": it_b, "rel_err": err_b, "extrapolated": False}
    pin = {"tol": pin_tol, "iterations": it_b + it_pin}
    del o
    return x, f, fig, pin


def reference_rule_iterations(p):
    """Iterations the reference's stopping rule (gamma < 1e-8 gamma0,
    femfunc.cpp:92) takes on this mesh, counted by the FP64 oracle on all host
    cores (the FP32 reference itself would take hours to count them)."""
    oracle = _oracle()
    o = oracle.Oracle(p, consistent=True).assemble()
    t0 = time.perf_counter()
    _, it = o.pcg(o.rhs(), tol=1e-8, rule=0)
    return it, time.perf_counter() - t0


def run_reference(args):
    """The reference arm: the reference's CPU algorithm (the oracle's FP32
    element-local port, pinned bit-exact to the reference's own CPU build),
    one thread as the reference. Each step times one sample of K_REF PCG
    iterations on the full mesh; the value is the extrapolated solve time."""
    world, rank, _ = _dist_env()
    if rank != 0:
        return 0
    from cudafemproject_gb300 import meshgen
    p = meshgen.cantilever_1p39m()
    iters, t_count = reference_rule_iterations(p)
    oracle = _oracle()
    timer = oracle.EbeTimer(p)
    k = K_REF
    for _ in range(args.warmup):
        timer.iters(1)
    samples = []
    t0 = time.time()
    for _ in range(args.steps):
        samples.append(timer.iters(k))
    wall = time.time() - t0
    iter_s = float(np.median(samples)) / k
    value = round((timer.init_s + iters * iter_s) * 1e3, 1)
    cb = {"value": value, "unit": "ms", "cores": 1, "host_cores": _host_cores(), "kind": "port",
          "sample": (f"oracle FP32 element-local restatement of gpuPCG_EbE_vec (sort-based assembly, 1 thread, as "
                     f"the reference): {args.steps} samples of {k} PCG iterations on the full mesh (median "
                     f"{iter_s:.3f} s/it) extrapolated to {iters} iterations, the reference stopping rule's count "
                     f"measured by the FP64 oracle on this mesh ({t_count:.1f} s on all host cores); setup "
                     f"{timer.setup_s:.2f} s not in the value"),
          "setup_s": round(timer.setup_s, 3), "pcg_init_s": round(timer.init_s, 4), "iter_s": round(iter_s, 4),
          "iterations": int(iters), "extrapolated": True}
    timer.close()
    ms_step = float(np.mean(samples)) * 1e3
    line = {"metric": METRIC, "value": value, "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 1), "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": DATA, "config": CONFIG,
            "impl": "reference", "precision": "FP32 throughout, stopping rule gamma < 1e-8 gamma0 (reference)",
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": round(wall, 1)}
    print(json.dumps(line), flush=True)
    return 0


def _line(metric, value, unit, higher, config, extra):
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": 1, "higher_is_better": higher,
            "data": "synthetic (seeded mesh generator, see config)", "config": config}
    line.update(extra)
    print(json.dumps(line), flush=True)


def run_other_workload(args):
    """Measurements of the other configurations (not the driver's headline)."""
    import torch
    torch.cuda.set_device(0)
    from cudafemproject_gb300 import meshgen
    from cudafemproject_gb300.solver import BatchContext, FemContext
    if args.workload == "multi_rhs":
        # 24x24x96 tet box; each case a traction on z = max, direction uniform on the
        # sphere, magnitude log-uniform in [1e2, 1e4] (seed 1: k directions, then k magnitudes)
        nx, ny, nz = 24, 24, 96
        E3 = np.stack([FemContext(meshgen.box_3d(nx, ny, nz, traction=t), semantics="consistent").rhs()
                       for t in ((1.0, 0, 0), (0, 1.0, 0), (0, 0, 1.0))])
        ctx = FemContext(meshgen.box_3d(nx, ny, nz), semantics="consistent")
        kw = dict(precision="fp32_refine", tol=1e-4, stop_rule="residual", outer_tol=1e-8, max_iter=20000)
        rng = np.random.default_rng(1)
        for k in (64, 256):
            d = rng.standard_normal((k, 3))
            d /= np.linalg.norm(d, axis=1, keepdims=True)
            F = (d * (10.0 ** rng.uniform(2, 4, size=k))[:, None]) @ E3
            ctx.pcg_multi(F, **kw)
            U, infos = ctx.pcg_multi(F, **kw)
            ms_multi = infos[0]["solve_ms"]
            single = [ctx.pcg(F[i], **kw)[1]["solve_ms"] for i in range(4)]
            ms_single = float(np.mean(single[1:]))
            err = max(float(np.linalg.norm(U[i] - ctx.pcg(F[i], "fp64", tol=1e-12, stop_rule="residual")[0].ravel())
                            / np.linalg.norm(U[i])) for i in range(2))
            _line("multi-RHS solve time per load case to 1e-8 rel err", round(ms_multi / k, 3), "ms", False,
                  {"workload": f"24x24x96 tet box (331,776 tets, 181,875 DOF), {k} traction load cases",
                   "precision": "FP32 inner PCG + FP64 refinement"},
                  {"batched_ms_total": round(ms_multi, 1), "single_rhs_ms": round(ms_single, 3),
                   "per_rhs_speedup": round(ms_single / (ms_multi / k), 2), "rel_err_vs_fp64": err})
    elif args.workload == "batch":
        probs = meshgen.batch_boxes(64, seed=2)
        kw = dict(precision="fp32_refine", tol=1e-4, outer_tol=1e-8, max_iter=20000)
        b = BatchContext(probs)
        b.static_solve(**kw)
        us, infos = b.static_solve(**kw)
        ms_b = infos[0]["solve_ms"]
        b.close()
        seq, errs = 0.0, []
        for i, p in enumerate(probs):
            ctx = FemContext(p, semantics="consistent")
            ctx.static_solve(stop_rule="residual", **kw)
            u1, inf = ctx.static_solve(stop_rule="residual", **kw)
            seq += inf["solve_ms"]
            if i < 4:
                ref, _ = ctx.static_solve("fp64", tol=1e-13, stop_rule="residual", max_iter=40000,
                                          allow_not_converged=True)
                errs.append(float(np.linalg.norm(us[i] - ref) / np.linalg.norm(ref)))
            ctx.close()
        _line("batched independent meshes: solve time of all instances to 1e-8 rel err", round(ms_b, 1), "ms", False,
              {"workload": f"64 tet boxes n x n x 4n, n uniform in 8..40 (seed 2), E log-uniform [1e6, 1e8], "
                           f"nu uniform [0.2, 0.4]: {sum(p.n_elems for p in probs)} tets, "
                           f"{sum(p.n_dof for p in probs)} DOF", "precision": "FP32 inner PCG + FP64 refinement"},
              {"sequential_single_mesh_ms": round(seq, 1), "speedup_vs_sequential": round(seq / ms_b, 3),
               "max_iterations": max(i["iterations"] for i in infos), "rel_err_vs_fp64_first4": max(errs)})
    elif args.workload == "adjoint":
        run_adjoint_workload()
    elif args.workload == "dynamics":
        run_dynamics_workload()
    return 0


def run_adjoint_workload():
    """Tet cantilever 32x32x128 x 6 (786,432 tets), E_e = 2e7 exp(0.5 z_e) (seed 3),
    loss = f.u + 1/2 sum over 500 surface sensors |u_s - u_obs|^2, u_obs from a
    second field (seed 4). Gradient by the adjoint; checked by central finite
    differences along a random direction and on the 20 elements of largest
    sensitivity (relative step 1e-4)."""
    from cudafemproject_gb300 import meshgen
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(32, 32, 128, traction=(0.0, -1e3, 0.0))
    rng = np.random.default_rng(3)
    young = 2e7 * np.exp(0.5 * rng.standard_normal(p.n_elems))
    surf = np.nonzero((p.nodes[:, 0] <= 1e-9) | (p.nodes[:, 0] >= 1 - 1e-9) | (p.nodes[:, 1] <= 1e-9) |
                      (p.nodes[:, 1] >= 1 - 1e-9) | (p.nodes[:, 2] >= 4 - 1e-9))[0]
    sensors = rng.choice(surf, size=500, replace=False)
    young_obs = 2e7 * np.exp(0.5 * np.random.default_rng(4).standard_normal(p.n_elems))
    kw = dict(precision="fp32_refine", tol=1e-4, stop_rule="residual", outer_tol=1e-13, max_iter=40000)
    p.elem_E = young_obs
    ctx = FemContext(p, semantics="consistent")
    f = ctx.rhs()
    u_obs = ctx.pcg(f, **kw)[0].reshape(-1, 3)[sensors]
    ctx.set_young(young)

    def loss(u):
        u = u.reshape(-1, 3)
        return float(f @ u.ravel() + 0.5 * np.sum((u[sensors] - u_obs) ** 2))

    u, inf_f = ctx.pcg(f, **kw)
    g = f.copy().reshape(-1, 3)
    g[sensors] += u.reshape(-1, 3)[sensors] - u_obs
    dE, _, inf_a = ctx.adjoint(u, g.ravel(), **kw)
    t_total = inf_f["solve_ms"] + inf_a["solve_ms"]
    # central differences
    rng2 = np.random.default_rng(7)
    v = rng2.standard_normal(p.n_elems) * young
    h = 1e-4
    ctx.set_young(young + h * v)
    lp = loss(ctx.pcg(f, **kw)[0])
    ctx.set_young(young - h * v)
    lm = loss(ctx.pcg(f, **kw)[0])
    fd_dir = (lp - lm) / (2 * h)
    ad_dir = float(dE @ v)
    errs = []
    for e in np.argsort(-np.abs(dE * young))[:20]:
        y = young.copy()
        y[e] *= 1 + h
        ctx.set_young(y)
        lp = loss(ctx.pcg(f, **kw)[0])
        y[e] = young[e] * (1 - h)
        ctx.set_young(y)
        lm = loss(ctx.pcg(f, **kw)[0])
        fd = (lp - lm) / (2 * h * young[e])
        errs.append(abs(fd - dE[e]) / abs(dE[e]))
    ctx.set_young(young)
    _line("adjoint gradient: forward + adjoint solve time", round(t_total, 2), "ms", False,
          {"workload": "tet cantilever 32x32x128 x 6 (786,432 tets, 421,443 DOF), E_e = 2e7 exp(0.5 z_e) seed 3, "
                       "loss f.u + 1/2 |u_s - u_obs|^2 at 500 surface sensors, u_obs from field seed 4",
           "precision": "FP32 inner PCG + FP64 refinement to true rel. residual 1e-13"},
          {"forward_ms": round(inf_f["solve_ms"], 2), "adjoint_ms": round(inf_a["solve_ms"], 2),
           "fd_directional_rel_err": abs(fd_dir - ad_dir) / abs(ad_dir),
           "fd_20_elements_max_rel_err": max(errs), "fd_20_elements_median_rel_err": float(np.median(errs))})


def run_dynamics_workload():
    """Tet column 1x1x8, 32x32x256 x 6 (1,572,864 tets), rho 2000, E 2e7, nu 0.25,
    base clamped, Ricker point force (25 Hz, -z) at the top centre. Explicit
    central difference (lumped mass) at 0.5 x the stability limit from 100
    power iterations on M_L^-1 K (seed 5), 5000 steps; implicit Newmark
    beta 0.25 gamma 0.5 (GN22 beta1 = beta2 = 0.5), dt 1 ms, 1000 steps,
    warm-started PCG per step."""
    from cudafemproject_gb300 import meshgen
    from cudafemproject_gb300.meshio import WaveletParams
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(32, 32, 256, lz=8.0, E=2e7, nu=0.25, rho=2000.0, traction=(0.0, 0.0, 0.0),
                       point_load=("top_centre", (0.0, 0.0, -1.0)))
    ctx = FemContext(p, semantics="consistent")
    X = p.nodes[p.elems]
    vol = np.abs(np.einsum("ij,ij->i", X[:, 1] - X[:, 0], np.cross(X[:, 2] - X[:, 0], X[:, 3] - X[:, 0]))) / 6
    m = np.zeros(p.n_nodes)
    np.add.at(m, p.elems.ravel(), np.repeat(p.rho * vol / 4, 4))
    minv = np.repeat(1.0 / m, 3)
    x = np.random.default_rng(5).standard_normal(p.n_dof)
    lam = 0.0
    for _ in range(100):
        y = minv * ctx.matvec(x, "fp64")
        lam = float(np.linalg.norm(y) / np.linalg.norm(x))
        x = y / np.linalg.norm(y)
    dt = 0.5 * 2.0 / np.sqrt(lam)
    w = WaveletParams("ricker", 25.0, 0.0, 1.0)
    res = {}
    for prec in ("fp32", "fp64"):
        ctx.dyn(0.5, 0.0, dt, 10 * dt * 1.0000001, precision=prec, wavelet=w)
        u, info = ctx.dyn(0.5, 0.0, dt, 5000 * dt * 1.0000001, precision=prec, wavelet=w)
        res["explicit_" + prec] = {"steps": info["steps"], "ms": round(info["solve_ms"], 1),
                                   "steps_per_s": round(info["steps"] / (info["solve_ms"] * 1e-3), 1)}
    ue32, _ = ctx.dyn(0.5, 0.0, dt, 200 * dt * 1.0000001, precision="fp32", wavelet=w)
    ue64, _ = ctx.dyn(0.5, 0.0, dt, 200 * dt * 1.0000001, precision="fp64", wavelet=w)
    res["explicit_fp32_vs_fp64_rel_diff_200_steps"] = float(np.linalg.norm(ue32 - ue64) / np.linalg.norm(ue64))
    u, info = ctx.dyn(0.5, 0.5, 1e-3, 1000 * 1e-3 * 1.0000001, precision="fp64", wavelet=w, pcg_tol=1e-10,
                      stop_rule="residual", warm_start=True)
    res["implicit_fp64"] = {"steps": info["steps"], "ms": round(info["solve_ms"], 1),
                            "steps_per_s": round(info["steps"] / (info["solve_ms"] * 1e-3), 1),
                            "pcg_iterations": info["pcg_iterations"]}
    u32, info = ctx.dyn(0.5, 0.5, 1e-3, 1000 * 1e-3 * 1.0000001, precision="fp32", wavelet=w, pcg_tol=1e-6,
                        stop_rule="residual", warm_start=True)
    res["implicit_fp32"] = {"steps": info["steps"], "ms": round(info["solve_ms"], 1),
                            "steps_per_s": round(info["steps"] / (info["solve_ms"] * 1e-3), 1),
                            "pcg_iterations": info["pcg_iterations"],
                            "rel_diff_vs_fp64": float(np.linalg.norm(u32 - u) / np.linalg.norm(u))}
    _line("elastodynamics steps/s (explicit, FP32)", res["explicit_fp32"]["steps_per_s"], "steps/s", True,
          {"workload": "tet column 1x1x8, 32x32x256 x 6 (1,572,864 tets, 839,619 DOF), Ricker 25 Hz point force",
           "explicit_dt": dt, "omega_max": float(np.sqrt(lam))}, res)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--small", action="store_true", help="a 24x24x96 box (profiling runs)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-oracle", action="store_true", help="measure errors against the GPU FP64 solution instead")
    ap.add_argument("--no-multi", action="store_true", help="skip the 64-case multi-RHS leg")
    ap.add_argument("--no-configs", action="store_true", help="skip the adjoint, dynamics and batched-mesh legs")
    ap.add_argument("--workload", default="cantilever", choices=["cantilever", "multi_rhs", "batch", "adjoint", "dynamics"],
                    help="cantilever: the headline solve; the others measure the remaining configurations "
                         "(one JSON line each, single GPU)")
    args = ap.parse_args()
    if args.workload != "cantilever" and args.impl != "reference":
        return run_other_workload(args)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)

    world, rank, local = _dist_env()
    from cudafemproject_gb300 import meshgen
    if args.small:
        p = meshgen.box_3d(24, 24, 96, jitter=0.2, seed=0, traction=(0.0, -1e3, 0.0))
    else:
        p = meshgen.cantilever_1p39m()
    # 1. the FP64 oracle solution of this mesh, on the host cores, before any GPU work
    x_orc, f_orc, cpu_fp64, pin = (None, None, None, None)
    if not args.no_oracle and world == 1:
        x_orc, f_orc, cpu_fp64, pin = oracle_solution(p)

    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from cudafemproject_gb300 import capi
    from cudafemproject_gb300.solver import FemContext
    import ctypes as C

    t0 = time.time()
    ctx = FemContext(p, semantics="consistent")
    setup_ms = (time.time() - t0) * 1e3
    L = capi.lib()
    nd = p.n_dof
    f_host = ctx.rhs()
    # FP64 GPU solution converged to relative residual 1e-13 (untimed)
    x64, inf64c = ctx.pcg(f_host, "fp64", tol=1e-13, stop_rule="residual", max_iter=40000, allow_not_converged=True)
    x64 = np.asarray(x64)
    xr = x_orc if x_orc is not None else x64
    nref = np.linalg.norm(xr)

    def err(u):
        return float(np.linalg.norm(np.asarray(u).ravel() - xr) / nref)

    accuracy = {"target": "rel. displacement error <= 1e-8 against " +
                ("the FP64 oracle solution (host cores, rel. residual %g)" % pin["tol"] if x_orc is not None
                 else "the GPU FP64 solution (oracle skipped)")}
    if x_orc is not None:
        accuracy["rhs_rel_diff_vs_oracle"] = float(np.max(np.abs(f_host - f_orc)) / np.max(np.abs(f_orc)))
        accuracy["rel_err_vs_oracle_fp64_converged"] = err(x64)
        accuracy["oracle_iterations"] = pin["iterations"]

    # resident inputs for the device-side timing
    f_dev = torch.tensor(f_host, device="cuda")
    u_dev = torch.zeros(nd, dtype=torch.float64, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def solve(kw, f=f_dev, out=u_dev):
        return ctx.pcg(f, out=out, allow_not_converged=True, **kw)

    # Calibration (untimed): for each method the loosest stopping tolerance
    # whose answer is within TARGET_ERR of the oracle solution.
    plain64 = None
    for tol in (1e-6, 1e-7, 1e-8, 1e-9, 1e-10, 1e-11, 1e-12):
        kw = dict(precision="fp64", tol=tol, stop_rule="residual", max_iter=40000)
        _, i64 = solve(kw)
        if err(u_dev.cpu().numpy()) <= TARGET_ERR:
            plain64 = kw
            break
    # inner tolerances from 0.2 up continue the FP32 search direction across
    # refinement steps (FP64 residual replacement); tighter ones restart
    refine, best = None, None
    for inner in (0.5, 0.4, 0.3, 0.25, 0.2, 1e-3):
        for outer in (1e-6, 1e-7, 1e-8, 1e-9, 1e-10):
            kw = dict(precision="fp32_refine", tol=inner, stop_rule="residual", outer_tol=outer, max_outer=30,
                      max_iter=40000)
            _, i32 = solve(kw)
            if err(u_dev.cpu().numpy()) <= TARGET_ERR:
                if best is None or i32["solve_ms"] < best:
                    refine, best = kw, i32["solve_ms"]
                break
    if refine is None or plain64 is None:
        raise SystemExit(f"calibration failed to reach {TARGET_ERR}: refine={refine} fp64={plain64}")
    for _ in range(args.warmup):
        solve(refine)
    torch.cuda.synchronize()
    times, infos = [], []
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
    accuracy["rel_err_vs_oracle_refine" if x_orc is not None else "rel_err_refine"] = err(u_dev.cpu().numpy())
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
    accuracy["rel_err_vs_oracle_fp64" if x_orc is not None else "rel_err_fp64"] = err(u_dev.cpu().numpy())
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
    config = dict(CONFIG)
    if args.small:
        config["workload"] = WORKLOAD_SMALL
    line = {
        "metric": METRIC, "value": round(ms, 3), "unit": "ms", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": DATA, "config": config,
        "precision": (f"FP32 inner PCG (rel. residual {refine['tol']:g}) + FP64 refinement (true rel. residual "
                      f"{refine['outer_tol']:g}); plain FP64 arm: recursive rel. residual {plain64['tol']:g}"),
        "accuracy": accuracy,
        "fp64_ms": round(ms64, 3), "speedup_vs_fp64": round(ms64 / ms, 3),
        "pcg_iterations": its, "outer_iterations": infos[-1]["outer_iterations"],
        # FP32 halo sums use atomics, so the inner iteration count varies a little from run to run
        "steps_ms": {"min": round(min(times), 3), "median": round(float(np.median(times)), 3),
                     "max": round(max(times), 3)},
        "steps_pcg_iterations": {"min": min(i["iterations"] for i in infos),
                                 "max": max(i["iterations"] for i in infos)},
        "ps_per_tet_iteration": round(ms * 1e9 / (ctx.counts()["n_elems"] * float(np.mean([i["iterations"] for i in infos]))), 2),
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
    if rank == 0 and world == 1 and not args.no_multi:
        line["multi_rhs"] = multi_rhs_leg(torch, check_oracle=not args.no_oracle)
    if rank == 0 and world == 1 and not args.no_configs:
        line["adjoint"] = adjoint_leg(check_oracle=not args.no_oracle)
        line["dynamics"] = dynamics_leg()
        line["batch"] = batch_leg(check_oracle=not args.no_oracle)
    if rank == 0 and world == 1 and not args.no_cpu:
        # reference rule iteration count on the GPU (FP32, gamma < 1e-8 gamma0) for the extrapolation
        _, ir = ctx.pcg(f_dev, out=u_dev, precision="fp32", tol=1e-8, stop_rule="reference",
                        allow_not_converged=True)
        line["cpu_baseline"] = cpu_baseline(p, K_REF, ir["iterations"],
                                            "measured in this run by the GPU FP32 PCG with the same rule")
        if cpu_fp64 is not None:
            line["cpu_baseline_fp64_mt"] = cpu_fp64
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def multi_rhs_leg(torch, check_oracle: bool = True, k: int = 64):
    """64 traction load cases on the 24x24x96 tet box (331,776 tets, 181,875
    DOF): each case a traction on z = max, direction uniform on the sphere,
    magnitude log-uniform in [1e2, 1e4] (seed 1: k directions, then k
    magnitudes), solved to 1e-8 relative error as one multi-RHS PCG (FP32 +
    FP64 refinement) and one case at a time. Each path's inner and outer
    tolerances are calibrated (untimed) to its fastest setting that reaches
    1e-8 on the first and last case against FP64 solutions."""
    from cudafemproject_gb300 import meshgen
    from cudafemproject_gb300.solver import FemContext
    nx, ny, nz = 24, 24, 96
    E3 = np.stack([FemContext(meshgen.box_3d(nx, ny, nz, traction=t), semantics="consistent").rhs()
                   for t in ((1.0, 0, 0), (0, 1.0, 0), (0, 0, 1.0))])
    pb = meshgen.box_3d(nx, ny, nz)
    ctx = FemContext(pb, semantics="consistent")
    rng = np.random.default_rng(1)
    d = rng.standard_normal((k, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    F = (d * (10.0 ** rng.uniform(2, 4, size=k))[:, None]) @ E3
    probe = (0, k - 1)
    ref = {i: np.asarray(ctx.pcg(F[i], "fp64", tol=1e-13, stop_rule="residual", max_iter=40000)[0]) for i in probe}
    err = lambda i, u: float(np.linalg.norm(np.asarray(u).ravel() - ref[i]) / np.linalg.norm(ref[i]))

    def calibrate(run):
        """inner tolerance -> (ms, kw) of the loosest outer tolerance reaching the target"""
        found = {}
        for inner in (0.4, 0.3, 0.2, 1e-4):
            for outer in (1e-6, 1e-7, 1e-8, 1e-9):
                kw = dict(precision="fp32_refine", tol=inner, stop_rule="residual", outer_tol=outer, max_outer=100,
                          max_iter=20000)
                ms, e, its = run(kw)
                if e <= TARGET_ERR:
                    found[inner] = (ms, kw, its)
                    break
        return found

    def run_single(kw):
        infs = [ctx.pcg(F[i], **kw)[1] for i in (1, 2, 3)]
        e = max(err(i, ctx.pcg(F[i], **kw)[0]) for i in probe)
        return float(np.median([i["solve_ms"] for i in infs])), e, float(np.median([i["iterations"] for i in infs]))

    def run_multi(kw):
        U, infos = ctx.pcg_multi(F, **kw)
        return infos[0]["solve_ms"], max(err(i, U[i]) for i in probe), infos[0]["kernel_launches"] / 2.0

    single = calibrate(run_single)
    multi = calibrate(run_multi)
    torch.cuda.synchronize()
    # equal settings: the restarted refinement (inner 1e-4) on both paths, timed again
    same_kw = multi[1e-4][1]
    U, infos = ctx.pcg_multi(F, **same_kw)
    ms_multi = infos[0]["solve_ms"]
    launches_multi = infos[0]["kernel_launches"]
    s_kw = dict(same_kw)
    s_kw["outer_tol"] = single[1e-4][1]["outer_tol"]
    s_inf = [ctx.pcg(F[i], **s_kw)[1] for i in range(1, 6)]
    ms_single = float(np.median([i["solve_ms"] for i in s_inf]))
    best_s = min(single.values(), key=lambda v: v[0])
    best_m = min(multi.values(), key=lambda v: v[0])
    out = {"workload": f"24x24x96 tet box (331,776 tets, 181,875 DOF), {k} traction load cases (seed 1)",
           "precision": "FP32 inner PCG + FP64 refinement to 1e-8 relative error on every path",
           "equal_settings": {"inner": same_kw["tol"], "outer_multi": same_kw["outer_tol"],
                              "outer_single": s_kw["outer_tol"]},
           "batched_ms_total": round(ms_multi, 2), "ms_per_case": round(ms_multi / k, 3),
           "single_rhs_ms": round(ms_single, 3), "per_rhs_speedup": round(ms_single / (ms_multi / k), 2),
           "best_settings": {"multi_inner": best_m[1]["tol"], "multi_ms_per_case": round(best_m[0] / k, 3),
                             "single_inner": best_s[1]["tol"], "single_ms": round(best_s[0], 3),
                             "per_rhs_speedup": round(best_s[0] / (best_m[0] / k), 2)},
           "max_iterations": max(i["iterations"] for i in infos)}
    # the batching gain of the PCG iteration itself: 400 FP32 iterations of
    # one case against 400 of all k cases
    # (a context of its own: the cases all active from the first iteration)
    kw_it = dict(precision="fp32", tol=1e-30, stop_rule="residual", max_iter=400, allow_not_converged=True)
    ctx.pcg(F[0], **kw_it)
    t1 = float(np.median([ctx.pcg(F[0], **kw_it)[1]["solve_ms"] for _ in range(3)])) / 400
    ctx_k = FemContext(pb, semantics="consistent")
    ctx_k.pcg_multi(F, **kw_it)
    tk = min(ctx_k.pcg_multi(F, **kw_it)[1][0]["solve_ms"] for _ in range(2)) / 400
    ctx_k.close()
    out["pcg_iteration_ms"] = {"single": round(t1, 5), "multi": round(tk, 5),
                               "per_rhs_throughput_ratio": round(k * t1 / tk, 2)}
    if check_oracle:
        oracle = _oracle()
        o = oracle.Oracle(pb, consistent=True).assemble()
        errs = []
        for i in probe:
            xo, _ = o.pcg(F[i], tol=1e-12, rule=1)
            errs.append(float(np.linalg.norm(U[i] - xo) / np.linalg.norm(xo)))
        out["rel_err_vs_oracle_cases_0_and_last"] = max(errs)
    ctx.close()
    return out


def adjoint_leg(check_oracle: bool = True):
    """Adjoint gradient on the tet cantilever 32x32x128 x 6 (786,432 tets,
    421,443 DOF) with E_e = 2e7 exp(0.5 z_e), z_e standard normal (seed 3);
    loss = f.u + 1/2 sum over 500 surface sensors |u_s - u_obs|^2, u_obs from a
    second modulus field (seed 4). Forward and adjoint solves by FP32 PCG +
    FP64 refinement to a true relative residual of 1e-13; dL/dE against the
    FP64 oracle's adjoint gradient of the same mesh and against central
    differences along a random direction (relative step 1e-4)."""
    from cudafemproject_gb300 import meshgen
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(32, 32, 128, traction=(0.0, -1e3, 0.0))
    rng = np.random.default_rng(3)
    young = 2e7 * np.exp(0.5 * rng.standard_normal(p.n_elems))
    surf = np.nonzero((p.nodes[:, 0] <= 1e-9) | (p.nodes[:, 0] >= 1 - 1e-9) | (p.nodes[:, 1] <= 1e-9) |
                      (p.nodes[:, 1] >= 1 - 1e-9) | (p.nodes[:, 2] >= 4 - 1e-9))[0]
    sensors = rng.choice(surf, size=500, replace=False)
    young_obs = 2e7 * np.exp(0.5 * np.random.default_rng(4).standard_normal(p.n_elems))
    kw = dict(precision="fp32_refine", tol=0.4, stop_rule="residual", outer_tol=1e-13, max_outer=200, max_iter=40000)
    p.elem_E = young_obs
    ctx = FemContext(p, semantics="consistent")
    f = ctx.rhs()
    u_obs = np.asarray(ctx.pcg(f, **kw)[0]).reshape(-1, 3)[sensors]
    p.elem_E = young
    ctx.set_young(young)
    ctx.pcg(f, **kw)
    u, inf_f = ctx.pcg(f, **kw)
    g = f.copy().reshape(-1, 3)
    g[sensors] += np.asarray(u).reshape(-1, 3)[sensors] - u_obs
    dE, df, inf_a = ctx.adjoint(u, g.ravel(), **kw)

    def loss(uu):
        uu = np.asarray(uu).reshape(-1, 3)
        return float(f @ uu.ravel() + 0.5 * np.sum((uu[sensors] - u_obs) ** 2))

    v = np.random.default_rng(7).standard_normal(p.n_elems) * young
    h = 1e-4
    ctx.set_young(young + h * v)
    lp = loss(ctx.pcg(f, **kw)[0])
    ctx.set_young(young - h * v)
    lm = loss(ctx.pcg(f, **kw)[0])
    ctx.set_young(young)
    fd = (lp - lm) / (2 * h)
    out = {"workload": "tet cantilever 32x32x128 x 6 (786,432 tets, 421,443 DOF), E_e = 2e7 exp(0.5 z_e) seed 3, "
                       "compliance + 500-sensor misfit (u_obs from field seed 4)",
           "forward_ms": round(inf_f["solve_ms"], 2), "adjoint_ms": round(inf_a["solve_ms"], 2),
           "fd_directional_rel_err": abs(fd - float(dE @ v)) / abs(float(dE @ v))}
    ctx.close()
    if check_oracle:
        oracle = _oracle()
        o = oracle.Oracle(p, consistent=True).assemble()
        uo, _ = o.pcg(f, tol=1e-12, rule=1)
        go = f.copy().reshape(-1, 3)
        go[sensors] += uo.reshape(-1, 3)[sensors] - u_obs
        lam, _ = o.pcg(go.ravel(), tol=1e-12, rule=1)
        gE = o.grad_E(lam, uo)
        out["rel_err_vs_oracle_dLdE"] = float(np.linalg.norm(dE - gE) / np.linalg.norm(gE))
        out["rel_err_vs_oracle_dLdf"] = float(np.linalg.norm(np.asarray(df) - lam) / np.linalg.norm(lam))
    return out


def dynamics_leg():
    """Elastodynamics on the tet column 1x1x8, 32x32x256 x 6 (1,572,864 tets,
    839,619 DOF), rho 2000, E 2e7, nu 0.25, base clamped, Ricker point force
    (25 Hz, -z) at the top centre, consistent semantics. Explicit central
    difference (lumped mass) at 0.5 x the stability limit (100 power iterations
    on M_L^-1 K, seed 5): 2000 FP32 and 200 FP64 steps. Implicit Newmark (beta
    0.25, gamma 0.5), dt 1 ms, warm-started PCG per step: 100 FP32 steps
    (relative residual 1e-6) and 20 FP64 steps (1e-10)."""
    from cudafemproject_gb300 import meshgen
    from cudafemproject_gb300.meshio import WaveletParams
    from cudafemproject_gb300.solver import FemContext
    p = meshgen.box_3d(32, 32, 256, lz=8.0, E=2e7, nu=0.25, rho=2000.0, traction=(0.0, 0.0, 0.0),
                       point_load=("top_centre", (0.0, 0.0, -1.0)))
    ctx = FemContext(p, semantics="consistent")
    X = p.nodes[p.elems]
    vol = np.abs(np.einsum("ij,ij->i", X[:, 1] - X[:, 0], np.cross(X[:, 2] - X[:, 0], X[:, 3] - X[:, 0]))) / 6
    m = np.zeros(p.n_nodes)
    np.add.at(m, p.elems.ravel(), np.repeat(p.rho * vol / 4, 4))
    minv = np.repeat(1.0 / m, 3)
    x = np.random.default_rng(5).standard_normal(p.n_dof)
    lam = 0.0
    for _ in range(100):
        y = minv * ctx.matvec(x, "fp64")
        lam = float(np.linalg.norm(y) / np.linalg.norm(x))
        x = y / np.linalg.norm(y)
    dt = 0.5 * 2.0 / np.sqrt(lam)
    w = WaveletParams("ricker", 25.0, 0.0, 1.0)
    out = {"workload": "tet column 1x1x8, 32x32x256 x 6 (1,572,864 tets, 839,619 DOF), Ricker 25 Hz point force",
           "explicit_dt": dt}
    ctx.dyn(0.5, 0.0, dt, 10 * dt * 1.0000001, precision="fp32", wavelet=w)
    for prec, n in (("fp32", 2000), ("fp64", 200)):
        _, info = ctx.dyn(0.5, 0.0, dt, n * dt * 1.0000001, precision=prec, wavelet=w)
        out["explicit_" + prec + "_steps_per_s"] = round(info["steps"] / (info["solve_ms"] * 1e-3), 1)
    ue32, _ = ctx.dyn(0.5, 0.0, dt, 200 * dt * 1.0000001, precision="fp32", wavelet=w)
    ue64, _ = ctx.dyn(0.5, 0.0, dt, 200 * dt * 1.0000001, precision="fp64", wavelet=w)
    out["explicit_fp32_vs_fp64_rel_diff_200_steps"] = float(np.linalg.norm(ue32 - ue64) / np.linalg.norm(ue64))
    for prec, n, tol in (("fp32", 100, 1e-6), ("fp64", 20, 1e-10)):
        _, info = ctx.dyn(0.5, 0.5, 1e-3, n * 1e-3 * 1.0000001, precision=prec, wavelet=w, pcg_tol=tol,
                          stop_rule="residual", warm_start=True)
        out["implicit_" + prec + "_steps_per_s"] = round(info["steps"] / (info["solve_ms"] * 1e-3), 1)
        out["implicit_" + prec + "_pcg_iterations_per_step"] = round(info["pcg_iterations"] / info["steps"], 1)
    ctx.close()
    return out


def batch_leg(check_oracle: bool = True):
    """64 independent tet boxes n x n x 4n, n uniform in 8..40 (seed 2), E
    log-uniform in [1e6, 1e8], nu uniform in [0.2, 0.4], each clamped at z=0
    with a traction on its top face: solved together in one persistent launch
    per kernel (per-instance convergence masks, graph replay) against the same
    solves one mesh after the other, both FP32 PCG + FP64 refinement (inner
    1e-4, outer 1e-8). Errors against the FP64 oracle for the two smallest
    boxes and against GPU FP64 solutions for the two largest."""
    from cudafemproject_gb300 import meshgen
    from cudafemproject_gb300.solver import BatchContext, FemContext
    probs = meshgen.batch_boxes(64, seed=2)
    kw = dict(precision="fp32_refine", tol=1e-4, stop_rule="residual", outer_tol=1e-8, max_iter=20000)
    b = BatchContext(probs)
    b.static_solve(**kw)
    us, infos = b.static_solve(**kw)
    ms_b = infos[0]["solve_ms"]
    b.close()
    sizes = np.array([p.n_elems for p in probs])
    tet_its = float(np.dot(sizes, [i["iterations"] for i in infos]))
    small = list(np.argsort(sizes)[:2])
    large = list(np.argsort(sizes)[-2:])
    seq, errs, seq_its = 0.0, {}, []
    for i, p in enumerate(probs):
        ctx = FemContext(p, semantics="consistent")
        ctx.static_solve(**kw)
        _, inf = ctx.static_solve(**kw)
        seq += inf["solve_ms"]
        seq_its.append(inf["iterations"])
        if i in large:
            ref, _ = ctx.static_solve("fp64", tol=1e-13, stop_rule="residual", max_iter=60000, allow_not_converged=True)
            errs[f"box_{i}_vs_gpu_fp64"] = float(np.linalg.norm(us[i] - ref) / np.linalg.norm(ref))
        ctx.close()
    if check_oracle:
        oracle = _oracle()
        for i in small:
            xo, _ = oracle.Oracle(probs[i], consistent=True).assemble().static(tol=1e-12, rule=1)
            errs[f"box_{i}_vs_oracle"] = float(np.linalg.norm(us[i].ravel() - xo) / np.linalg.norm(xo))
    return {"workload": f"64 tet boxes n x n x 4n, n uniform in 8..40 (seed 2), E log-uniform [1e6, 1e8], nu uniform "
                        f"[0.2, 0.4]: {int(sizes.sum())} tets, {sum(p.n_dof for p in probs)} DOF",
            "batched_ms": round(ms_b, 1), "sequential_ms": round(seq, 1), "speedup_vs_sequential": round(seq / ms_b, 3),
            "max_iterations": max(i["iterations"] for i in infos),
            # time per tet and inner PCG iteration (the work each instance needs): the batched solve
            # against the same solves one by one, comparable with the headline solve's
            "ps_per_tet_iteration": {"batched": round(ms_b * 1e9 / tet_its, 2),
                                     "sequential": round(seq * 1e9 / float(np.dot(sizes, seq_its)), 2)},
            "rel_err": errs}


if __name__ == "__main__":
    sys.exit(main())
