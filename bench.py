"""Benchmark of the ubootgl fluid step on one GB300.

Workload (the metric's configuration): one 4096 x 2048 staggered-MAC grid,
float32 u/v/p, uint8 flag; solid top/bottom walls plus 12 seeded solid
discs (radius 20-60 cells at W = 1024, scaled to W); inflow u = 1.0;
initial velocity 1.0 + 0.1 * Gaussian-smoothed (sigma 8) noise; mu = 1e-4;
dt = 0.5 h / max|u| computed on the device every step.  A "step" is
Simulation::step (simulation.cpp:356-374): diffusion, bicubic
semi-Lagrangian advection, projection with the reference's two multigrid
V-cycles, boundary conditions.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  `value` is whole-job Mcell-steps/s with all fields
resident in HBM; `e2e` is the same metric through the C ABI with host
buffers (each step uploads vx, vy from pinned host memory and downloads the
display fields vx_current, vy_current).  The reference arm times the CPU
step on the host cores (see --impl reference).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W_DEFAULT, H_DEFAULT = 4096, 2048
# the headline metric as the benchmark specification names it; `value` is the
# FP32 drop-in (the reference's step: 2 V-cycles), `modes` the mixed
# solvers and `served` the p50/p99 latencies
METRIC = "Mcell-steps/s at 4096x2048 (FP32 vs mixed, \u22641e-5 resid); served p50/p99 latency"


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def workload(W, H, seed=2024):
    from ubootgl_gb300 import workload as WL
    flag = WL.disc_flag(W, H, n_discs=12, r_range=(20, 60), seed=seed)
    vx, vy = WL.initial_velocity(flag, seed=seed + 1)
    return flag, vx, vy


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.proc = None
        self.lines = []
        self.gpu = gpu_index

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def workload_name(W, H):
    """config.workload of both arms."""
    return "fluid step %dx%d, 12 discs, FP32, 2 V-cycles, dt=0.5h/max|u|" % (W, H)


def time_cpu_step(W, H, budget_s=20.0, min_steps=3, max_steps=None, threads=None, warmup=1):
    """The reference step on the host cores: oracle/_ref (the reference's own
    simulation.cpp built from source with its own -Ofast -march=native) where
    it builds (x86-64), else the C restatement of it built for speed (-O3
    -ffast-math; the parity build of the restatement is never timed).
    Returns (Mcell-steps/s, info)."""
    from oracle import oracle as O
    flag, vx, vy = workload(W, H)
    threads = threads or cpu_threads()
    kind = "port"
    sim = None
    try:
        if O.ref_available():
            # the classic (deterministic) red-black schedule needs H/T < 100
            sim = O.RefSim(flag, threads=max(threads, H // 100 + 1))
            kind = "reference"
    except Exception:
        sim = None
    if sim is None:
        O.set_threads(threads, fast=True)
        sim = O.PortSim(flag, fast=True)
    for n in ("vx", "vy", "vx_back", "vy_back"):
        sim.set(n, vx if n.startswith("vx") else vy)
    from ubootgl_gb300 import workload as WL
    h = sim.h
    for _ in range(max(1, warmup)):
        sim.step(WL.cfl_dt(sim.get("vx"), sim.get("vy"), h))
    n, t_total = 0, 0.0
    while True:
        dt = WL.cfl_dt(sim.get("vx"), sim.get("vy"), h)
        t0 = time.perf_counter()
        sim.step(dt)
        t_total += time.perf_counter() - t0
        n += 1
        if (n >= min_steps and t_total >= budget_s) or (max_steps and n >= max_steps):
            break
    val = W * H * n / t_total / 1e6
    return val, {"kind": kind, "cores": threads, "steps": n, "seconds": t_total,
                 "build": ("reference sources, -Ofast -march=native" if kind == "reference"
                           else "C restatement, -O3 -ffast-math -funroll-loops, OpenMP"),
                 "sample": "%dx%d full steps (2 V-cycles), %d timed after %d warm-up; "
                           "dt = 0.5 h/max|u| computed outside the timed call"
                           % (W, H, n, max(1, warmup))}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    W, H = args.width, args.height
    steps = max(1, args.steps)
    # each timed step is one full CPU step of the workload: K steps after W
    # warm-up steps, as the GPU arm (at ~0.1 s per step on 16 cores the
    # default run takes a few seconds; K is capped at 500)
    val, info = time_cpu_step(W, H, budget_s=0.0, min_steps=min(steps, 500),
                              max_steps=min(steps, 500), warmup=args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(val, 3), "unit": "Mcell-steps/s",
        "n_gpus": args.gpus, "steps": info["steps"], "warmup": args.warmup,
        "ms_per_step": round(1e3 * info["seconds"] / info["steps"], 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded disc mask + smoothed-noise velocity)",
        "config": {"workload": workload_name(W, H), "parallelism": "host cores"},
        "cpu_baseline": {"value": round(val, 3), "unit": "Mcell-steps/s", "cores": info["cores"],
                         "kind": info["kind"], "sample": info["sample"], "build": info["build"]},
        "e2e": {"value": round(val, 3), "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    if info["kind"] == "port":
        line["note"] = ("the reference's step uses x86 AVX2 intrinsics (interpolators.hpp) and "
                        "does not build on this aarch64 host; its C restatement is timed instead")
    print(json.dumps(line), flush=True)


def run_ours(args):
    import ctypes as C

    rank, world, local = dist_env()
    from ubootgl_gb300 import _lib as L
    from ubootgl_gb300.simulation import Simulation

    lib = L.load()
    W, H = args.width, args.height
    flag, vx, vy = workload(W, H, seed=2024 + rank)
    sim = Simulation(flag, 1.0, 1e-4)
    sim.set("vx", vx)
    sim.set("vy", vy)
    sim.set("vx_back", vx)
    sim.set("vy_back", vy)
    stream = C.c_void_p()
    L.check(lib.ubg_stream(sim._h, C.byref(stream)))

    import torch
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    ext_stream = torch.cuda.ExternalStream(stream.value, device=dev)
    pg = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        pg = dist

    def barrier():
        if pg:
            pg.barrier()

    # multigrid tiles and tail size for this grid (bit-identical results)
    tune = sim.autotune() if not args.no_autotune else None
    for _ in range(args.warmup):
        sim.step_cfl(0.5)
    sim.sync()

    # ---- timed region: K steps, fields resident in HBM
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    barrier()
    sim.sync()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(ext_stream)
    for _ in range(args.steps):
        sim.step_cfl(0.5)
    ev1.record(ext_stream)
    sim.sync()
    barrier()
    clk = clocks.stop()
    prof = sim.profile_read()
    cells = W * H
    ms, value = replica_throughput(ev0.elapsed_time(ev1), cells, args.steps, world, pg, dev)
    ms_step = ms / args.steps
    launches_per_step = prof["kernel_launches"]

    # ---- dominant kernel timing (CUDA events on the handle's stream)
    kt = kernel_timing(sim, lib, W, H, reps=args.profile_steps)

    # ---- end-to-end through the C ABI with host buffers
    e2e = end_to_end(sim, L, lib, W, H, max(3, min(args.steps, args.e2e_steps)), barrier, pg,
                     world, dev)

    if rank != 0:
        return

    # ---- the plain FP32 step at scale with tracers (8192 x 4096)
    scale = scale_bench(L, lib, args.scale_steps, args.warmup, dev) if args.scale_steps > 0 else {}

    # ---- the solver modes on the same workload (extensions): the tolerance
    # solver in FP32 / FP16 / BF16 to the same relative residual, and the
    # fixed two-cycle mixed solvers
    modes = {}
    if args.tol_steps > 0:
        for prec in ("fp32", "fp16", "bf16"):
            modes["tol_" + prec] = time_tolerance(L, lib, flag, vx, vy, prec, args.tol_steps,
                                                  args.warmup, dev, args.tol)
        base = modes["tol_fp32"]["value"]
        for prec in ("fp16", "bf16"):
            modes["tol_" + prec]["vs_fp32_at_equal_tol"] = round(modes["tol_" + prec]["value"] / base, 3)
    if args.mode_steps > 0:
        for prec in ("fp16", "bf16"):
            modes["fixed_" + prec] = time_mode(L, lib, flag, vx, vy, prec, args.mode_steps,
                                               args.warmup, dev)
        # the advection option: bilinearSample for the back-trace
        modes["fp32_bilinear_advect"] = time_mode(L, lib, flag, vx, vy, "fp32", args.mode_steps,
                                                  args.warmup, dev, advect="bilinear")

    # ---- batched uneven instances and the served stream (extensions)
    batched, served = {}, {}
    if args.batch > 0:
        for prec in args.batch_precisions.split(","):
            batched[prec] = batch_bench(L, lib, args.batch, args.batch_steps, args.warmup, prec)
        # small members, where one launch per kernel over the batch pays most
        batched["fp32_small"] = batch_bench(L, lib, args.batch, args.batch_steps, args.warmup,
                                            "fp32", wmin=128, wmax=512)
    if args.serve_sessions > 0:
        # the FP32 drop-in (two V-cycles), fused continuous batching: the
        # specified 2000 req/s and a rate sweep
        served["fixed_fp32_fused"] = serve_arm(L, args, "fp32", "fused", None,
                                               [250, 500, 1000, 2000], spec_rate=args.serve_rate)
        # the tolerance solver at the same divergence tolerance in FP32 and
        # mixed precision (pool threads, one stream per request)
        for prec in args.serve_precisions.split(","):
            served["tol_%s" % prec] = serve_arm(L, args, prec, "streams", args.serve_tol,
                                                [25, 50, 100, 200, 400, 800])

    line = {
        "metric": METRIC, "value": round(value, 2), "unit": "Mcell-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded disc mask + smoothed-noise velocity)",
        "config": {"workload": workload_name(W, H),
                   "solver": "FP32 drop-in: the reference's step with its 2 V-cycles (value); "
                             "tolerance solver (FP32 / FP16 / BF16 coarse levels, residual "
                             "<= tol) and fixed mixed solvers in modes; served stream in served",
                   "grid": [W, H], "parallelism": "replicas" if world > 1 else "single",
                   "l2": "inputs larger than L2: step working set %.0f MB > 129 MB"
                         % (working_set_bytes(W, H) / 1e6)},
        "autotune": ({"tail_cells": tune["tail_cells"],
                      "cluster_top": tune.get("cluster_top"),
                      "vcycle_us": tune.get("vcycle_us"),
                      "cluster_trial_us": [t["vcycle_us"] for t in tune.get("trials", [])
                                           if t.get("what") == "cluster"],
                      "tiles": [(lv["pre"], lv["post"]) for lv in tune["levels"]]}
                     if tune else None),
        "clocks": clk,
        "gpu_launches": int(launches_per_step * args.steps),
        "e2e": e2e,
        "roofline": kt["roofline"],
        "kernels": kt["detail"],
        "profiled_step_ms": kt["profiled_step_ms"],
        "modes": modes,
        "scale": scale,
        "batched": batched,
        "served": served,
    }
    if not args.no_cpu_baseline:
        val, info = time_cpu_step(W, H, budget_s=args.cpu_budget)
        line["cpu_baseline"] = {"value": round(val, 3), "unit": "Mcell-steps/s",
                                "cores": info["cores"], "kind": info["kind"],
                                "sample": info["sample"], "build": info["build"]}
    print(json.dumps(line), flush=True)


def time_tolerance(L, lib, flag, vx, vy, precision, steps, warmup, dev, tol):
    """Whole steps with the tolerance solver (flexible CG preconditioned by
    the tolerance hierarchy's V-cycle, coarse levels in `precision`) until
    ||r|| <= tol ||f_c|| every projection; CUDA events on the simulation's
    stream around `steps` steps (the solver synchronises once per V-cycle to
    test the residual, inside the timed region)."""
    import ctypes as C
    import torch
    from ubootgl_gb300.simulation import Simulation
    H, W = flag.shape
    sim = Simulation(flag, 1.0, 1e-4)
    sim.set_options(solver_mode=L.SOLVE_TOLERANCE, tol=tol, max_vcycles=200, precision=precision)
    for n, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
        sim.set(n, a)
    stream = C.c_void_p()
    L.check(lib.ubg_stream(sim._h, C.byref(stream)))
    ext = torch.cuda.ExternalStream(stream.value, device=dev)
    for _ in range(max(3, warmup)):
        sim.step_cfl(0.5)
    sim.sync()
    cycles, rels = [], []
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(steps):
        sim.step_cfl(0.5)
        c, r = sim.solver_stats()
        cycles.append(c)
        rels.append(r)
    e1.record(ext)
    sim.sync()
    ms = e0.elapsed_time(e1)
    finite = bool(np.isfinite(sim.get("p")).all())
    # per kernel class (direct launches with event pairs), a few steps
    sim.profile(True)
    sim.profile_reset()
    nprof = 3
    for _ in range(nprof):
        sim.step_cfl(0.5)
    sim.sync()
    classes = sim.profile_classes()
    sim.profile(False)
    sim.close()
    kern = {k: {"ms_per_step": round(v[0] / nprof, 4), "launches_per_step": round(v[1] / nprof, 1)}
            for k, v in sorted(classes.items(), key=lambda kv: -kv[1][0])}
    return {"value": round(W * H * steps / (ms / 1e3) / 1e6, 2), "unit": "Mcell-steps/s",
            "ms_per_step": round(ms / steps, 4), "steps": steps, "tol": tol, "kernels": kern,
            "vcycles_per_projection": round(float(np.mean(cycles)), 2),
            "vcycles_max": int(max(cycles)), "residual_max": float("%.3e" % max(rels)),
            "solver": "flexible CG (FP64 pressure, FP32 vectors, FP64 norms) preconditioned by "
                      "one V-cycle: level 0 FP32, coarse levels %s" % precision,
            "fields_finite": finite}


def time_mode(L, lib, flag, vx, vy, precision, steps, warmup, dev, advect="bicubic"):
    """Whole steps with the mixed-precision pressure solver (2 defect
    corrections, each one 16-bit V-cycle, in the captured step graph), or
    with precision "fp32" the plain step with the advection option, timed
    with CUDA events on the simulation's stream."""
    import ctypes as C
    import torch
    from ubootgl_gb300.simulation import Simulation
    H, W = flag.shape
    sim = Simulation(flag, 1.0, 1e-4)
    sim.set_options(solver_mode=L.SOLVE_FIXED, vcycles=2, precision=precision, advect=advect)
    for n, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
        sim.set(n, a)
    stream = C.c_void_p()
    L.check(lib.ubg_stream(sim._h, C.byref(stream)))
    ext = torch.cuda.ExternalStream(stream.value, device=dev)
    sim.autotune()
    for _ in range(max(3, warmup)):
        sim.step_cfl(0.5)
    sim.sync()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(ext)
    for _ in range(steps):
        sim.step_cfl(0.5)
    e1.record(ext)
    sim.sync()
    ms = e0.elapsed_time(e1)
    finite = bool(np.isfinite(sim.get("p")).all())
    # per kernel class (direct launches with event pairs), a few steps
    sim.profile(True)
    sim.profile_reset()
    for _ in range(5):
        sim.step_cfl(0.5)
    sim.sync()
    classes = sim.profile_classes()
    sim.profile(False)
    sim.close()
    kern = {k: {"ms_per_step": round(v[0] / 5, 4), "launches_per_step": round(v[1] / 5, 1)}
            for k, v in sorted(classes.items(), key=lambda kv: -kv[1][0])}
    return {"value": round(W * H * steps / (ms / 1e3) / 1e6, 2), "unit": "Mcell-steps/s",
            "ms_per_step": round(ms / steps, 5), "steps": steps, "kernels": kern,
            "solver": ("2 FP32 defect corrections, 16-bit (%s) V-cycle, FP64 norms and coarse "
                       "solve" % precision if precision != "fp32"
                       else "the reference's 2 FP32 V-cycles"),
            "advect": advect, "fields_finite": finite}


def batch_bench(L, lib, n, steps, warmup, precision, seed=11, wmin=128, wmax=2048):
    """Batched uneven instances: n simulations, widths log-uniform in
    [wmin, wmax] (multiples of 32), height = width / 2, each with its own
    seeded disc mask (8-15 % solid) and inflow speed (uniform [0.5, 1.5]);
    every member autotuned; all advance one step per batch graph launch.
    Host wall clock around K batch steps (synchronised), against the same
    members stepped one call each on their own streams."""
    from ubootgl_gb300 import workload as WL
    from ubootgl_gb300.simulation import Batch, Simulation
    widths = WL.log_uniform_widths(n, wmin, wmax, seed)
    sims, cells = [], 0
    for i, W in enumerate(widths):
        H = W // 2
        flag, vx, vy = WL.instance(W, H, seed * 1000 + i)
        sim = Simulation(flag, 1.0, 1e-4)
        if precision != "fp32":
            sim.set_options(precision=precision)
        for nm, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
            sim.set(nm, a)
        sims.append(sim)
        cells += W * H
    t0 = time.perf_counter()
    for sim in sims:
        sim.autotune()
    t_tune = time.perf_counter() - t0
    batch = Batch(sims)
    for _ in range(max(3, warmup)):
        batch.step(cfl=0.5)
    batch.sync()
    t0 = time.perf_counter()
    for _ in range(steps):
        batch.step(cfl=0.5)
    batch.sync()
    for s in sims:
        s.sync()
    t_batch = time.perf_counter() - t0
    t0 = time.perf_counter()
    for _ in range(steps):
        for s in sims:
            s.step_cfl(0.5)
    for s in sims:
        s.sync()
    t_seq = time.perf_counter() - t0
    finite = all(bool(np.isfinite(s.get("p")).all()) for s in sims[:4])
    batch.close()
    for s in sims:
        s.close()
    return {"value": round(cells * steps / t_batch / 1e6, 2), "unit": "Mcell-steps/s",
            "instances": n, "total_cells": cells, "steps": steps,
            "ms_per_batch_step": round(1e3 * t_batch / steps, 4),
            "one_call_per_member_value": round(cells * steps / t_seq / 1e6, 2),
            "autotune_s": round(t_tune, 2), "precision": precision, "fields_finite": finite,
            "widths": "log-uniform [%d, %d], h = w/2" % (wmin, wmax),
            "timing": "host wall clock, synchronised"}


def serve_open(L, n_sessions, budget_gb, max_active, precision, mode, tol=None, seed=5,
               wmin=256, wmax=4096, fuse_cells=None):
    """Opens n_sessions resident sessions, widths log-uniform in [wmin, wmax]
    (height = width / 2) under a device-memory budget.  Session fields are
    crops of one seeded 4096 x 2048 instance (walls re-applied, own inflow
    speed); tol selects the tolerance solver.  Every session takes one
    warm-up step."""
    from ubootgl_gb300 import workload as WL
    from ubootgl_gb300.simulation import Server
    rng = np.random.default_rng(seed)
    base_flag, base_vx, base_vy = WL.instance(4096, 2048, seed)
    srv = Server(int(budget_gb * (1 << 30)), max_active=max_active, mode=mode,
                 fuse_cells=fuse_cells)
    ids, cells = [], {}
    t0 = time.perf_counter()
    for W in WL.log_uniform_widths(n_sessions, wmin, wmax, seed + 1):
        H = W // 2
        flag = base_flag[:H, :W].copy()
        flag[0, :] = 0.0
        flag[H - 1, :] = 0.0
        u = np.float32(rng.uniform(0.5, 1.5))
        vx = base_vx[:H, :W - 1].copy()
        vy = base_vy[:H - 1, :W].copy()
        vx[:, 0] = u
        vx *= flag[:, :-1] * flag[:, 1:]
        vy *= flag[:-1, :] * flag[1:, :]
        vy[0, :] = 0.0
        sid = srv.open(flag, vx, vy, precision=precision, tol=tol)
        if sid is not None:
            ids.append(sid)
            cells[sid] = W * H
    for r in [srv.submit(s, 1) for s in ids]:
        srv.wait(r)
    info = {"sessions": len(ids), "rejected_sessions": srv.stats()["rejected_sessions"],
            "device_gb": round(srv.stats()["device_bytes_used"] / 2 ** 30, 2),
            "budget_gb": budget_gb, "widths": [wmin, wmax], "max_active": max_active,
            "precision": precision, "mode": mode,
            "solver": ("tolerance, relative residual %g" % tol) if tol else "fixed, 2 V-cycles",
            "open_s": round(time.perf_counter() - t0, 2)}
    return srv, ids, cells, info


def serve_point(srv, ids, cells, rate, duration, seed):
    """Step requests arrive as a Poisson process (`rate` per second for
    `duration` seconds), each for k ~ U[1, 20] device-CFL steps of a session
    drawn uniformly; the run ends when every request has completed.
    Sustained: everything completed within max(0.5 s, duration / 4) of the
    last arrival window."""
    rng = np.random.default_rng(seed)
    base = srv.stats()
    t, arrivals = 0.0, []
    while True:
        t += rng.exponential(1.0 / rate)
        if t > duration:
            break
        arrivals.append((t, ids[int(rng.integers(len(ids)))], int(rng.integers(1, 21))))
    offered = sum(cells[s] * k for _, s, k in arrivals) / duration
    t0 = time.perf_counter()
    reqs = []
    for at, s, k in arrivals:
        d = at - (time.perf_counter() - t0)
        if d > 0:
            time.sleep(d)
        reqs.append(srv.submit(s, k))
    srv.drain()
    wall = time.perf_counter() - t0
    st = srv.stats()
    lat = np.array([srv.wait(r) for r in reqs]) if reqs else np.zeros(1)
    cs = st["cell_steps"] - base["cell_steps"]
    return {"rate_per_s": rate, "duration_s": duration, "requests": len(arrivals),
            "completed": st["completed"] - base["completed"],
            "p50_ms": round(float(np.percentile(lat, 50)), 3),
            "p99_ms": round(float(np.percentile(lat, 99)), 3),
            "max_ms": round(float(lat.max()), 3),
            "value": round(cs / wall / 1e6, 2), "unit": "Mcell-steps/s",
            "offered_mcell_steps_per_s": round(offered / 1e6, 1),
            "sustained": bool(wall <= duration + max(0.5, duration / 4)),
            "fused_steps": st["fused_steps"] - base["fused_steps"],
            "fused_member_steps": st["fused_member_steps"] - base["fused_member_steps"],
            "wall_s": round(wall, 2)}


def serve_arm(L, args, precision, mode, tol, rates, spec_rate=None):
    """One served configuration: sessions opened once, then a sweep of request
    rates (stopping at the first rate that is not sustained), plus the
    specified rate if given.  Reports the highest sustained rate."""
    srv, ids, cells, info = serve_open(L, args.serve_sessions, args.serve_budget_gb,
                                       args.serve_active, precision, mode, tol)
    sweep = []
    for i, rate in enumerate(rates):
        pt = serve_point(srv, ids, cells, rate, args.serve_seconds, seed=100 + i)
        sweep.append(pt)
        if not pt["sustained"]:
            break
    out = dict(info)
    ok = [p for p in sweep if p["sustained"]]
    out["max_sustained_rate_per_s"] = ok[-1]["rate_per_s"] if ok else None
    out["at_max_sustained"] = ok[-1] if ok else None
    out["sweep"] = sweep
    if spec_rate is not None:
        out["at_specified_rate"] = serve_point(srv, ids, cells, spec_rate, args.serve_seconds,
                                               seed=99)
    srv.close()
    return out


def replica_throughput(ms_local, cells, steps, world, pg, device):
    """Replicas only: every rank steps its own grid; the job's time is the
    slowest rank's (MAX over ranks) and the job's throughput counts every
    rank's cells.  Returns (ms, Mcell-steps/s)."""
    ms = float(ms_local)
    if pg is not None and world > 1:
        import torch
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        ms = float(t.item())
    return ms, cells * steps * world / (ms / 1e3) / 1e6


def working_set_bytes(W, H):
    n = W * H
    return n * (4 * 4 + 4 * 2 + 4 * 2 + 1) * 4 // 3 + n * 4 * 2


# Algorithmic bytes per cell of each kernel class (FP32 fields, uint8 flag,
# every input read once and every output written once), per launch; a fused
# launch counts the unfused stages it replaces.  The level-0 smoother
# launches alternate between pre-smoothing (3 red-black sweeps of 13 B/cell
# + residual 13 + restriction 5) and post-smoothing (prolongation 6.25 +
# correction 12 + 3 sweeps of 13); the timed mean covers both, so the
# figure is the mean of the two, 57.125 B/cell.
SMOOTH_L0_PRE = 3 * 13.0 + 13.0 + 5.0
SMOOTH_L0_POST = 6.25 + 12.0 + 3 * 13.0
ALG_BYTES_PER_CELL = {
    "smooth_l0": (SMOOTH_L0_PRE + SMOOTH_L0_POST) / 2,
    "resid_restrict_l0": 9.0 + 1.0,     # read p, f, flag; write rc (1/4 cell)
    "diffuse": 2 * (4 + 4 + 1),         # one sweep of vx and vy
    "advect": 2 * 4 + 1 + 2 * 4,        # read vx, vy, flag; write vx, vy
    "divergence": 8 + 4,
    "gradient": 4 + 1 + 8 + 8,
}


def profiled_traffic(W, H):
    """DRAM bytes (read + write) per level-0 k_mg launch from the committed
    ncu summary of this workload, or None if there is none for this size."""
    fn = os.path.join(ROOT, "profiles", "k_mg_level0_%dx%d.txt" % (W, H))
    try:
        for line in open(fn):
            if line.startswith("dram_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def scale_bench(L, lib, steps, warmup, dev, W=8192, H=4096, ntr=1 << 20, npts=30):
    """The plain FP32 step at scale: one 8192 x 4096 grid (33.5 M cells),
    400 seeded discs of radius 20-60 cells, 2^20 tracers (ring of 30 points,
    draw_tracers_cs.cpp:97) advected every step; `steps` steps of fluid step
    + tracer step, CUDA events on the simulation's stream.  Reports per
    kernel class its mean launch time and algorithmic GB/s, the tracer step
    alone, and the V-cycles per projection (the reference's 2; the tolerance
    solver's count to 1e-6 at this size for comparison)."""
    import ctypes as C
    import torch
    from ubootgl_gb300 import workload as WL
    from ubootgl_gb300.simulation import Simulation, Tracers
    flag = WL.disc_flag(W, H, n_discs=400, r_range=(20.0 * 1024 / W, 60.0 * 1024 / W), seed=2026)
    vx, vy = WL.initial_velocity(flag, seed=2027)
    sim = Simulation(flag, 1.0, 1e-4)
    for n, a in (("vx", vx), ("vy", vy), ("vx_back", vx), ("vy_back", vy)):
        sim.set(n, a)
    pdim = (np.float32(1.0), np.float32(np.float32(1.0) * np.float32(H) / np.float32(W)))
    tr = Tracers(sim, ntr, npts)
    tr.upload(*WL.seed_tracers(flag, ntr, npts, pdim, seed=2028))
    stream = C.c_void_p()
    L.check(lib.ubg_stream(sim._h, C.byref(stream)))
    ext = torch.cuda.ExternalStream(stream.value, device=dev)
    sim.autotune()
    k = 0
    for _ in range(max(3, warmup)):
        sim.step_cfl(0.5)
        tr.step(sim.last_dt(), 7 + k)
        k += 1
    sim.sync()
    e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    e0.record(ext)
    for _ in range(steps):
        sim.step_cfl(0.5)
        tr.step(sim.last_dt(), 7 + k)
        k += 1
    e1.record(ext)
    sim.sync()
    ms = e0.elapsed_time(e1)
    # the tracer step alone
    reps = 20
    dt = sim.last_dt()
    e0.record(ext)
    for i in range(reps):
        tr.step(dt, 100 + i)
    e2.record(ext)
    sim.sync()
    tr_ms = e0.elapsed_time(e2) / reps
    # per kernel class (direct launches with event pairs)
    sim.profile(True)
    sim.profile_reset()
    nprof = 5
    for _ in range(nprof):
        sim.step_cfl(0.5)
    sim.sync()
    classes = sim.profile_classes()
    sim.profile(False)
    peak = measured_peaks().get("hbm_gbs") or 6800.0
    cells = W * H
    kern = {}
    for name, (kms, n) in sorted(classes.items(), key=lambda kv: -kv[1][0]):
        d = {"ms_per_step": round(kms / nprof, 4), "launches_per_step": round(n / nprof, 1),
             "mean_launch_ms": round(kms / n, 5)}
        if name in ALG_BYTES_PER_CELL:
            gbs = ALG_BYTES_PER_CELL[name] * cells / (kms / n / 1e3) / 1e9
            d["alg_gbs"] = round(gbs, 1)
            d["frac_of_measured_hbm"] = round(gbs / peak, 3)
        kern[name] = d
    vcycles = sim.solver_stats()[0]
    tr_alg = 36.0 * ntr
    finite = bool(np.isfinite(sim.get("p")).all())
    pts, st, en, ag = tr.download()
    heads = pts[np.arange(ntr), en % npts]
    inside = float(np.mean((heads[:, 0] >= 0) & (heads[:, 0] <= pdim[0]) &
                           (heads[:, 1] >= 0) & (heads[:, 1] <= pdim[1])))
    del tr
    # the tolerance solver's V-cycles to 1e-6 at this size (3 steps per
    # precision of the coarse levels)
    tol_cycles = {}
    for prec in ("fp32", "fp16"):
        sim.set_options(solver_mode=L.SOLVE_TOLERANCE, tol=1e-6, max_vcycles=200, precision=prec)
        tol_cycles[prec] = []
        for _ in range(3):
            sim.step_cfl(0.5)
            tol_cycles[prec].append(sim.solver_stats())
    sim.close()
    return {"workload": "fluid step %dx%d, 400 discs r 20-60 cells (%.1f %% solid), FP32, "
                        "2 V-cycles, dt=0.5h/max|u|, + %d tracers x %d points"
                        % (W, H, 100.0 * (1.0 - flag.mean()), ntr, npts),
            "steps": steps, "value": round(cells * steps / (ms / 1e3) / 1e6, 2),
            "unit": "Mcell-steps/s (fluid + tracer step)", "ms_per_step": round(ms / steps, 4),
            "tracer_step_ms": round(tr_ms, 4),
            "tracer_alg_gbs": round(tr_alg / (tr_ms / 1e3) / 1e9, 1),
            "tracer_alg_bytes": "36 B per tracer (positions r/w, ring pointers, age) plus the "
                                "velocity / flag gathers",
            "vcycles_per_projection": vcycles, "tolerance_vcycles_to_1e-6":
                {k: [[c, float("%.2e" % r)] for c, r in v] for k, v in tol_cycles.items()},
            "kernels": kern, "fields_finite": finite, "tracer_heads_inside": round(inside, 4)}


def kernel_timing(sim, lib, W, H, reps=30):
    """Per-kernel durations from CUDA events on the simulation's stream,
    recorded around every launch of `reps` further steps (direct launches:
    profiling mode does not use the step graph)."""
    sim.profile(True)
    sim.profile_reset()
    for _ in range(reps):
        sim.step_cfl(0.5)
    sim.sync()
    classes = sim.profile_classes()
    step_ms = sim.profile_read()["step_ms"]
    sim.profile(False)
    peaks = measured_peaks()
    peak = peaks.get("hbm_gbs")
    peak_src = "measured (MEASURED_PEAKS.json hbm_gbs)"
    if not peak:
        peak, peak_src = 6800.0, "fallback"
    cells = W * H
    total = sum(v[0] for v in classes.values()) or 1.0
    detail = {}
    for name, (ms, n) in sorted(classes.items(), key=lambda kv: -kv[1][0]):
        d = {"share": round(ms / total, 4), "launches_per_step": round(n / reps, 2),
             "mean_ms": round(ms / n, 5)}
        if name in ALG_BYTES_PER_CELL:
            gbs = ALG_BYTES_PER_CELL[name] * cells / (ms / n / 1e3) / 1e9
            d["alg_gbs"] = round(gbs, 1)
        detail[name] = d
    dom = "smooth_l0"
    ms_l = classes[dom][0] / classes[dom][1]
    alg = ALG_BYTES_PER_CELL[dom] * cells
    compulsory = 13.0 * cells
    achieved = alg / (ms_l / 1e3) / 1e9
    ach_c = compulsory / (ms_l / 1e3) / 1e9
    roof = {"bound": "hbm", "kernel": "k_mg level 0 (3 red-black sweeps per launch, temporally "
                                      "blocked in shared memory, with the residual + restriction "
                                      "or the prolongation + correction of the level)",
            "alg_bytes_per_cell": ALG_BYTES_PER_CELL[dom],
            "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
            "frac": round(achieved / peak, 3), "peak_source": peak_src,
            "traffic": profiled_traffic(W, H), "launch_ms": round(ms_l, 5),
            "alg_bytes_per_launch": alg,
            "achieved_compulsory": round(ach_c, 1),
            "frac_compulsory": round(ach_c / peak, 3),
            "compulsory_bytes_per_launch": compulsory}
    return {"roofline": roof, "detail": detail, "profiled_step_ms": round(step_ms, 4)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            return json.load(fh)
    except Exception:
        return {}


def end_to_end(sim, L, lib, W, H, steps, barrier, pg, world, dev):
    """Same metric through the public C ABI with host buffers: every step
    copies its velocity state host -> device from pinned memory
    (ubg_io_upload_async), runs (ubg_step_cfl) and copies its resulting
    velocity device -> host (ubg_io_download_async); the copies of one step
    overlap the kernels of its neighbours (two host buffer sets, alternating).
    The timed region ends when the last result is on the host."""
    import torch
    hin = [(L.PinnedArray((H, W - 1)), L.PinnedArray((H - 1, W))) for _ in range(2)]
    hout = [(L.PinnedArray((H, W - 1)), L.PinnedArray((H - 1, W))) for _ in range(2)]
    for a, b in hin:
        a.array[:] = sim.get("vx")
        b.array[:] = sim.get("vy")

    def one(i):
        a, b = hin[i & 1]
        L.check(lib.ubg_io_upload_async(sim._h, L.fptr(a.array), L.fptr(b.array)))
        sim.step_cfl(0.5)
        c, d = hout[i & 1]
        L.check(lib.ubg_io_download_async(sim._h, L.fptr(c.array), L.fptr(d.array)))

    for i in range(3):
        one(i)
    L.check(lib.ubg_io_wait(sim._h))
    barrier()
    t0 = time.perf_counter()
    for i in range(steps):
        one(i)
    L.check(lib.ubg_io_wait(sim._h))
    t1 = time.perf_counter()
    barrier()
    sec = t1 - t0
    if pg:
        t = torch.tensor([sec], device=dev)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        sec = float(t.item())
    val = W * H * steps * world / sec / 1e6
    b_in = 4 * ((W - 1) * H + W * (H - 1))
    return {"value": round(val, 2), "unit": "Mcell-steps/s", "h2d_bytes_per_step": b_in,
            "d2h_bytes_per_step": b_in, "steps": steps,
            "ms_per_step": round(1e3 * sec / steps, 4)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--width", type=int, default=W_DEFAULT)
    ap.add_argument("--height", type=int, default=H_DEFAULT)
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-steps", type=int, default=30)
    ap.add_argument("--e2e-steps", type=int, default=200)
    ap.add_argument("--mode-steps", type=int, default=500,
                    help="timed steps per fixed-mode mixed-precision solver (0: skip)")
    ap.add_argument("--scale-steps", type=int, default=50,
                    help="steps of the 8192x4096 + 2^20 tracers leg (0: skip)")
    ap.add_argument("--tol-steps", type=int, default=10,
                    help="timed steps per tolerance-mode precision (0: skip)")
    ap.add_argument("--tol", type=float, default=1e-6,
                    help="relative residual of the tolerance modes")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--batch", type=int, default=256, help="batched instances (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=50)
    ap.add_argument("--batch-precisions", default="fp32,fp16")
    ap.add_argument("--serve-sessions", type=int, default=512, help="served sessions (0: skip)")
    ap.add_argument("--serve-rate", type=float, default=2000.0)
    ap.add_argument("--serve-seconds", type=float, default=2.0)
    ap.add_argument("--serve-tol", type=float, default=1e-5,
                    help="relative residual of the served tolerance-mode arms")
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--serve-active", type=int, default=32)
    ap.add_argument("--serve-precisions", default="fp32,fp16")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
