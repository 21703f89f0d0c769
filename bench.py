"""Benchmark: cell-updates/s of the KKS step on one GB300.

Workload (the single-grid configuration): 2D 4096 x 4096 grid, dx = 5 nm,
16 enriched stripes and 64 particles at seeded positions, zero-flux
boundaries, 5-point Laplacian, explicit Euler at the stability-limited dt,
Philox nucleation every 100 steps (seed 42, the reference's physical
nucleation parameters).  One benchmark step = 100 time steps + the
nucleation call of that interval.  The headline `value` is the FP32
precision form with fields resident in HBM; `fp64` is the plain FP64 fused
step on the same workload; `e2e` goes through the C ABI with host buffers
(upload of the four FP64 fields, 100 steps, read-out) every step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank runs an independent replica on its own GPU
(replicas only: the grids do not exchange data), so scaling is weak.
"""
import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "phasefield-precipitate-aging_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "cell-updates/s FP32 vs plain FP64 on one GB300 at stated error; p50/p99 latency"
N_SIDE = 4096
STEPS_PER_BENCH_STEP = 100
NUC_LAUNCHES = 3  # kernels per nucleation call: decide, FP64 decisions, paint
NUC = dict(sigma=(0.13, 0.13), unit_a=0.352e-9)
WORKLOAD = (f"single 2D grid {N_SIDE}x{N_SIDE}, dx=5nm, 16 enriched stripes + 64 particles "
            f"(seeded), zero-flux, 5-point Laplacian, KKS-stable dt, Philox nucleation every "
            f"{STEPS_PER_BENCH_STEP} steps (seed 42); one bench step = {STEPS_PER_BENCH_STEP} "
            f"time steps + 1 nucleation call")


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the sampler is running before the timed region starts (bounded wait)
            t0 = time.time()
            while not self.rows and time.time() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except OSError:
            self.proc = None
        self.t_begin = time.time()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append((time.time(), [c.strip() for c in line.split(",")]))

    def __exit__(self, *a):
        self.t_end = time.time()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        """Samples taken inside the timed region (all samples if none were)."""
        end = getattr(self, "t_end", time.time())
        rows = [r for t, r in self.rows if self.t_begin <= t <= end] or [r for _, r in self.rows]
        sm = [float(r[1]) for r in rows if len(r) > 8 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if len(r) > 8 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows if len(r) > 8
                          for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def spin_up(grid, seconds=1.5):
    """Untimed steps until `seconds` have passed, after the warm-up steps, so
    that the timed region starts at steady clocks (a first run on a GPU fresh
    from idle sampled 1987 MHz, the next one 2070)."""
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        grid.run(STEPS_PER_BENCH_STEP)
        grid.sync()


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_value(kernel, key):
    """A `key: value` line of the committed ncu summary of `kernel`, if any."""
    path = os.path.join(ROOT, "profiles", f"{kernel}.txt")
    try:
        for line in open(path):
            if line.startswith(key + ":"):
                return float(line.split(":", 1)[1])
    except OSError:
        pass
    return None


def profiled_traffic(kernel):
    """dram read+write bytes per launch from the committed ncu summary, if any."""
    return profiled_value(kernel, "traffic_bytes_per_launch")


def cpu_model():
    """The host CPU's model name (lscpu / /proc/cpuinfo), for the baseline's record."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.machine()


def cpu_baseline(fields, params, steps, fast=True):
    """The CPU oracle (the reference's step semantics, reference host flags,
    OpenMP on every host core) on the same workload."""
    import oracle as O
    O.build(fast=True)
    lib = O.Oracle(os.path.join(ROOT, "oracle", "liboracle_fast.so" if fast else "liboracle.so"))
    prm = O.OrcParams.from_dict(params)
    t0 = time.perf_counter()
    lib.run2d(fields, prm, steps)
    return time.perf_counter() - t0


def reference_gpu_baseline(fields, steps=10):
    """The reference's own CUDA step (src/discretization.cu's kernels, built
    from source for sm_103a into oracle/_ref/ref_step.cubin and launched in its
    order and shapes by oracle/ref_gpu.py, nucleation off) on the same grid:
    a baseline timed beside ours, never the measured path."""
    import ref_gpu
    if not os.path.exists(ref_gpu.CUBIN):
        return {"unavailable": "oracle/_ref/ref_step.cubin not built "
                               "(make -C oracle ref-gpu needs the reference checkout)"}
    import oracle as O
    drv = ref_gpu.Driver(ref_gpu.CUBIN)
    try:
        t = ref_gpu.time_reference(drv, fields, O.model_params(), steps)
    finally:
        drv.close()
    ny, nx = fields[0].shape
    return {"value": (nx - 2) * (ny - 2) / t, "unit": "cell-updates/s", "ms_per_step": 1e3 * t,
            "kind": "the reference's own CUDA kernels (src/discretization.cu, "
                    "src/parabola625.cu), FP64, launched in src/main.cpp's order on one stream "
                    "without its host waits",
            "sample": f"{steps} time steps of the same grid after 2 warm-up steps, nucleation off"}


def run_reference(args, ws, rank):
    """--impl reference: the CPU path timed on this host's cores."""
    if rank != 0:
        return
    from pfa_gb300 import ic, lib as pl
    fields = ic.config2(n=N_SIDE)
    import oracle as O
    params = O.model_params().as_dict()
    per = 2  # time steps per bench step of this arm (a bounded sample)
    for _ in range(args.warmup):
        cpu_baseline(fields, params, per)
    t = 0.0
    for _ in range(args.steps):
        t += cpu_baseline(fields, params, per)
    cells = N_SIDE * N_SIDE
    value = cells * per * args.steps / t
    cores = os.cpu_count()
    line = {"metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "sample": f"{per} time steps of the full grid per step"},
            "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": cores,
                             "kind": "port", "cpu": cpu_model(),
                             "sample": f"{per} FP64 time steps of the {N_SIDE}^2 grid per step"},
            "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


BATCH_COUNT = 64
BATCH_WORKLOAD = (f"batch of {BATCH_COUNT} 2D grids, sides log-uniform in [128, 2048] (seed 3), "
                  f"per-grid matrix / enrichment compositions from the alloy ranges, dx=5nm, "
                  f"zero-flux, 5-point Laplacian, KKS-stable dt; one launch per time step over "
                  f"all grids; one bench step = {STEPS_PER_BENCH_STEP} time steps")
GRID3D_SIDE = 512
GRID3D_WORKLOAD = (f"single 3D grid {GRID3D_SIDE}^3, dx=5nm, enriched slab 64 thick + 32 spheres "
                   f"R=6 (seeded), zero-flux, 7-point Laplacian, KKS-stable dt, Philox nucleation "
                   f"every {STEPS_PER_BENCH_STEP} steps (seed 42); one bench step = "
                   f"{STEPS_PER_BENCH_STEP} time steps + 1 nucleation call")


def _line(args, ws, metric_value, t, workload, config, **extra):
    line = {"metric": METRIC, "value": metric_value, "unit": "cell-updates/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "config": dict({"workload": workload}, **config)}
    line.update(extra)
    return line


def bench_batch(args, ws, rank, local, barrier, max_over_ranks, pl, ic):
    """The many-grids workload: all grids resident in one batch arena."""
    sides = ic.batch_sides(BATCH_COUNT, seed=3 + 100 * rank)
    fields = [ic.batch_grid(s, seed=1000 + k) for k, s in enumerate(sides)]
    cells = sum(s * s for s in sides)
    params = pl.model_params()
    arena = sum(pl.Batch.footprint(f[0].shape) for f in fields) + (1 << 20)
    b = pl.Batch(params, arena)
    slots = [b.add(f) for f in fields]
    tuned_ms = b.tune(reps=5)
    launch = b.launch()
    b.run(args.warmup * STEPS_PER_BENCH_STEP)
    b.sync()
    barrier()
    with ClockSampler(local) as clk:
        ms = b.run_timed(args.steps * STEPS_PER_BENCH_STEP)
    barrier()
    t = max_over_ranks(ms / 1e3)
    value = ws * cells * STEPS_PER_BENCH_STEP * args.steps / t
    if args.only == "value":
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "cell-updates/s",
                              "ms_per_step": 1e3 * t / args.steps, "partial": "value only"}))
        b.close()
        return
    kms = b.run_timed(400) / 400
    peak, peak_kind = measured_peak_hbm()
    achieved = 48 * cells / (kms / 1e3) / 1e9
    # one-at-a-time FP64 loop over the same grids (the single-grid FP64 step)
    n64 = 10
    t64 = 0.0
    for f in fields:
        g = pl.Grid2D(f, params, precision="fp64")
        g.run(2)
        t64 += g.run_timed(n64) / 1e3
        g.close()
    fp64_value = cells * n64 / t64
    # stated error on the three largest grids after 400 steps
    big = sorted(range(len(sides)), key=lambda k: -sides[k])[:3]
    eb = pl.Batch(params, arena)
    es = {k: eb.add(fields[k]) for k in big}
    eb.run(400)
    err = [0.0] * 4
    for k in big:
        g = pl.Grid2D(fields[k], params, precision="fp64")
        g.run(400)
        for i, (x, y) in enumerate(zip(eb.read(es[k]), g.read())):
            err[i] = max(err[i], float(np.max(np.abs(x[1:-1, 1:-1] - y[1:-1, 1:-1]))))
        g.close()
    eb.close()
    b.close()
    # e2e: every bench step adds all grids from host memory, runs, reads them back
    import torch
    host = [[torch.from_numpy(a).pin_memory().numpy() for a in f] for f in fields]
    outs = [[torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy() for a in f]
            for f in fields]
    be = pl.Batch(params, arena)
    be.set_launch(launch["rows"], launch["persistent"])

    def e2e_step():
        ss = [be.add(h) for h in host]
        be.run(STEPS_PER_BENCH_STEP)
        for s, o in zip(ss, outs):
            be.read(s, o)
        for s in ss:
            be.remove(s)

    e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    barrier()
    te_serial = max_over_ranks(time.perf_counter() - t0)
    # pipelined: bench steps are independent jobs on two alternating batches.
    # Job k's adds (asynchronous) and steps are enqueued on one batch, then job
    # k-1's grids are read back and removed from the other while job k computes.
    bp = [be, pl.Batch(params, arena)]
    bp[1].set_launch(launch["rows"], launch["persistent"])
    ss = [bp[1].add(h) for h in host]  # warm the second batch's graphs
    bp[1].run(STEPS_PER_BENCH_STEP)
    for s_, o in zip(ss, outs):
        bp[1].read(s_, o)
    for s_ in ss:
        bp[1].remove(s_)

    def drain(job):
        y, ys = job
        for s_, o in zip(ys, outs):
            y.read(s_, o)
        for s_ in ys:
            y.remove(s_)

    barrier()
    t0 = time.perf_counter()
    pending = None
    for k in range(args.steps):
        x = bp[k % 2]
        xs = [x.add(h) for h in host]
        x.run(STEPS_PER_BENCH_STEP)
        if pending:
            drain(pending)
        pending = (x, xs)
    drain(pending)
    barrier()
    te = max_over_ranks(time.perf_counter() - t0)
    for x in bp:
        x.close()
    io = sum(4 * f[0].size * 8 for f in fields)
    if rank == 0:
        line = _line(args, ws, value, t, BATCH_WORKLOAD,
                     {"grids": BATCH_COUNT, "cells": cells, "precision": "fp32",
                      "launch": launch, "tuned_ms_per_step": tuned_ms,
                      "l2": "inputs larger than L2 (FP32 state 48 B/cell, 2.3 GB)",
                      "parallelism": f"replicas x{ws}"},
                     fp64={"value": fp64_value, "unit": "cell-updates/s",
                           "how": "one grid at a time, single-grid FP64 step",
                           "speedup_fp32_over_fp64": value / ws / fp64_value},
                     max_field_error={"vs": "fp64 GPU step", "steps": 400,
                                      "grids": [sides[k] for k in big],
                                      "x_Cr": err[0], "x_Nb": err[1], "phi_delta": err[2],
                                      "phi_laves": err[3]},
                     roofline={"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                               "frac": achieved / peak, "traffic": profiled_traffic("batch_f32_64"),
                               "kernel": "k_batch_f32", "bytes_per_cell": 48, "kernel_ms": kms,
                               "peak_kind": peak_kind},
                     cpu_baseline=None,
                     e2e={"value": ws * cells * STEPS_PER_BENCH_STEP * args.steps / te,
                          "unit": "cell-updates/s", "h2d_bytes_per_step": io,
                          "d2h_bytes_per_step": io,
                          "mode": "independent jobs on two alternating batches: job k's adds "
                                  "and steps are enqueued, then job k-1's grids are read back "
                                  "and removed while job k computes",
                          "serial": {"value": ws * cells * STEPS_PER_BENCH_STEP * args.steps
                                     / te_serial, "unit": "cell-updates/s",
                                     "mode": "one batch: add all, run, read all, remove all"}},
                     gpu_launches=args.steps * STEPS_PER_BENCH_STEP,
                     clocks=clk.summary())
        print(json.dumps(line))


def bench_error(args, ws, rank, local, barrier, max_over_ranks, pl, ic):
    """Stated error at the configurations' full step counts: the FP32 form
    against the FP64 step on the 4096^2 grid (10000 steps, nucleation every
    100 steps with the same seed in both), the 512^3 grid (2000 steps) and
    the batch of 64 uneven grids (5000 steps, each grid against its own FP64
    run).
    Prints one JSON line; `value` is the FP32 rate of the 2D run."""
    if rank != 0:
        return
    out = {}
    p2 = pl.model_params()
    f2 = ic.config2(n=N_SIDE)
    n2 = args.steps if args.steps > 10 else 10000
    runs = {}
    for prec in ("fp32", "fp64"):
        g = pl.Grid2D(f2, p2, precision=prec)
        g.set_nucleation(seed=42, geometry=pl.NUC_REFERENCE_GEOMETRY, interval=100,
                         sigma=NUC["sigma"], unit_a=NUC["unit_a"], d=(p2["dx"],) * 3,
                         dt_nuc=100 * p2["dt"])
        ms = g.run_timed(n2)
        runs[prec] = (g.read(), ms)
        g.close()
    err = [float(np.max(np.abs(a[1:-1, 1:-1] - b[1:-1, 1:-1])))
           for a, b in zip(runs["fp32"][0], runs["fp64"][0])]
    out["grid4096"] = {"steps": n2, "x_Cr": err[0], "x_Nb": err[1], "phi_delta": err[2],
                       "phi_laves": err[3], "fp32_ms": runs["fp32"][1],
                       "fp64_ms": runs["fp64"][1]}
    side = args.side or GRID3D_SIDE
    n3 = 2000
    p3 = pl.model_params(dim=3)
    f3 = ic.grid3d(side, side, side, seed=4, slab=64, n_particles=32, radius=6.0)
    res3 = {}
    for prec in ("fp32", "fp64"):
        g = pl.Grid3D(f3, p3, precision=prec)
        g.set_nucleation(seed=42, interval=100, sigma=NUC["sigma"], unit_a=NUC["unit_a"],
                         d=(p3["dx"],) * 3, dt_nuc=100 * p3["dt"])
        res3[prec] = (g.run_timed(n3), g.read())
        g.close()
    err3 = [float(np.max(np.abs(a[1:-1, 1:-1, 1:-1] - b[1:-1, 1:-1, 1:-1])))
            for a, b in zip(res3["fp32"][1], res3["fp64"][1])]
    out["grid3d"] = {"side": side, "steps": n3, "x_Cr": err3[0], "x_Nb": err3[1],
                     "phi_delta": err3[2], "phi_laves": err3[3], "fp32_ms": res3["fp32"][0],
                     "fp64_ms": res3["fp64"][0]}
    # the batch of 64 uneven grids, 5000 steps in the batched FP32 form, each
    # grid against its own FP64 run
    nb = 5000
    sides = ic.batch_sides(BATCH_COUNT, seed=3)
    fields = [ic.batch_grid(sd, seed=1000 + k) for k, sd in enumerate(sides)]
    arena = sum(pl.Batch.footprint(f[0].shape) for f in fields) + (1 << 20)
    b = pl.Batch(p2, arena)
    slots = [b.add(f) for f in fields]
    tb = b.run_timed(nb)
    errb = [0.0] * 4
    t64 = 0.0
    for f, sl in zip(fields, slots):
        g = pl.Grid2D(f, p2, precision="fp64")
        t64 += g.run_timed(nb)
        for i, (x, y) in enumerate(zip(b.read(sl), g.read())):
            errb[i] = max(errb[i], float(np.max(np.abs(x[1:-1, 1:-1] - y[1:-1, 1:-1]))))
        g.close()
    b.close()
    out["batch64"] = {"grids": BATCH_COUNT, "steps": nb, "x_Cr": errb[0], "x_Nb": errb[1],
                      "phi_delta": errb[2], "phi_laves": errb[3], "fp32_ms": tb,
                      "fp64_ms_one_at_a_time": t64}
    value = N_SIDE * N_SIDE * n2 / (runs["fp32"][1] / 1e3)
    args.steps = 1
    print(json.dumps(_line(args, ws, value, runs["fp32"][1] / 1e3,
                           "stated-error study: FP32 form vs FP64 at full step counts",
                           {"bound": 1e-5}, max_field_error=out)))


def bench_grid3d(args, ws, rank, local, barrier, max_over_ranks, pl, ic):
    """The 3D workload, FP32 form vs the FP64 step."""
    n = args.side or GRID3D_SIDE
    fields = ic.grid3d(n, n, n, seed=4 + rank, slab=64, n_particles=32, radius=6.0)
    params = pl.model_params(dim=3)
    cells = n ** 3
    g = pl.Grid3D(fields, params, precision="fp32")
    g.set_nucleation(seed=42, interval=STEPS_PER_BENCH_STEP, sigma=NUC["sigma"],
                     unit_a=NUC["unit_a"], d=(params["dx"],) * 3,
                     dt_nuc=STEPS_PER_BENCH_STEP * params["dt"])
    g.run(args.warmup * STEPS_PER_BENCH_STEP)
    barrier()
    with ClockSampler(local) as clk:
        ms = g.run_timed(args.steps * STEPS_PER_BENCH_STEP)
    barrier()
    t = max_over_ranks(ms / 1e3)
    value = ws * cells * STEPS_PER_BENCH_STEP * args.steps / t
    if args.only == "value":
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "cell-updates/s",
                              "ms_per_step": 1e3 * t / args.steps, "partial": "value only"}))
        g.close()
        return
    g.set_nucleation(interval=0)  # the step kernel alone for the roofline
    g.run(2)
    kms = g.run_timed(50) / 50
    # e2e: every bench step uploads the four FP64 fields from page-locked host
    # memory, runs 100 steps with nucleation and reads the fields back
    import torch
    host_in = [torch.from_numpy(a).pin_memory().numpy() for a in fields]
    host_out = [torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
                for a in fields]
    g.set_nucleation(seed=42, interval=STEPS_PER_BENCH_STEP, sigma=NUC["sigma"],
                     unit_a=NUC["unit_a"], d=(params["dx"],) * 3,
                     dt_nuc=STEPS_PER_BENCH_STEP * params["dt"])

    def e2e_step():
        g.upload(host_in)
        g.run(STEPS_PER_BENCH_STEP)
        g.read(host_out)

    e2e_step()
    barrier()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(e2e_steps):
        e2e_step()
    barrier()
    te_serial = max_over_ranks(time.perf_counter() - t0)
    # pipelined: independent jobs on two alternating handles, job k+1's upload
    # and job k-1's read-out overlapping job k's steps (every job's copies
    # inside the timed region)
    g2 = pl.Grid3D(fields, params, precision="fp32")
    g2.set_nucleation(seed=42, interval=STEPS_PER_BENCH_STEP, sigma=NUC["sigma"],
                      unit_a=NUC["unit_a"], d=(params["dx"],) * 3,
                      dt_nuc=STEPS_PER_BENCH_STEP * params["dt"])
    g2.upload(host_in)
    g2.run(STEPS_PER_BENCH_STEP)
    g2.read(host_out)
    host_out2 = [host_out, [torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
                            for a in fields]]
    gp = [g, g2]
    pipe_steps = max(2, min(args.steps, 8))
    barrier()
    t0 = time.perf_counter()
    gp[0].upload(host_in, wait=False)
    for k in range(pipe_steps):
        d, o = gp[k % 2], gp[(k + 1) % 2]
        if k + 1 < pipe_steps:
            o.upload(host_in, wait=False)
        d.run(STEPS_PER_BENCH_STEP)
        d.read(host_out2[k % 2], wait=False)
    for x in gp:
        x.sync()
    barrier()
    te = max_over_ranks(time.perf_counter() - t0)
    g.close()
    g2.close()
    io_bytes = 4 * fields[0].size * 8
    g64 = pl.Grid3D(fields, params, precision="fp64")
    g64.run(2)
    ms64 = g64.run_timed(6) / 6
    g64.close()
    peak, peak_kind = measured_peak_hbm()
    achieved = 48 * cells / (kms / 1e3) / 1e9
    if rank == 0:
        workload = GRID3D_WORKLOAD if n == GRID3D_SIDE else GRID3D_WORKLOAD.replace(
            f"{GRID3D_SIDE}^3", f"{n}^3")
        line = _line(args, ws, value, t, workload,
                     {"nx": n, "ny": n, "nz": n, "precision": "fp32",
                      "l2": "inputs larger than L2 (FP32 state 6.4 GB)",
                      "parallelism": f"replicas x{ws}"},
                     fp64={"value": cells / (ms64 / 1e3), "unit": "cell-updates/s",
                           "ms_per_step": ms64,
                           "speedup_fp32_over_fp64": value / ws / (cells / (ms64 / 1e3))},
                     roofline={"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                               "frac": achieved / peak, "traffic": profiled_traffic("step3d_f32_512"),
                               "kernel": "k_stream3d_f32", "bytes_per_cell": 48, "kernel_ms": kms,
                               "peak_kind": peak_kind},
                     cpu_baseline=None,
                     e2e={"value": ws * cells * STEPS_PER_BENCH_STEP * pipe_steps / te,
                          "unit": "cell-updates/s", "h2d_bytes_per_step": io_bytes,
                          "d2h_bytes_per_step": io_bytes, "steps": pipe_steps,
                          "mode": "independent jobs on two alternating handles: job k+1's "
                                  "upload and job k-1's read-out (pfa3d_upload_async / "
                                  "pfa3d_read_async, page-locked buffers) overlap job k's steps",
                          "serial": {"value": ws * cells * STEPS_PER_BENCH_STEP * e2e_steps
                                     / te_serial, "unit": "cell-updates/s", "steps": e2e_steps,
                                     "mode": "one handle: upload, run, read back"}},
                     gpu_launches=args.steps * (STEPS_PER_BENCH_STEP + NUC_LAUNCHES),
                     clocks=clk.summary())
        print(json.dumps(line))


SERVE_COUNT = 24
SERVE_WORKLOAD = (f"serving trace of {SERVE_COUNT} requests (seed 5): Poisson arrivals 20/s, size "
                  f"uniform over {{256^2, 1024^2, 4096^2, 128^3, 256^3}}, steps uniform in "
                  f"[2000, 20000], compositions from the alloy ranges; FP32 form, continuous "
                  f"batching (2D grids in one batch, 3D grids on their own streams), FIFO "
                  f"admission by device footprint; one bench step = the whole trace")


def bench_serve(args, ws, rank, local, barrier, max_over_ranks, pl, ic):
    """Latency and aggregate throughput of the serving layer on a request trace."""
    from pfa_gb300.serve import GpuBackend, Request, Server, fifo_latencies, latency_stats
    args.steps = 1  # the whole trace is the one timed step
    trace = ic.serve_trace(SERVE_COUNT, seed=5 + 100 * rank)
    reqs = [Request(t["rid"], ic.serve_fields(t), t["steps"], t["arrival"]) for t in trace]
    work = sum(r.cells * r.steps for r in reqs)
    p2, p3 = pl.model_params(), pl.model_params(dim=3)
    arena = 48 << 30
    budget3 = 48 << 30

    def serve_once(realtime=True, requests=reqs):
        be = GpuBackend(pl, p2, p3, arena, budget3)
        srv = Server(be, tick_steps=STEPS_PER_BENCH_STEP)
        done = srv.run_trace(requests, realtime=realtime)
        be.close()
        return done, srv

    # warm-up: the same trace scaled down to 300 steps per request
    warm = [Request(r.rid, r.fields, 300, 0.0) for r in reqs[:8]]
    for _ in range(max(1, args.warmup // 3)):
        be = GpuBackend(pl, p2, p3, arena, budget3)
        Server(be, tick_steps=STEPS_PER_BENCH_STEP).run_trace(warm, realtime=False)
        be.close()
    barrier()
    with ClockSampler(local) as clk:
        done, srv = serve_once()
    barrier()
    span = max(r.finished for r in done) - min(r.req.arrival for r in done)
    t = max_over_ranks(span)
    value = ws * work / t
    stats = latency_stats(done)
    # the same trace with every initial condition built on the device from its
    # recipe (no host fields, no upload)
    rreqs = [Request(t_["rid"], None, t_["steps"], t_["arrival"], recipe=ic.serve_recipe(t_))
             for t_ in trace]
    barrier()
    done_r, _ = serve_once(requests=rreqs)
    barrier()
    span_r = max_over_ranks(max(r.finished for r in done_r) - min(r.req.arrival for r in done_r))
    stats_r = latency_stats(done_r)
    # one-at-a-time FP64: each request's FP64 step time measured on a sample,
    # queueing in arrival order computed from those service times
    service = []
    for r in reqs:
        t0 = time.perf_counter()
        if r.dim == 2:
            g = pl.Grid2D(r.fields, p2, precision="fp64")
        else:
            g = pl.Grid3D(r.fields, p3, precision="fp64")
        g.run(2)
        sample = 10 if r.cells > 4e6 else 40
        ms = g.run_timed(sample) / sample
        g.read()
        g.close()
        setup = time.perf_counter() - t0 - 1e-3 * ms * (sample + 2)
        service.append(max(0.0, setup) + 1e-3 * ms * r.steps)
    arr = [r.arrival for r in reqs]
    lat64 = fifo_latencies(arr, service)
    span64 = max(a + l for a, l in zip(arr, lat64)) - min(arr)
    if rank == 0:
        line = _line(args, ws, value, t, SERVE_WORKLOAD,
                     {"requests": SERVE_COUNT, "cell_updates": work, "precision": "fp32",
                      "tick_steps": STEPS_PER_BENCH_STEP, "ticks": srv.ticks,
                      "budget_bytes": {"2d_arena": arena, "3d": budget3},
                      "l2": "inputs larger than L2",
                      "parallelism": f"replicas x{ws}"},
                     latency=dict(stats, unit="s", what="arrival to result read back"),
                     fp64={"value": work / span64, "unit": "cell-updates/s",
                           "how": "one request at a time in arrival order, FP64 step; service "
                                  "times from measured per-request step times",
                           "p50_s": float(np.percentile(lat64, 50)),
                           "p99_s": float(np.percentile(lat64, 99))},
                     cpu_baseline=None,
                     e2e={"value": value, "unit": "cell-updates/s",
                          "h2d_bytes_per_step": sum(4 * r.fields[0].size * 8 for r in reqs),
                          "d2h_bytes_per_step": sum(4 * r.fields[0].size * 8 for r in reqs)},
                     ic_on_device={"value": ws * work / span_r, "unit": "cell-updates/s",
                                   "p50_s": stats_r["p50_s"], "p99_s": stats_r["p99_s"],
                                   "how": "the same trace, initial conditions built on the "
                                          "device from recipes (pfa_ic_recipe), no upload"},
                     gpu_launches=srv.step_launches + 2 * len(reqs),
                     clocks=clk.summary())
        print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp32k"])
    ap.add_argument("--workload", default="grid4096",
                    choices=["grid4096", "batch64", "grid3d512", "serve", "error"],
                    help="grid4096: the headline single-grid workload; batch64 / grid3d512: "
                         "the many-grids and 3D workloads")
    ap.add_argument("--side", type=int, default=0,
                    help="grid3d512 only: another cube side (smaller profiler captures)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--only", default="all", choices=["all", "value"],
                    help="'value': only the device-resident timed run (for profiler captures)")
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.warmup < 3:
        args.warmup = 3

    if args.impl == "reference":
        if ws > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
        run_reference(args, ws, rank)
        return

    import torch
    from pfa_gb300 import build, ic, lib as pl
    build.build()
    L = pl.load()
    pl.check(L.pfa_set_device(local), "pfa_set_device")
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    fields = ic.config2(seed=2 + rank, n=N_SIDE)
    params = pl.model_params()
    cells = N_SIDE * N_SIDE
    nuc_kw = dict(seed=42, geometry=pl.NUC_REFERENCE_GEOMETRY, interval=STEPS_PER_BENCH_STEP,
                  sigma=NUC["sigma"], unit_a=NUC["unit_a"], d=(params["dx"],) * 3,
                  dt_nuc=STEPS_PER_BENCH_STEP * params["dt"])

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    if args.workload != "grid4096":
        fn = {"batch64": bench_batch, "grid3d512": bench_grid3d, "serve": bench_serve,
              "error": bench_error}[args.workload]
        fn(args, ws, rank, local, barrier, max_over_ranks, pl, ic)
        if dist is not None:
            dist.destroy_process_group()
        return

    # ---- device-resident FP32 precision form (headline value) ----
    g = pl.Grid2D(fields, params, precision=args.precision)
    g.set_nucleation(**nuc_kw)
    g.run(args.warmup * STEPS_PER_BENCH_STEP)
    g.sync()
    spin_up(g)
    barrier()
    with ClockSampler(local) as clk:
        ms = g.run_timed(args.steps * STEPS_PER_BENCH_STEP)
    barrier()
    t = max_over_ranks(ms / 1e3)
    value = ws * cells * STEPS_PER_BENCH_STEP * args.steps / t
    if args.only == "value":
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "cell-updates/s",
                              "ms_per_step": 1e3 * t / args.steps, "partial": "value only"}))
        g.close()
        return

    # kernel-only time of the step kernel (no nucleation): average launch
    g2 = pl.Grid2D(fields, params, precision=args.precision)
    g2.run(200)
    kms = g2.run_timed(400) / 400
    g2.close()
    bytes_per_cell = 48 if args.precision == "fp32" else 64
    peak, peak_kind = measured_peak_hbm()
    achieved = bytes_per_cell * cells / (kms / 1e3) / 1e9
    kname = "step2d_f32_4096" if args.precision == "fp32" else "step2d_f32k_4096"
    traffic = profiled_traffic(kname)

    # ---- plain FP64 fused step on the same workload ----
    g64 = pl.Grid2D(fields, params, precision="fp64")
    g64.set_nucleation(**nuc_kw)
    g64.run(STEPS_PER_BENCH_STEP)
    ms64 = g64.run_timed(STEPS_PER_BENCH_STEP)
    fp64_value = cells * STEPS_PER_BENCH_STEP / (ms64 / 1e3)

    # ---- stated error: FP32 form vs FP64 after the same 400 steps ----
    ga = pl.Grid2D(fields, params, precision=args.precision)
    gb = pl.Grid2D(fields, params, precision="fp64")
    ga.run(400)
    gb.run(400)
    fa, fb = ga.read(), gb.read()
    err = [float(np.max(np.abs(a[1:-1, 1:-1] - b[1:-1, 1:-1]))) for a, b in zip(fa, fb)]
    ga.close()
    gb.close()
    g64.close()

    # ---- e2e through the C ABI with host buffers ----
    host_in = []
    host_out = []
    for a in fields:
        h = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
        h[...] = a
        host_in.append(h)
        host_out.append(torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy())
    ge = pl.Grid2D(fields, params, precision=args.precision)
    ge.set_nucleation(**nuc_kw)
    for _ in range(1):
        ge.upload(host_in)
        ge.run(STEPS_PER_BENCH_STEP)
        ge.read(host_out)
    # serial: each bench step uploads, runs and reads back on one handle
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ge.upload(host_in)
        ge.run(STEPS_PER_BENCH_STEP)
        ge.read(host_out)
    barrier()
    te_serial = max_over_ranks(time.perf_counter() - t0)
    # pipelined: bench steps are independent jobs on two alternating handles;
    # job k+1's upload and job k-1's read-out (asynchronous entry points,
    # page-locked buffers) overlap job k's steps.  Every job's copies are
    # inside the timed region.
    host_out2 = [[torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
                  for a in fields] for _ in range(2)]
    gp = [ge, pl.Grid2D(fields, params, precision=args.precision)]
    gp[1].set_nucleation(**nuc_kw)
    for x in gp:  # warm the second handle's graphs and transfer events
        x.upload(host_in)
        x.run(STEPS_PER_BENCH_STEP)
        x.read(host_out)
    barrier()
    t0 = time.perf_counter()
    gp[0].upload(host_in, wait=False)
    for k in range(args.steps):
        d, o = gp[k % 2], gp[(k + 1) % 2]
        if k + 1 < args.steps:
            o.upload(host_in, wait=False)
        d.run(STEPS_PER_BENCH_STEP)
        d.read(host_out2[k % 2], wait=False)
    for x in gp:
        x.sync()
    barrier()
    te = max_over_ranks(time.perf_counter() - t0)
    for x in gp:
        x.close()
    e2e_value = ws * cells * STEPS_PER_BENCH_STEP * args.steps / te
    e2e_serial = ws * cells * STEPS_PER_BENCH_STEP * args.steps / te_serial
    io_bytes = 4 * fields[0].size * 8

    line = None
    if rank == 0:
        cpu = None
        if not args.no_cpu:
            sample_steps = 3
            tc = cpu_baseline(fields, pl.model_params(), sample_steps)
            cpu = {"value": cells * sample_steps / tc, "unit": "cell-updates/s",
                   "cores": os.cpu_count(), "kind": "port", "cpu": cpu_model(),
                   "sample": f"{sample_steps} FP64 time steps of the {N_SIDE}^2 grid, "
                             f"OpenMP, reference host flags"}
        ref_gpu = reference_gpu_baseline(fields)
        if "value" in ref_gpu:
            ref_gpu["speedup_fp32_over_reference_gpu"] = value / ws / ref_gpu["value"]
        line = {
            "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "nx": N_SIDE, "ny": N_SIDE,
                       "precision": args.precision, "dt": params["dt"],
                       "l2": "inputs larger than L2 (FP32 state 6 x 67 MB)",
                       "parallelism": f"replicas x{ws}"},
            "fp64": {"value": fp64_value, "unit": "cell-updates/s",
                     "ms_per_step": ms64, "speedup_fp32_over_fp64": value / ws / fp64_value,
                     "fp64_flops_per_cell": profiled_value("step2d_f64_4096",
                                                           "fp64_flops_per_cell"),
                     "bound": "FP64 pipe"},
            "max_field_error": {"vs": "fp64 GPU step (pinned to the reference at 1e-12)",
                                "steps": 400, "x_Cr": err[0], "x_Nb": err[1],
                                "phi_delta": err[2], "phi_laves": err[3]},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "k_stream_f32", "bytes_per_cell": bytes_per_cell,
                         "kernel_ms": kms, "peak_kind": peak_kind,
                         # secondary: the 32 B/cell floor of the four fields alone
                         "no_compensation_floor": {
                             "bytes_per_cell": 32,
                             "achieved": 32 * cells / (kms / 1e3) / 1e9,
                             "frac": 32 * cells / (kms / 1e3) / 1e9 / peak}},
            "cpu_baseline": cpu,
            "reference_gpu": ref_gpu,
            "e2e": {"value": e2e_value, "unit": "cell-updates/s", "h2d_bytes_per_step": io_bytes,
                    "d2h_bytes_per_step": io_bytes,
                    "mode": "independent jobs on two alternating CudaData handles: job k+1's "
                            "upload and job k-1's read-out (pfa_upload_fields_async / "
                            "pfa_read_out_result_async, page-locked buffers) overlap job k's "
                            "steps",
                    "serial": {"value": e2e_serial, "unit": "cell-updates/s",
                               "mode": "one handle: upload, run, read back, one after another"}},
            "gpu_launches": args.steps * (STEPS_PER_BENCH_STEP + NUC_LAUNCHES),
            "clocks": clk.summary(),
        }
        print(json.dumps(line))
    g.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
