"""Benchmark: cell-updates/s of the KKS step on one GB300.

One default run prints one JSON line covering every workload:

* headline (`value`, `e2e`, `roofline`, `fp64`, `cpu_baseline`,
  `reference_gpu`): the single-grid workload, a 2D 4096 x 4096 grid, dx = 5
  nm, the 256^2 grid's recipe (4 particles R = 8) with 16 enriched stripes at
  seeded positions, zero-flux boundaries, 5-point Laplacian, explicit Euler
  at the stability-limited dt, Philox nucleation every 100 steps (seed 42,
  the reference's physical nucleation parameters).  One benchmark step = 100
  time steps + the nucleation call of that interval.  `value` is the FP32
  precision form with fields resident in HBM; `fp64` the plain FP64 fused
  step on the same grid; `e2e` goes through the C ABI with host buffers
  (upload of the four FP64 fields, 100 steps, read-out) every step;
* `batch64`: 64 uneven grids (sides log-uniform 128-2048), one launch per
  time step;
* `grid3d512`: the 512^3 grid with the 7-point Laplacian;
* `serve`: a Poisson-arrival request trace (200 requests) through the
  continuous-batching server, latency split into queue wait and service;
* `max_field_error`: the FP32 form against the FP64 step at each
  configuration's full step count (4096^2 after 10 000 steps, 512^3 after
  2000, the batch after 5000).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload all|grid4096|batch64|grid3d512|serve|error]

Under torchrun each rank runs an independent replica on its own GPU
(replicas only: the grids do not exchange data), so scaling is weak; at
N > 1 the default run measures the headline workload only.
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
FULL_RUN_STEPS = 10000  # the 4096^2 workload's step count
WORKLOAD = (f"single 2D grid {N_SIDE}x{N_SIDE}, dx=5nm, 16 enriched stripes + 4 particles R=8 "
            f"(seeded), zero-flux, 5-point Laplacian, KKS-stable dt, Philox nucleation every "
            f"{STEPS_PER_BENCH_STEP} steps (seed 42); one bench step = {STEPS_PER_BENCH_STEP} "
            f"time steps + 1 nucleation call")
ERROR_BOUND = 1e-5


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def rank_sync(dist, device):
    """The barrier and the max-over-ranks reduction that bracket every timed
    region (dist None: one process).  device: where the reduction's tensor
    lives ("cuda" under NCCL, where the barrier also waits for the device;
    "cpu" under gloo)."""
    def barrier():
        if dist is not None:
            dist.barrier()
        if device == "cuda":
            import torch
            torch.cuda.synchronize()

    def max_over_ranks(x):
        if dist is None:
            return x
        import torch
        t = torch.tensor([x], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    return barrier, max_over_ranks


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
    """Untimed steps until `seconds` have passed, so that the timed region
    starts at steady clocks (a first run on a GPU fresh from idle sampled
    1987 MHz, the next one 2070).  Run it on a scratch grid: the step time
    depends on how far a grid has evolved (nuclei accumulate)."""
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
            "same_config_note": "a bounded sample of the same grid: FP64 time steps without the "
                                "nucleation call, compared per cell-update",
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
SERVE_COUNT = 200
SERVE_RATE = 20.0


def serve_workload(count):
    return (f"serving trace of {count} requests (seed 5): Poisson arrivals {SERVE_RATE:g}/s, "
            f"size uniform over {{256^2, 1024^2, 4096^2, 128^3, 256^3}}, steps uniform in "
            f"[2000, 20000], compositions from the alloy ranges; FP32 form, continuous batching "
            f"(2D grids in one batch, 3D grids on their own streams), FIFO admission by device "
            f"footprint; one bench step = the whole trace")


class Ctx:
    """What every workload needs: arguments, ranks, the barrier and the
    max-over-ranks reduction, the library binding and the generators."""

    def __init__(self, args, ws, rank, local, barrier, max_over_ranks, pl, ic):
        self.args, self.ws, self.rank, self.local = args, ws, rank, local
        self.barrier, self.max_over_ranks = barrier, max_over_ranks
        self.pl, self.ic = pl, ic


def roofline(kernel, kms, cells, bytes_per_cell, profile):
    """Roofline of one step kernel: algorithmic bytes per launch over its
    average launch time (CUDA events on its stream) against the measured HBM
    copy bandwidth; traffic from the committed ncu summary."""
    peak, peak_kind = measured_peak_hbm()
    achieved = bytes_per_cell * cells / (kms / 1e3) / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": profiled_traffic(profile), "kernel": kernel,
            "bytes_per_cell": bytes_per_cell, "kernel_ms": kms, "peak_kind": peak_kind}


def pinned(shape):
    import torch
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


def max_err(a, b):
    """Per-field max |a - b| over the interior."""
    return [float(np.max(np.abs(x[(slice(1, -1),) * x.ndim] - y[(slice(1, -1),) * y.ndim])))
            for x, y in zip(a, b)]


def err_dict(e, **kw):
    return dict(kw, x_Cr=e[0], x_Nb=e[1], phi_delta=e[2], phi_laves=e[3])


# ---------------------------------------------------------------------------
def grid4096(c, quick_error=True):
    """The headline workload; returns its JSON line (rank 0) or None."""
    args, ws, rank, pl, ic = c.args, c.ws, c.rank, c.pl, c.ic
    import torch
    # --side resizes the grid of a value-only run (smaller profiler captures)
    side = args.side if args.only == "value" and args.side else N_SIDE
    fields = ic.config2(seed=2 + rank, n=side)
    params = pl.model_params()
    cells = side * side
    nuc_kw = dict(seed=42, geometry=pl.NUC_REFERENCE_GEOMETRY, interval=STEPS_PER_BENCH_STEP,
                  sigma=NUC["sigma"], unit_a=NUC["unit_a"], d=(params["dx"],) * 3,
                  dt_nuc=STEPS_PER_BENCH_STEP * params["dt"])

    # ---- device-resident FP32 precision form (headline value) ----
    # clocks brought up on a scratch copy of the workload; the timed grid
    # then runs its W warm-up bench steps and its K timed ones from the
    # initial condition (bench steps W+1 .. W+K of the workload)
    gs = pl.Grid2D(fields, params, precision=args.precision)
    gs.set_nucleation(**nuc_kw)
    spin_up(gs)
    gs.close()
    g = pl.Grid2D(fields, params, precision=args.precision)
    g.set_nucleation(**nuc_kw)
    g.run(args.warmup * STEPS_PER_BENCH_STEP)
    g.sync()
    c.barrier()
    with ClockSampler(c.local) as clk:
        ms = g.run_timed(args.steps * STEPS_PER_BENCH_STEP)
    c.barrier()
    t = c.max_over_ranks(ms / 1e3)
    value = ws * cells * STEPS_PER_BENCH_STEP * args.steps / t
    g.close()
    if args.only == "value":
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": "cell-updates/s",
                              "ms_per_step": 1e3 * t / args.steps, "partial": "value only",
                              "nx": side, "ny": side}))
        return None

    # the whole 10 000-step run of the workload from its initial condition
    # (nuclei accumulate, so later steps take longer than the early ones)
    gf = pl.Grid2D(fields, params, precision=args.precision)
    gf.set_nucleation(**nuc_kw)
    msf = gf.run_timed(FULL_RUN_STEPS)
    gf.close()
    full_run = {"value": cells * FULL_RUN_STEPS / (msf / 1e3), "unit": "cell-updates/s",
                "ms_per_step": msf / (FULL_RUN_STEPS / STEPS_PER_BENCH_STEP),
                "steps": FULL_RUN_STEPS,
                "what": "all 10 000 steps of the workload in one timed run (nucleation every 100)"}

    # the denser variant of the same grid (64 particles), device-resident
    f64p = ic.config2(seed=2 + rank, n=N_SIDE, n_particles=64)
    gd = pl.Grid2D(f64p, params, precision=args.precision)
    gd.set_nucleation(**nuc_kw)
    gd.run(args.warmup * STEPS_PER_BENCH_STEP)
    c.barrier()
    msd = gd.run_timed(args.steps * STEPS_PER_BENCH_STEP)
    gd.close()
    dense = {"value": cells * STEPS_PER_BENCH_STEP * args.steps / (msd / 1e3),
             "unit": "cell-updates/s", "ms_per_step": msd / args.steps,
             "workload": "the same grid with 64 particles R=8 instead of 4"}

    # kernel-only time of the step kernel (no nucleation): average launch
    g2 = pl.Grid2D(fields, params, precision=args.precision)
    g2.run(200)
    kms = g2.run_timed(400) / 400
    g2.close()
    bytes_per_cell = 48 if args.precision == "fp32" else 64
    kname = "step2d_f32_4096" if args.precision == "fp32" else "step2d_f32k_4096"
    roof = roofline("k_stream_f32", kms, cells, bytes_per_cell, kname)
    # secondary: the 32 B/cell floor of the four fields alone
    roof["no_compensation_floor"] = {"bytes_per_cell": 32,
                                     "achieved": 32 * cells / (kms / 1e3) / 1e9,
                                     "frac": 32 * cells / (kms / 1e3) / 1e9 / roof["peak"]}

    # ---- plain FP64 fused step on the same workload ----
    g64 = pl.Grid2D(fields, params, precision="fp64")
    g64.set_nucleation(**nuc_kw)
    g64.run(STEPS_PER_BENCH_STEP)
    ms64 = g64.run_timed(STEPS_PER_BENCH_STEP)
    g64.close()
    fp64_value = cells * STEPS_PER_BENCH_STEP / (ms64 / 1e3)
    # the variable-mobility form (FP64) on the same grid
    gv = pl.Grid2D(fields, params, precision="fp64", mobility="variable")
    gv.run(2)
    msv = gv.run_timed(10) / 10
    gv.close()
    # and its FP32 form (the flux as div (D(X, Y) grad x^gamma), Kahan-compensated)
    gw = pl.Grid2D(fields, params, precision=args.precision, mobility="variable")
    gw.run(3)
    msw = gw.run_timed(STEPS_PER_BENCH_STEP) / STEPS_PER_BENCH_STEP
    gw.close()

    err = None
    if quick_error:
        # stated error after 400 steps (the full-length figures: --workload error)
        ga = pl.Grid2D(fields, params, precision=args.precision)
        gb = pl.Grid2D(fields, params, precision="fp64")
        ga.run(400)
        gb.run(400)
        err = err_dict(max_err(ga.read(), gb.read()),
                       vs="fp64 GPU step (pinned to the reference at 1e-12)", steps=400)
        ga.close()
        gb.close()

    # ---- e2e through the C ABI with host buffers ----
    host_in = []
    for a in fields:
        h = pinned(a.shape)
        h[...] = a
        host_in.append(h)
    host_out = [pinned(a.shape) for a in fields]
    ge = pl.Grid2D(fields, params, precision=args.precision)
    ge.set_nucleation(**nuc_kw)
    ge.upload(host_in)
    ge.run(STEPS_PER_BENCH_STEP)
    ge.read(host_out)
    # serial: each bench step uploads, runs and reads back on one handle
    c.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        ge.upload(host_in)
        ge.run(STEPS_PER_BENCH_STEP)
        ge.read(host_out)
    c.barrier()
    te_serial = c.max_over_ranks(time.perf_counter() - t0)
    # pipelined: bench steps are independent jobs on two alternating handles;
    # job k+1's upload and job k-1's read-out (asynchronous entry points,
    # page-locked buffers) overlap job k's steps.  Every job's copies are
    # inside the timed region.
    host_out2 = [[pinned(a.shape) for a in fields] for _ in range(2)]
    gp = [ge, pl.Grid2D(fields, params, precision=args.precision)]
    gp[1].set_nucleation(**nuc_kw)
    for x in gp:  # warm the second handle's graphs and transfer events
        x.upload(host_in)
        x.run(STEPS_PER_BENCH_STEP)
        x.read(host_out)
    c.barrier()
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
    c.barrier()
    te = c.max_over_ranks(time.perf_counter() - t0)
    for x in gp:
        x.close()
    e2e_value = ws * cells * STEPS_PER_BENCH_STEP * args.steps / te
    e2e_serial = ws * cells * STEPS_PER_BENCH_STEP * args.steps / te_serial
    io_bytes = 4 * fields[0].size * 8
    if rank != 0:
        return None

    cpu = None
    if not args.no_cpu:
        sample_steps = 3
        tc = cpu_baseline(fields, pl.model_params(), sample_steps)
        cpu = {"value": cells * sample_steps / tc, "unit": "cell-updates/s",
               "cores": os.cpu_count(), "kind": "port", "cpu": cpu_model(),
               "sample": f"{sample_steps} FP64 time steps of the {N_SIDE}^2 grid, "
                         f"OpenMP, reference host flags"}
        # the 256^2 workload at its full 1000 steps
        f1 = ic.config1()
        t1 = cpu_baseline(f1, pl.model_params(), 1000)
        cpu["c1"] = {"value": (f1[0].shape[0] - 2) * (f1[0].shape[1] - 2) * 1000 / t1,
                     "unit": "cell-updates/s", "seconds": t1,
                     "sample": "the 256^2 grid (one stripe, four particles), 1000 FP64 steps"}
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
                 "fp64_flops_per_cell": profiled_value("step2d_f64_4096", "fp64_flops_per_cell"),
                 "bound": "FP64 pipe",
                 "variable_mobility": {"value": cells / (msv / 1e3), "unit": "cell-updates/s",
                                       "ms_per_step": msv,
                                       "what": "the reference's disabled variable-mobility "
                                               "Cahn-Hilliard, FP64 (pfa_set_mobility)"}},
        "variable_mobility_fp32": {"value": cells / (msw / 1e3), "unit": "cell-updates/s",
                                   "ms_per_step": msw, "speedup_over_fp64": msv / msw,
                                   "bytes_per_cell": 48,
                                   "hbm_frac": 48 * cells / (msw / 1e3) / 1e9 / roof["peak"],
                                   "what": "the variable-mobility step in the FP32 form "
                                           f"({args.precision}), no nucleation"},
        "roofline": roof,
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
        "full_run": full_run,
        "grid4096_dense": dense,
        "gpu_launches": args.steps * (STEPS_PER_BENCH_STEP + NUC_LAUNCHES),
        "clocks": clk.summary(),
    }
    if err is not None:
        line["max_field_error"] = err
    return line


# ---------------------------------------------------------------------------
def batch64(c):
    """The many-grids workload: all grids resident in one batch arena."""
    args, ws, rank, pl, ic = c.args, c.ws, c.rank, c.pl, c.ic
    sides = ic.batch_sides(BATCH_COUNT, seed=3 + 100 * rank)
    fields = [ic.batch_grid(s, seed=1000 + k) for k, s in enumerate(sides)]
    cells = sum(s * s for s in sides)
    params = pl.model_params()
    arena = sum(pl.Batch.footprint(f[0].shape) for f in fields) + (1 << 20)
    b = pl.Batch(params, arena)
    for f in fields:
        b.add(f)
    tuned_ms = b.tune(reps=5)
    launch = b.launch()
    b.run(args.warmup * STEPS_PER_BENCH_STEP)
    b.sync()
    c.barrier()
    with ClockSampler(c.local) as clk:
        ms = b.run_timed(args.steps * STEPS_PER_BENCH_STEP)
    c.barrier()
    t = c.max_over_ranks(ms / 1e3)
    value = ws * cells * STEPS_PER_BENCH_STEP * args.steps / t
    kms = b.run_timed(400) / 400
    b.close()
    # one-at-a-time FP64 loop over the same grids (the single-grid FP64 step)
    n64 = 10
    t64 = 0.0
    for f in fields:
        g = pl.Grid2D(f, params, precision="fp64")
        g.run(2)
        t64 += g.run_timed(n64) / 1e3
        g.close()
    fp64_value = cells * n64 / t64
    # e2e: every bench step adds all grids from host memory, runs, reads them back
    host = [[pinned(a.shape) for a in f] for f in fields]
    for h, f in zip(host, fields):
        for x, a in zip(h, f):
            x[...] = a
    outs = [[pinned(a.shape) for a in f] for f in fields]
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
    c.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    c.barrier()
    te_serial = c.max_over_ranks(time.perf_counter() - t0)
    # pipelined: bench steps are independent jobs on two alternating batches.
    # Job k's adds and steps are enqueued on one batch, then job k-1's grids
    # are read back (pfa_batch_read_async, one set of page-locked output
    # arrays per batch) and removed from the other; nothing waits for the GPU
    # until the end, where both batches are synchronised inside the timed
    # region.
    outs2 = [outs, [[pinned(a.shape) for a in f] for f in fields]]
    bp = [be, pl.Batch(params, arena)]
    bp[1].set_launch(launch["rows"], launch["persistent"])
    ss = [bp[1].add(h) for h in host]  # warm the second batch's graphs
    bp[1].run(STEPS_PER_BENCH_STEP)
    for s_, o in zip(ss, outs):
        bp[1].read(s_, o)
    for s_ in ss:
        bp[1].remove(s_)

    def drain(job):
        y, ys, o = job
        for s_, oo in zip(ys, o):
            y.read_async(s_, oo)
        for s_ in ys:
            y.remove(s_)

    c.barrier()
    t0 = time.perf_counter()
    pending = None
    for k in range(args.steps):
        x = bp[k % 2]
        xs = [x.add(h) for h in host]
        x.run(STEPS_PER_BENCH_STEP)
        if pending:
            drain(pending)
        pending = (x, xs, outs2[k % 2])
    drain(pending)
    for x in bp:
        x.sync()
    c.barrier()
    te = c.max_over_ranks(time.perf_counter() - t0)
    for x in bp:
        x.close()
    io = sum(4 * f[0].size * 8 for f in fields)
    return {
        "workload": BATCH_WORKLOAD, "value": value, "unit": "cell-updates/s",
        "ms_per_step": 1e3 * t / args.steps, "steps": args.steps,
        "config": {"grids": BATCH_COUNT, "cells": cells, "precision": "fp32",
                   "launch": launch, "tuned_ms_per_step": tuned_ms,
                   "l2": "inputs larger than L2 (FP32 state 48 B/cell, 2.3 GB)",
                   "parallelism": f"replicas x{ws}"},
        "fp64": {"value": fp64_value, "unit": "cell-updates/s",
                 "how": "one grid at a time, single-grid FP64 step",
                 "speedup_fp32_over_fp64": value / ws / fp64_value},
        "roofline": roofline("k_batch_f32", kms, cells, 48, "batch_f32_64"),
        "e2e": {"value": ws * cells * STEPS_PER_BENCH_STEP * args.steps / te,
                "unit": "cell-updates/s", "h2d_bytes_per_step": io, "d2h_bytes_per_step": io,
                "mode": "independent jobs on two alternating batches: job k's adds and steps "
                        "are enqueued, then job k-1's grids are read back (asynchronous "
                        "reads) and removed while job k computes; both batches synchronised "
                        "at the end",
                "serial": {"value": ws * cells * STEPS_PER_BENCH_STEP * args.steps / te_serial,
                           "unit": "cell-updates/s",
                           "mode": "one batch: add all, run, read all, remove all"}},
        "gpu_launches": args.steps * STEPS_PER_BENCH_STEP,
        "clocks": clk.summary(),
    }


# ---------------------------------------------------------------------------
def grid3d512(c):
    """The 3D workload, FP32 form vs the FP64 step."""
    args, ws, rank, pl, ic = c.args, c.ws, c.rank, c.pl, c.ic
    n = args.side or GRID3D_SIDE
    fields = ic.grid3d(n, n, n, seed=4 + rank, slab=64, n_particles=32, radius=6.0)
    params = pl.model_params(dim=3)
    cells = n ** 3
    nuc = dict(seed=42, interval=STEPS_PER_BENCH_STEP, sigma=NUC["sigma"], unit_a=NUC["unit_a"],
               d=(params["dx"],) * 3, dt_nuc=STEPS_PER_BENCH_STEP * params["dt"])
    g = pl.Grid3D(fields, params, precision="fp32")
    g.set_nucleation(**nuc)
    g.run(args.warmup * STEPS_PER_BENCH_STEP)
    c.barrier()
    with ClockSampler(c.local) as clk:
        ms = g.run_timed(args.steps * STEPS_PER_BENCH_STEP)
    c.barrier()
    t = c.max_over_ranks(ms / 1e3)
    value = ws * cells * STEPS_PER_BENCH_STEP * args.steps / t
    if args.only == "value":
        g.close()
        return {"workload": GRID3D_WORKLOAD, "value": value, "unit": "cell-updates/s",
                "ms_per_step": 1e3 * t / args.steps, "partial": "value only"}
    g.set_nucleation(interval=0)  # the step kernel alone for the roofline
    g.run(2)
    kms = g.run_timed(50) / 50
    # e2e: every bench step uploads the four FP64 fields from page-locked host
    # memory, runs 100 steps with nucleation and reads the fields back
    host_in = []
    for a in fields:
        h = pinned(a.shape)
        h[...] = a
        host_in.append(h)
    host_out = [pinned(a.shape) for a in fields]
    g.set_nucleation(**nuc)

    def e2e_step():
        g.upload(host_in)
        g.run(STEPS_PER_BENCH_STEP)
        g.read(host_out)

    e2e_step()
    c.barrier()
    t0 = time.perf_counter()
    e2e_steps = max(1, min(args.steps, 3))
    for _ in range(e2e_steps):
        e2e_step()
    c.barrier()
    te_serial = c.max_over_ranks(time.perf_counter() - t0)
    # pipelined: independent jobs on two alternating handles, job k+1's upload
    # and job k-1's read-out overlapping job k's steps (every job's copies
    # inside the timed region)
    g2 = pl.Grid3D(fields, params, precision="fp32")
    g2.set_nucleation(**nuc)
    g2.upload(host_in)
    g2.run(STEPS_PER_BENCH_STEP)
    g2.read(host_out)
    host_out2 = [host_out, [pinned(a.shape) for a in fields]]
    gp = [g, g2]
    pipe_steps = max(2, min(args.steps, 8))
    c.barrier()
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
    c.barrier()
    te = c.max_over_ranks(time.perf_counter() - t0)
    g.close()
    g2.close()
    io_bytes = 4 * fields[0].size * 8
    g64 = pl.Grid3D(fields, params, precision="fp64")
    g64.run(2)
    ms64 = g64.run_timed(6) / 6
    g64.close()
    workload = GRID3D_WORKLOAD if n == GRID3D_SIDE else GRID3D_WORKLOAD.replace(
        f"{GRID3D_SIDE}^3", f"{n}^3")
    return {
        "workload": workload, "value": value, "unit": "cell-updates/s",
        "ms_per_step": 1e3 * t / args.steps, "steps": args.steps,
        "config": {"nx": n, "ny": n, "nz": n, "precision": "fp32",
                   "l2": "inputs larger than L2 (FP32 state 6.4 GB)",
                   "parallelism": f"replicas x{ws}"},
        "fp64": {"value": cells / (ms64 / 1e3), "unit": "cell-updates/s", "ms_per_step": ms64,
                 "speedup_fp32_over_fp64": value / ws / (cells / (ms64 / 1e3))},
        "roofline": roofline("k_stream3d_f32", kms, cells, 48, "step3d_f32_512"),
        "e2e": {"value": ws * cells * STEPS_PER_BENCH_STEP * pipe_steps / te,
                "unit": "cell-updates/s", "h2d_bytes_per_step": io_bytes,
                "d2h_bytes_per_step": io_bytes, "steps": pipe_steps,
                "mode": "independent jobs on two alternating handles: job k+1's upload and "
                        "job k-1's read-out (pfa3d_upload_async / pfa3d_read_async, "
                        "page-locked buffers) overlap job k's steps",
                "serial": {"value": ws * cells * STEPS_PER_BENCH_STEP * e2e_steps / te_serial,
                           "unit": "cell-updates/s", "steps": e2e_steps,
                           "mode": "one handle: upload, run, read back"}},
        "gpu_launches": args.steps * (STEPS_PER_BENCH_STEP + NUC_LAUNCHES),
        "clocks": clk.summary(),
    }


# ---------------------------------------------------------------------------
def serve(c, count=SERVE_COUNT, recipes=True, compare_host_fields=False):
    """Latency and aggregate throughput of the serving layer on a request
    trace.  recipes: every request carries its initial condition as a recipe
    the device builds (pfa_ic_recipe), else as host fields uploaded on
    admission."""
    from pfa_gb300.serve import GpuBackend, Request, Server, fifo_latencies, latency_stats
    args, ws, rank, pl, ic = c.args, c.ws, c.rank, c.pl, c.ic
    trace = ic.serve_trace(count, seed=5 + 100 * rank, rate=SERVE_RATE)

    def requests(from_recipes):
        if from_recipes:
            return [Request(t["rid"], None, t["steps"], t["arrival"], recipe=ic.serve_recipe(t))
                    for t in trace]
        return [Request(t["rid"], ic.serve_fields(t), t["steps"], t["arrival"]) for t in trace]

    reqs = requests(recipes)
    work = sum(r.cells * r.steps for r in reqs)
    p2, p3 = pl.model_params(), pl.model_params(dim=3)
    arena, budget3 = 64 << 30, 64 << 30

    def serve_once(rs, realtime=True):
        be = GpuBackend(pl, p2, p3, arena, budget3)
        srv = Server(be, tick_steps=STEPS_PER_BENCH_STEP)
        done = srv.run_trace(rs, realtime=realtime)
        be.close()
        return done, srv

    # warm-up: the first requests of the trace at 300 steps each
    warm = [Request(r.rid, r.fields, 300, 0.0, recipe=r.recipe) for r in reqs[:8]]
    serve_once(warm, realtime=False)
    c.barrier()
    with ClockSampler(c.local) as clk:
        done, srv = serve_once(reqs)
    c.barrier()
    first = min(r.req.arrival for r in done)
    span = c.max_over_ranks(max(r.finished for r in done) - first)
    value = ws * work / span
    stats = latency_stats(done)
    queue = np.array([r.admitted - r.req.arrival for r in done])
    service = np.array([r.finished - r.admitted for r in done])
    arrivals_span = max(t["arrival"] for t in trace) - min(t["arrival"] for t in trace)
    out = {
        "workload": serve_workload(count), "value": value, "unit": "cell-updates/s",
        "ms_per_step": 1e3 * span, "steps": 1,
        "config": {"requests": count, "cell_updates": work, "precision": "fp32",
                   "tick_steps": STEPS_PER_BENCH_STEP, "ticks": srv.ticks,
                   "initial_conditions": "built on the device from each request's recipe"
                   if recipes else "host fields uploaded on admission",
                   "budget_bytes": {"2d_arena": arena, "3d": budget3},
                   "parallelism": f"replicas x{ws}"},
        "latency": dict(stats, unit="s", what="arrival to result read back"),
        "queue": {"p50_s": float(np.percentile(queue, 50)),
                  "p99_s": float(np.percentile(queue, 99)), "max_s": float(queue.max()),
                  "what": "arrival to admission (waiting for device footprint)"},
        "service": {"p50_s": float(np.percentile(service, 50)),
                    "p99_s": float(np.percentile(service, 99)), "max_s": float(service.max()),
                    "what": "admission to result read back (sharing the GPU with the "
                            "requests admitted beside it)"},
        # offered work per second of arrivals over what the GPU delivers
        "offered_load": work / max(arrivals_span, 1e-9) / (value / ws),
        "gpu_launches": srv.step_launches,
        "clocks": clk.summary(),
    }
    if compare_host_fields:
        done_h, _ = serve_once(requests(not recipes))
        span_h = c.max_over_ranks(max(r.finished for r in done_h) - first)
        st = latency_stats(done_h)
        out["other_ic"] = {"value": ws * work / span_h, "p50_s": st["p50_s"],
                           "p99_s": st["p99_s"],
                           "how": "host fields uploaded on admission" if recipes else
                                  "initial conditions built on the device from recipes"}
    # one-at-a-time FP64, modelled: each size's FP64 step time and its
    # set-up (upload, read-back, free) measured on one request of that size;
    # a request's service = set-up + steps x step time; FIFO in arrival order
    per_size = {}
    for t_ in trace:
        key = (t_["dim"], t_["side"])
        if key in per_size:
            continue
        f = ic.serve_fields(t_)
        t0 = time.perf_counter()
        g = (pl.Grid2D(f, p2, precision="fp64") if t_["dim"] == 2
             else pl.Grid3D(f, p3, precision="fp64"))
        g.run(2)
        sample = 10 if np.prod([n - 2 for n in f[0].shape]) > 4e6 else 40
        ms = g.run_timed(sample) / sample
        g.read()
        g.close()
        setup = max(0.0, time.perf_counter() - t0 - 1e-3 * ms * (sample + 2))
        per_size[key] = (setup, 1e-3 * ms)
    svc = [per_size[(t_["dim"], t_["side"])][0] + per_size[(t_["dim"], t_["side"])][1] *
           t_["steps"] for t_ in trace]
    arr = [t_["arrival"] for t_ in trace]
    lat64 = fifo_latencies(arr, svc)
    span64 = max(a + l for a, l in zip(arr, lat64)) - min(arr)
    out["fp64"] = {"kind": "modelled", "value": work / span64, "unit": "cell-updates/s",
                   "p50_s": float(np.percentile(lat64, 50)),
                   "p99_s": float(np.percentile(lat64, 99)),
                   "how": "one request at a time in arrival order with the FP64 step; each "
                          "size's step time and set-up (upload, read-back) measured on one "
                          "request, service = set-up + steps x step time, queueing computed "
                          "(running the loop would take hours)",
                   "step_ms": {f"{d}d{s}": 1e3 * v[1] for (d, s), v in per_size.items()}}
    # the model against whole requests run for real: the first request of
    # each of the two smallest sizes in the trace, FP64, all its steps,
    # from upload to read-back
    checks = []
    for key in sorted(per_size, key=lambda k: k[1] ** k[0])[:2]:
        t_ = next(t for t in trace if (t["dim"], t["side"]) == key)
        f = ic.serve_fields(t_)
        t0 = time.perf_counter()
        g = (pl.Grid2D(f, p2, precision="fp64") if t_["dim"] == 2
             else pl.Grid3D(f, p3, precision="fp64"))
        g.run(t_["steps"])
        g.read()
        g.close()
        measured = time.perf_counter() - t0
        modelled = per_size[key][0] + per_size[key][1] * t_["steps"]
        checks.append({"request": f"{key[0]}d{key[1]}, {t_['steps']} steps",
                       "measured_s": measured, "modelled_s": modelled,
                       "ratio": measured / modelled})
    out["fp64"]["check"] = checks
    return out


# ---------------------------------------------------------------------------
def stated_error(c):
    """Stated error at the configurations' full step counts: the FP32 form
    against the FP64 step on the 4096^2 grid (10000 steps, nucleation every
    100 steps with the same seed in both), the 512^3 grid (2000 steps) and
    the batch of 64 uneven grids (5000 steps, each grid against its own FP64
    run)."""
    args, pl, ic = c.args, c.pl, c.ic
    out = {"vs": "the FP64 GPU step (pinned to the reference's kernels at 1e-12)",
           "metric": "per field max |FP32 - FP64| over the interior", "bound": ERROR_BOUND}
    p2 = pl.model_params()
    f2 = ic.config2(n=N_SIDE)
    n2 = args.error_steps or 10000
    runs = {}
    for prec in ("fp32", "fp64"):
        g = pl.Grid2D(f2, p2, precision=prec)
        g.set_nucleation(seed=42, geometry=pl.NUC_REFERENCE_GEOMETRY, interval=100,
                         sigma=NUC["sigma"], unit_a=NUC["unit_a"], d=(p2["dx"],) * 3,
                         dt_nuc=100 * p2["dt"])
        ms = g.run_timed(n2)
        runs[prec] = (g.read(), ms)
        g.close()
    out["grid4096"] = err_dict(max_err(runs["fp32"][0], runs["fp64"][0]), steps=n2,
                               fp32_ms=runs["fp32"][1], fp64_ms=runs["fp64"][1])
    side = args.side or GRID3D_SIDE
    n3 = min(2000, n2)
    p3 = pl.model_params(dim=3)
    f3 = ic.grid3d(side, side, side, seed=4, slab=64, n_particles=32, radius=6.0)
    res3 = {}
    for prec in ("fp32", "fp64"):
        g = pl.Grid3D(f3, p3, precision=prec)
        g.set_nucleation(seed=42, interval=100, sigma=NUC["sigma"], unit_a=NUC["unit_a"],
                         d=(p3["dx"],) * 3, dt_nuc=100 * p3["dt"])
        res3[prec] = (g.run_timed(n3), g.read())
        g.close()
    out["grid3d"] = err_dict(max_err(res3["fp32"][1], res3["fp64"][1]), side=side, steps=n3,
                             fp32_ms=res3["fp32"][0], fp64_ms=res3["fp64"][0])
    # the batch of 64 uneven grids in the batched FP32 form; each grid's own
    # FP64 run on its own stream, all enqueued before any is read back
    nb = min(5000, n2)
    sides = ic.batch_sides(BATCH_COUNT, seed=3)
    fields = [ic.batch_grid(sd, seed=1000 + k) for k, sd in enumerate(sides)]
    arena = sum(pl.Batch.footprint(f[0].shape) for f in fields) + (1 << 20)
    b = pl.Batch(p2, arena)
    slots = [b.add(f) for f in fields]
    tb = b.run_timed(nb)
    grids = [pl.Grid2D(f, p2, precision="fp64") for f in fields]
    t0 = time.perf_counter()
    for g in grids:
        g.run(nb)
    errb = [0.0] * 4
    for g, sl in zip(grids, slots):
        e = max_err(b.read(sl), g.read())
        errb = [max(x, y) for x, y in zip(errb, e)]
    t64 = time.perf_counter() - t0
    for g in grids:
        g.close()
    b.close()
    out["batch64"] = err_dict(errb, grids=BATCH_COUNT, steps=nb, fp32_ms=tb,
                              fp64_s_concurrent=t64)
    out["max"] = max(max(out[k][f] for f in ("x_Cr", "x_Nb", "phi_delta", "phi_laves"))
                     for k in ("grid4096", "grid3d", "batch64"))
    return out


# ---------------------------------------------------------------------------
def _print_single(c, res):
    """One workload's result as its own contract line."""
    args, ws = c.args, c.ws
    line = {"metric": METRIC, "value": res.pop("value"), "unit": res.pop("unit"), "n_gpus": ws,
            "steps": res.pop("steps", args.steps), "warmup": args.warmup,
            "ms_per_step": res.pop("ms_per_step"), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict({"workload": res.pop("workload")}, **res.pop("config", {})),
            "cpu_baseline": None}
    line.update(res)
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp32k"])
    ap.add_argument("--workload", default="all",
                    choices=["all", "grid4096", "batch64", "grid3d512", "serve", "error"],
                    help="all: the headline line with every other workload inside it; "
                         "the others print one workload's own line")
    ap.add_argument("--side", type=int, default=0,
                    help="grid3d512 / error: another cube side; grid4096 with --only value: "
                         "another square side (smaller profiler captures)")
    ap.add_argument("--requests", type=int, default=SERVE_COUNT, help="serve: trace length")
    ap.add_argument("--error-steps", type=int, default=0,
                    help="error: 2D step count (default 10000; 3D and batch take min(n, 2000 / "
                         "5000))")
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

    barrier, max_over_ranks = rank_sync(dist, "cuda")
    c = Ctx(args, ws, rank, local, barrier, max_over_ranks, pl, ic)
    w = args.workload
    if w in ("all", "grid4096"):
        line = grid4096(c, quick_error=(w == "grid4096" or ws > 1))
        if w == "all" and ws == 1 and args.only == "all":
            line["batch64"] = batch64(c)
            line["grid3d512"] = grid3d512(c)
            line["serve"] = serve(c, count=args.requests)
            line["max_field_error"] = stated_error(c)
        elif w == "all" and line is not None and ws > 1:
            line["other_workloads"] = "measured at N=1 only (replicas of the headline here)"
        if line is not None and rank == 0:
            print(json.dumps(line))
    elif w == "batch64":
        res = batch64(c)
        if rank == 0:
            _print_single(c, res)
    elif w == "grid3d512":
        res = grid3d512(c)
        if rank == 0:
            _print_single(c, res)
    elif w == "serve":
        res = serve(c, count=args.requests, compare_host_fields=True)
        if rank == 0:
            _print_single(c, res)
    elif w == "error":
        if rank == 0:
            t0 = time.perf_counter()
            res = stated_error(c)
            g2 = res["grid4096"]
            _print_single(c, {"workload": "stated-error study: FP32 form vs FP64 at full step "
                                          "counts",
                              "value": N_SIDE * N_SIDE * g2["steps"] / (g2["fp32_ms"] / 1e3),
                              "unit": "cell-updates/s",
                              "ms_per_step": 1e3 * (time.perf_counter() - t0), "steps": 1,
                              "max_field_error": res})
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
