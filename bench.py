"""Benchmark of the upwind advection hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--arith auto|fixed|fma|exact] [--no-cpu-baseline]

Workload (one bench step): advect(100 steps, dt) of the 512^3 FP64 periodic
unit cube, v = (1.0, -0.7, 0.3), dt = 0.5 min_j dx_j/|v_j| = 0.5/512, initial
field = sphere indicator (centre 0.5^3, radius 0.2) + seeded uniform noise in
[0, 0.01) (seed 20261203).  Metric: FP64 cell updates per second (GCUPS).

  value        device-timed: K bench steps between CUDA events on the
               library's stream, field resident in HBM (1 GiB per buffer, far
               larger than L2, so no flush is needed between steps).
  e2e          the same metric through the public API with host buffers:
               every step uploads the initial field from pinned host memory,
               advects, downloads the field and reads the checksum
               (Upwind.advect_host_stream: the next upload and the previous
               download overlap each advect).  `serial_value` is the same
               cycle as separate set_field/advect/get_field/checksum calls.
  roofline     the step kernel's achieved bandwidth on the 16 B/cell-update
               algorithmic basis (read f once, write f once) against the
               measured HBM copy peak.
  cpu_baseline the reference algorithm (oracle/_ref when it was compiled in
               this tree, else the oracle's C restatement) on the host cores,
               on a bounded sample of the same workload.

  f64_paths    the FP64 arithmetics (EXACT, FMA) at the same workload.
  sharded      the distributed form: one (512 N) x 512 x 512 grid split into
               512-plane slabs, one per rank, halo planes exchanged every 3
               steps (NCCL between ranks, a device copy at N = 1).

`--impl reference` times that CPU implementation alone (the reference arm).
Under torchrun (N > 1) the headline runs one independent replica per rank and
rank 0 prints the aggregate; the sharded leg splits one grid over the ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_AXIS = 512
SHAPE = (N_AXIS, N_AXIS, N_AXIS)
VELOCITY = (1.0, -0.7, 0.3)
LENGTHS = (1.0, 1.0, 1.0)
TIME_STEPS = 100
DT = 0.5 / N_AXIS
SEED = 20261203
CENTER = (0.5, 0.5, 0.5)
RADIUS = 0.2
NOISE = 0.01
BYTES_PER_CELL_UPDATE = 16.0  # read f, write f (FP64)
WORKLOAD = "upwind3d_f64_512cube_100steps"


def configure(n_axis: int) -> None:
    """Cube size (512 for the benchmark; smaller cubes only for profiling)."""
    global N_AXIS, SHAPE, DT, WORKLOAD
    N_AXIS = n_axis
    SHAPE = (n_axis, n_axis, n_axis)
    DT = 0.5 / n_axis
    WORKLOAD = f"upwind3d_f64_{n_axis}cube_100steps"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def load_peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def load_traffic(kernel: str):
    """DRAM bytes per cell-update of `kernel` from the committed ncu summary
    (profiles/traffic_per_cell_update.txt: `<kernel> <bytes> <source>`)."""
    p = os.path.join(ROOT, "profiles", "traffic_per_cell_update.txt")
    try:
        for line in open(p):
            parts = line.split()
            if len(parts) >= 2 and parts[0] == kernel and not line.startswith("#"):
                return float(parts[1])
    except OSError:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the
    timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = []
        with open(self.file.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        smax = [num(r[2]) for r in rows if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4)
                          if r[5 + k].lower().startswith("active")})
        loaded = [s for s in sm if smax and s >= 0.3 * max(smax)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def cpu_sample(threads: int | None = None, time_steps: int = 2, one_thread: bool = False):
    """Reference algorithm on the host: a bounded sample of the workload (the
    full 512^3 field, `time_steps` time steps), all host threads; with
    one_thread also the restatement on a single core (one time step)."""
    from oracle import Port, Reference
    port = Port()
    f0 = port.sphere_noise(SHAPE, LENGTHS, CENTER, RADIUS, NOISE, SEED)
    threads = threads or os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    kind = "port"
    impl = port
    if Reference.available():
        try:
            impl = Reference()
            kind = "reference"
        except OSError:
            impl = port
    if kind == "reference":
        _, el = impl.advect_timed(SHAPE, VELOCITY, LENGTHS, f0, time_steps, DT)
    else:
        _, el = impl.advect_timed(SHAPE, VELOCITY, LENGTHS, f0, time_steps, DT, threads=threads)
    cells = float(np.prod(SHAPE)) * time_steps
    out = {"value": cells / el / 1e9, "unit": "GCUPS", "cores": threads, "kind": kind,
           "sample": f"{N_AXIS}^3 x {time_steps} time steps (of the workload's 100), "
                     f"{el:.2f} s, OMP_NUM_THREADS={threads}, "
                     + ("reference upwind.cxx compiled by oracle/Makefile" if kind == "reference"
                        else "oracle C restatement, -O3 -fopenmp -ffp-contract=off")}
    if one_thread:
        # the same restatement on one core, one time step
        _, el1 = port.advect_timed(SHAPE, VELOCITY, LENGTHS, f0, 1, DT, threads=1)
        out["one_thread"] = {"value": float(np.prod(SHAPE)) / el1 / 1e9, "unit": "GCUPS",
                             "cores": 1, "kind": "port",
                             "sample": f"{N_AXIS}^3 x 1 time step, {el1:.2f} s, 1 thread"}
    return out


BATCH_COUNT = 256
BATCH_STEPS = 50
BATCH_SEED = 20261203


def bench_batched(steps: int, warmup: int, stream, rank: int = 0, ws: int = 1) -> dict:
    """Batched form: 256 independent 3-D FP64 problems, axes uniform in
    [32, 160], velocities uniform in [-1, 1]^3, CFL 0.5, 50 steps, sphere
    initial fields (seeded centres/radii).  One persistent launch per advect
    (replayed from a CUDA graph), tuned by the library's autotuner, against
    the single-field kernel looped over the same instances.  With N ranks the
    instances are split by a size-balanced partition (no exchange during the
    advect); rates use the slowest rank's time."""
    import torch
    import fidibench_gb300 as fdb
    from fidibench_gb300.batch import random_instances
    from fidibench_gb300.sharding import gather_by_index, partition_instances, reduce_max

    all_specs = random_instances(BATCH_COUNT, BATCH_SEED)
    sizes = [int(np.prod(s["n"])) for s in all_specs]
    mine = partition_instances(sizes, ws)[rank]
    specs = [all_specs[i] for i in mine]
    b = fdb.Batch([(s["v"], s["L"], s["n"]) for s in specs])
    b.set_stream(stream)
    dts = [s["dt"] for s in specs]

    def reset():
        for k, i in enumerate(mine):
            s = all_specs[i]
            b.init_sphere(k, s["center"], s["radius"], 0.0, BATCH_SEED + i)

    reset()
    cells = float(sum(sizes))
    t0 = time.perf_counter()
    chosen = b.autotune(BATCH_STEPS, dts)
    tune_s = time.perf_counter() - t0

    def timed(fn):
        for _ in range(warmup):
            fn()
        stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return reduce_max(e0.elapsed_time(e1) / steps)

    reset()
    ms_batched = timed(lambda: b.advect(BATCH_STEPS, dts))
    # agreement after one advect from the initial fields: the looped
    # comparator at the batch's depth takes the same time blocks, so the
    # integer arithmetic gives bit-identical fields (compared via checksums)
    reset()
    b.advect(BATCH_STEPS, dts)
    sums_batched = gather_by_index(dict(zip(mine, b.checksums())), BATCH_COUNT)
    reset()
    b.advect_looped(BATCH_STEPS, dts)
    sums_looped = gather_by_index(dict(zip(mine, b.checksums())), BATCH_COUNT)
    # the timed comparator: the single-field kernel at each instance's
    # default depth, as looping Upwind.advect over the instances runs it
    b.set_tuning(depth=0)
    reset()
    ms_looped = timed(lambda: b.advect_looped(BATCH_STEPS, dts))
    b.close()
    gb = cells * BATCH_STEPS / (ms_batched * 1e-3) / 1e9
    gl = cells * BATCH_STEPS / (ms_looped * 1e-3) / 1e9
    agree = float(np.max(np.abs(sums_batched - sums_looped) / np.maximum(np.abs(sums_looped), 1e-300)))
    return {"workload": f"batch{BATCH_COUNT}_uneven32-160_{BATCH_STEPS}steps",
            "instances": BATCH_COUNT, "cells": int(cells), "time_steps": BATCH_STEPS,
            "ranks": ws, "batched_gcups": gb, "looped_gcups": gl, "ratio": gb / gl,
            "ms_per_advect_batched": ms_batched, "ms_per_advect_looped": ms_looped,
            "looped_depth": "single-field default per instance",
            "tuning": chosen, "autotune_s": tune_s, "graph_replay": True,
            "checksums_identical_at_equal_depth": bool(np.array_equal(sums_batched, sums_looped)),
            "checksum_rel_diff_batched_vs_looped": agree}


ADJ_N = 256
ADJ_STEPS = 200
ADJ_CKPT = 20
ADJ_V = (0.8, 0.5, -0.6)


def gaussian_random_field(n: int, corr_cells: float, seed: int, device):
    """Seeded Gaussian random field on the periodic n^3 grid: white noise
    smoothed by a Gaussian of standard deviation `corr_cells` cells (FFT),
    normalised to unit standard deviation."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    w = torch.randn((n, n, n), generator=g, device=device, dtype=torch.float64)
    k = torch.fft.fftfreq(n, device=device, dtype=torch.float64)
    kr = torch.fft.rfftfreq(n, device=device, dtype=torch.float64)
    k2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + kr[None, None, :] ** 2
    filt = torch.exp(-2.0 * (np.pi ** 2) * (corr_cells ** 2) * k2)
    f = torch.fft.irfftn(torch.fft.rfftn(w) * filt, s=(n, n, n))
    return (f - f.mean()) / f.std()


def bench_adjoint(stream) -> dict:
    """Adjoint form: 256^3, v = (0.8, 0.5, -0.6), dt = 0.5 min dx/|v|, 200
    steps; L = 0.5 ||f_T - target||^2 with a seeded Gaussian random field
    target (correlation length 8 cells).  Reports the adjoint/forward per-step
    cost of the default form (dL/dv in closed form), of the step-by-step form
    (checkpoints every 20 steps, recompute, a contraction per step) and of
    dL/df0 alone; the dot-product test and central finite differences
    (h = 1e-6) on 16 seeded directions and the 3 velocities (default form)."""
    import torch
    import fidibench_gb300 as fdb

    n3 = (ADJ_N,) * 3
    L = (1.0, 1.0, 1.0)
    dt = 0.5 * min(1.0 / ADJ_N / abs(v) for v in ADJ_V)
    up = fdb.Upwind(ADJ_V, L, n3)
    up.set_stream(stream)
    dev = torch.device("cuda", torch.cuda.current_device())
    up.init_sphere((0.5, 0.5, 0.5), 0.2, 0.01, SEED)
    f0 = torch.empty(ADJ_N ** 3, dtype=torch.float64, device=dev)
    up.get_field(f0)
    target = gaussian_random_field(ADJ_N, 8.0, SEED, dev).reshape(-1)

    def forward(x, vel=ADJ_V):
        up.set_velocity(vel)
        up.set_field(x)
        up.advect(ADJ_STEPS, dt)
        out = torch.empty_like(x)
        up.get_field(out)
        return out

    # forward step cost (the production advect)
    for _ in range(2):
        forward(f0)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    up.set_field(f0)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(3):
        up.advect(ADJ_STEPS, dt)
    e1.record(stream)
    e1.synchronize()
    fwd_ms_step = e0.elapsed_time(e1) / (3 * ADJ_STEPS)

    lam = forward(f0) - target
    timings = []
    for _ in range(2):
        up.set_field(f0)
        g0, gv = up.adjoint(ADJ_STEPS, dt, lam, checkpoint_every=ADJ_CKPT)
        timings.append(up.adjoint_timings())
    t = timings[-1]
    # the step-by-step form (checkpoints every ADJ_CKPT steps, recompute, one
    # contraction per transposed step) for comparison
    up.set_adjoint_form("stepwise")
    for _ in range(2):
        up.set_field(f0)
        g0_sw, gv_sw = up.adjoint(ADJ_STEPS, dt, lam, checkpoint_every=ADJ_CKPT)
        t_sw = up.adjoint_timings()
    up.set_adjoint_form("closed")
    sw_gv_rel = float(np.max(np.abs(np.asarray(gv) - np.asarray(gv_sw))) /
                      np.max(np.abs(np.asarray(gv_sw))))
    sw_g0_rel = float(torch.max(torch.abs(g0_sw - g0)) / torch.max(torch.abs(g0_sw)))
    # dL/df0 alone: the transposed problem (every upwind direction reversed)
    for _ in range(2):
        up.set_field(f0)
        g0_fast, _ = up.adjoint(ADJ_STEPS, dt, lam, velocity_grad=False)
        t_fast = up.adjoint_timings()
    fast_vs_full = float(torch.max(torch.abs(g0_fast - g0)) / torch.max(torch.abs(g0)))

    h = 1e-6

    def fd(fp, fm):
        rp, rm = fp - target, fm - target
        return float(torch.sum((rp - rm) * (rp + rm)).item()) / (4.0 * h)

    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED + 1)
    errs_f0 = []
    for _ in range(16):
        dvec = torch.randn(f0.shape, generator=gen, device=dev, dtype=torch.float64)
        exact = float(torch.dot(g0, dvec).item())
        errs_f0.append(abs(fd(forward(f0 + h * dvec), forward(f0 - h * dvec)) - exact) /
                       max(abs(exact), 1e-300))
    errs_v = []
    for j in range(3):
        vp, vm = list(ADJ_V), list(ADJ_V)
        vp[j] += h
        vm[j] -= h
        est = fd(forward(f0, vp), forward(f0, vm))
        errs_v.append(abs(est - gv[j]) / max(abs(gv[j]), 1e-300))
    up.set_velocity(ADJ_V)
    # dot-product test <A x, y> = <x, A^T y>
    x = torch.randn(f0.shape, generator=gen, device=dev, dtype=torch.float64)
    y = torch.randn(f0.shape, generator=gen, device=dev, dtype=torch.float64)
    ax = forward(x)
    up.set_field(x)
    aty, _ = up.adjoint(ADJ_STEPS, dt, y, checkpoint_every=ADJ_CKPT)
    lhs = float(torch.dot(ax, y).item())
    rhs = float(torch.dot(x, aty).item())
    up.close()
    adj_step = t["adjoint_ms"] / ADJ_STEPS
    rec_step = t["recompute_ms"] / ADJ_STEPS
    sw_adj = t_sw["adjoint_ms"] / ADJ_STEPS
    sw_rec = t_sw["recompute_ms"] / ADJ_STEPS
    a_sum = sum(abs(v) * dt * ADJ_N for v in ADJ_V)
    return {"workload": "adjoint_256cube_200steps_ckpt20", "dt": dt,
            "courant_sum": a_sum, "forward_ms_per_step": fwd_ms_step,
            "form": "closed: dL/da_j = S <lam^1, D_j f0>, lam^1 = (A^T)^(S-1) lam_T",
            "adjoint_ms_per_step": adj_step, "recompute_ms_per_step": rec_step,
            "adjoint_over_forward": adj_step / fwd_ms_step,
            "backward_incl_recompute_over_forward": (adj_step + rec_step) / fwd_ms_step,
            "call_over_forward": (t["forward_ms"] + t["recompute_ms"] + t["adjoint_ms"]) /
            ADJ_STEPS / fwd_ms_step,
            "adjoint_gcups": ADJ_N ** 3 / (adj_step * 1e-3) / 1e9,
            "stepwise": {"adjoint_ms_per_step": sw_adj, "recompute_ms_per_step": sw_rec,
                         "adjoint_over_forward": sw_adj / fwd_ms_step,
                         "backward_incl_recompute_over_forward": (sw_adj + sw_rec) / fwd_ms_step,
                         "call_over_forward": (t_sw["forward_ms"] + t_sw["recompute_ms"] +
                                               t_sw["adjoint_ms"]) / ADJ_STEPS / fwd_ms_step,
                         "grad_v_rel_diff_vs_closed": sw_gv_rel,
                         "grad_f0_rel_diff_vs_closed": sw_g0_rel},
            "f0_only_ms_per_step": t_fast["adjoint_ms"] / ADJ_STEPS,
            "f0_only_over_forward": t_fast["adjoint_ms"] / ADJ_STEPS / fwd_ms_step,
            "f0_only_vs_full_rel_maxnorm": fast_vs_full,
            "fd_max_rel_err_f0_16dirs": max(errs_f0), "fd_max_rel_err_velocity": max(errs_v),
            "dot_product_rel_err": abs(lhs - rhs) / abs(lhs), "grad_v": [float(x) for x in gv]}


LAP_N = 8000   # the reference laplacian driver's defaults (laplacian/cxx/laplacian.cxx:41-43)
LAP_DIMS = 2
LAP_ITERS = 10


def bench_batch_adjoint(stream) -> dict:
    """Batched adjoint with the velocity gradient: the recovery batch (64
    instances of 128^3, seeded velocities in [-1, 1]^3 rescaled to a Courant
    sum of 0.5, sphere fields), 100 steps, a seeded Gaussian lambda_T.  One
    batched advect against the closed form (one transposed persistent launch,
    one contraction launch, the forward) and the step-by-step form
    (checkpoints every 10 steps, recompute and contraction per step)."""
    import torch
    import fidibench_gb300 as fdb
    from fidibench_gb300.recovery import instance_specs, sphere_field

    count, n, steps = 64, 128, 100
    specs = instance_specs(count, n, SEED)
    dts = [sp["dt"] for sp in specs]
    dev = torch.device("cuda", torch.cuda.current_device())
    f0 = torch.cat([sphere_field(n, sp["center"], sp["radius"], dev).view(-1) for sp in specs])
    gen = torch.Generator(device=dev)
    gen.manual_seed(SEED + 2)
    lam = torch.randn(f0.numel(), generator=gen, device=dev, dtype=torch.float64)
    b = fdb.Batch([(sp["v"], (1.0, 1.0, 1.0), (n, n, n)) for sp in specs])
    b.set_stream(stream)

    def timed(fn, reps=2):
        fn()
        ms = []
        for _ in range(reps):
            b.set_fields(f0)
            stream.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out = fn()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        return min(ms), out

    b.set_fields(f0)
    adv_ms, _ = timed(lambda: b.advect(steps, dts))
    b.set_adjoint_form("closed")
    b.set_fields(f0)
    cl_ms, (_, gv_c) = timed(lambda: b.adjoint(steps, dts, lam))
    b.set_adjoint_form("stepwise")
    b.set_fields(f0)
    sw_ms, (_, gv_s) = timed(lambda: b.adjoint(steps, dts, lam, checkpoint_every=10))
    b.close()
    rel = float(np.max(np.abs(gv_c - gv_s)) / np.max(np.abs(gv_s)))
    return {"workload": "batch64_128cube_100steps", "instances": count,
            "advect_ms": adv_ms, "closed_ms": cl_ms, "stepwise_ms": sw_ms,
            "closed_over_advect": cl_ms / adv_ms, "stepwise_over_advect": sw_ms / adv_ms,
            "grad_v_rel_diff": rel,
            "timing": "CUDA events around each call, host-synchronising calls included"}


def bench_laplacian(stream, cpu: bool) -> dict:
    """Stencil Filter: the reference laplacian driver's default case, 2-D
    8000^2 on the unit square, input prod_i sin(2 pi x_i) at the cell centres,
    stencil -4 at the centre and +1 at +-1 along each axis, the reference's
    index wrap, timed loop 10 x (applyFilter; copyOutToIn).  Also the apply
    kernel alone (iterate: the copy becomes a buffer swap) against the FP64
    pipe (2 operations/clk/SM) and HBM; with the CPU leg, one apply checked
    bit for bit against the CPU restatement and that restatement's own rate."""
    import torch
    from fidibench_gb300.filter import Filter, laplacian_stencil

    dims = (LAP_N,) * LAP_DIMS
    st = laplacian_stencil(LAP_DIMS)
    x = (np.arange(LAP_N, dtype=np.float64) + 0.5) * (1.0 / LAP_N)
    s = np.sin(2.0 * np.pi * x)
    f0 = np.ascontiguousarray((s[:, None] * s[None, :]).reshape(-1))
    cells = float(f0.size)
    flt = Filter(dims, [0.0] * LAP_DIMS, [1.0] * LAP_DIMS, st)
    flt.set_stream(stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def timed(fn, reps):
        flt.set_in_data(f0)
        fn()  # warm-up
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / reps

    def loop():
        for _ in range(LAP_ITERS):
            flt.applyFilter()
            flt.copyOutToIn()

    ms_loop = timed(loop, 3) / LAP_ITERS
    ms_apply = timed(lambda: flt.iterate(LAP_ITERS), 3) / LAP_ITERS
    fp64_per_cell = sum(1 for w in st.values() if w not in (1.0, -1.0)) + (len(st) - 1)
    clock_hz = 2.07e9
    fp64_peak = 2.0 * 152 * clock_hz / 1e9  # GFLOP/s
    out = {
        "workload": f"laplacian{LAP_DIMS}d_{LAP_N}^{LAP_DIMS}_{LAP_ITERS}iters",
        "cells": int(cells), "iterations": LAP_ITERS, "wrap": "reference",
        "gcups_apply_copy_loop": cells / (ms_loop * 1e-3) / 1e9,
        "gcups_apply": cells / (ms_apply * 1e-3) / 1e9,
        "ms_per_apply": ms_apply,
        "fp64_ops_per_cell": fp64_per_cell,
        "fp64_gflops": fp64_per_cell * cells / (ms_apply * 1e-3) / 1e9,
        "fp64_frac_of_pipe": fp64_per_cell * cells / (ms_apply * 1e-3) / 1e9 / fp64_peak,
        "hbm_gbs_apply": 16.0 * cells / (ms_apply * 1e-3) / 1e9,
        "bound": "fp64 pipe (bit-identical products and sums in the reference's order)",
    }
    if cpu:
        from oracle import Port
        port = Port()
        flt.set_in_data(f0)
        flt.applyFilter()
        got = flt.out_data
        t0 = time.perf_counter()
        ref = port.filter_apply(dims, st, f0)
        t_cpu = time.perf_counter() - t0
        out["bit_identical_vs_cpu"] = bool(np.array_equal(got, ref))
        out["cpu_baseline"] = {"value": cells / t_cpu / 1e9, "unit": "GCUPS",
                               "cores": port.max_threads(), "kind": "port",
                               "sample": "one applyFilter at 8000^2 (oracle/filter_oracle.c, "
                                         "OpenMP, -O3 -ffp-contract=off)"}
    flt.close()
    return out


REF_TIME_STEPS_PER_BENCH_STEP = 10  # the reference arm's bounded sample per bench step


def bench_config(ws: int) -> dict:
    """The workload's config, identical in both arms."""
    return {"workload": WORKLOAD, "shape": list(SHAPE), "velocity": list(VELOCITY),
            "time_steps": TIME_STEPS, "dt": DT,
            "init": f"sphere r={RADIUS} + U[0,{NOISE}) noise, seed {SEED}",
            "l2": "inputs larger than L2 (1 GiB field per buffer)",
            "parallelism": f"replicas x{ws}"}


SHARD_PLANES = 512  # planes of axis 0 per rank in the sharded leg (weak scaling)


def bench_sharded(steps: int, warmup: int, ws: int) -> dict:
    """The distributed form (fidibench_gb300.distributed.DistributedUpwind):
    every rank owns a 512-plane slab of a (512 N) x 512 x 512 periodic grid
    (N = ranks: the headline workload per rank), v and dt of the headline,
    100 steps per advect, the K = 3 upwind halo planes exchanged every 3
    steps (NCCL send/recv between ranks; a device copy of the slab's own far
    end at N = 1).  Rates over all ranks, timed as the slowest rank."""
    import torch
    import fidibench_gb300 as fdb
    from fidibench_gb300.distributed import DistributedUpwind
    from fidibench_gb300.sharding import reduce_max

    n = (SHARD_PLANES * ws, N_AXIS, N_AXIS)
    d = DistributedUpwind(VELOCITY, LENGTHS, n, halo=3)
    # each rank's slab starts from the headline's initial field
    src = fdb.Upwind(VELOCITY, LENGTHS, (SHARD_PLANES, N_AXIS, N_AXIS))
    src.init_sphere(CENTER, RADIUS, NOISE, SEED)
    dev = torch.device("cuda", torch.cuda.current_device())
    f = torch.empty(SHARD_PLANES * N_AXIS * N_AXIS, dtype=torch.float64, device=dev)
    src.get_field(f)
    src.close()
    d.slab.set_own(f)
    d.stream.synchronize()  # the copy out of f ends before f is freed
    del f
    cur = d.stream  # the slab's stream: its copies, transfers and steps
    for _ in range(warmup):
        d.advect(TIME_STEPS, DT)
    cur.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(cur)
    for _ in range(steps):
        d.advect(TIME_STEPS, DT)
    e1.record(cur)
    e1.synchronize()
    ms = reduce_max(e0.elapsed_time(e1) / steps)
    cs = d.checksum()
    used = d.slab.arith_used
    d.close()
    cells = float(SHARD_PLANES) * N_AXIS * N_AXIS
    return {"workload": f"sharded_{SHARD_PLANES}x{N_AXIS}x{N_AXIS}_per_rank_{TIME_STEPS}steps",
            "ranks": ws, "global_shape": list(n), "halo_planes": d.halo,
            "exchange": "nccl send/recv" if ws > 1 else "device copy (one rank)",
            "arith": used, "ms_per_advect": ms,
            "gcups": ws * cells * TIME_STEPS / (ms * 1e-3) / 1e9, "checksum": cs,
            "scaling": "weak"}


def run_reference_arm(args, ws, rank) -> None:
    """The reference's CPU implementation of the path on the host cores: each
    bench step runs advect() over REF_TIME_STEPS_PER_BENCH_STEP of the
    workload's 100 time steps of the full 512^3 field (all host threads);
    `ms_per_step` is the wall time one such bench step measured, and `value`
    the cell-update rate over all timed bench steps."""
    if rank != 0:
        return
    from oracle import Port, Reference
    threads = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(threads))
    port = Port()
    f0 = port.sphere_noise(SHAPE, LENGTHS, CENTER, RADIUS, NOISE, SEED)
    kind, impl = "port", port
    if Reference.available():
        try:
            impl, kind = Reference(), "reference"
        except OSError:
            impl, kind = port, "port"
    nts = REF_TIME_STEPS_PER_BENCH_STEP

    def one_step() -> float:
        if kind == "reference":
            _, el = impl.advect_timed(SHAPE, VELOCITY, LENGTHS, f0, nts, DT)
        else:
            _, el = impl.advect_timed(SHAPE, VELOCITY, LENGTHS, f0, nts, DT, threads=threads)
        return el

    for _ in range(args.warmup):
        one_step()
    times = [one_step() for _ in range(args.steps)]
    total = sum(times)
    cells = float(np.prod(SHAPE))
    v = cells * nts * args.steps / total / 1e9
    what = ("reference upwind.cxx compiled by oracle/Makefile" if kind == "reference"
            else "oracle C restatement, -O3 -fopenmp -ffp-contract=off")
    sample = (f"{N_AXIS}^3 x {nts} time steps (of the workload's {TIME_STEPS}) per bench step, "
              f"{args.steps} bench steps in {total:.2f} s, OMP_NUM_THREADS={threads}, {what}")
    print(json.dumps({
        "impl": "reference", "metric": "FP64 GCUPS (upwind advection, 512^3 periodic)",
        "value": v, "unit": "GCUPS", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "arith": "f64 (the reference's operation order)",
        "time_steps_timed": nts,
        "config": bench_config(ws),
        "cpu_baseline": {"value": v, "unit": "GCUPS", "cores": threads, "kind": kind,
                         "sample": sample},
        "e2e": {"value": v, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--arith", default="auto", choices=["auto", "fixed", "fma", "exact"])
    ap.add_argument("--depth", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-f64-paths", action="store_true",
                    help="skip the FP64 (exact/fma) arithmetic figures")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-vs-looped leg")
    ap.add_argument("--no-sharded", action="store_true",
                    help="skip the distributed (slab-sharded) leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint leg")
    ap.add_argument("--no-recovery", action="store_true",
                    help="skip the batched adjoint (gradient-descent recovery) leg")
    ap.add_argument("--no-laplacian", action="store_true",
                    help="skip the stencil Filter (laplacian driver) leg")
    ap.add_argument("--n", type=int, default=512, help="cube size (profiling only)")
    ap.add_argument("--tz", type=int, default=0, help="fixed kernel z-tile override")
    ap.add_argument("--shape", type=int, default=-1, help="fixed kernel CTA shape (0..2)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    configure(args.n)

    ws, rank, local = dist_env()
    if args.impl == "reference":
        run_reference_arm(args, ws, rank)
        return

    import torch
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import fidibench_gb300 as fdb
    from fidibench_gb300._capi import lib

    up = fdb.Upwind(VELOCITY, LENGTHS, SHAPE, arith=args.arith, depth=args.depth)
    if args.tz:
        up.set_tile_z(args.tz)
    if args.shape >= 0:
        up.set_shape(args.shape)
    stream = torch.cuda.Stream()
    up.set_stream(stream)
    up.init_sphere(CENTER, RADIUS, NOISE, SEED)
    cells = float(np.prod(SHAPE))

    for _ in range(args.warmup):
        up.advect(TIME_STEPS, DT)
    stream.synchronize()
    arith_used = up.arith_used

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    # ---- device-timed region --------------------------------------------------
    clocks = ClockSampler(local) if rank == 0 else None
    barrier()
    l0 = lib.fdb_launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        up.advect(TIME_STEPS, DT)
    e1.record(stream)
    barrier()
    launches = int(lib.fdb_launch_count() - l0)
    ms_total = e0.elapsed_time(e1)
    clk = clocks.stop() if clocks else None
    t = torch.tensor([ms_total], device="cuda", dtype=torch.float64)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    value = ws * cells * TIME_STEPS * args.steps / (ms_max * 1e-3) / 1e9

    # ---- roofline of the step kernel --------------------------------------------
    peak, peak_kind = load_peaks()
    step_launches = max(launches, 1)
    cell_updates_per_launch = cells * TIME_STEPS * args.steps / step_launches
    avg_launch_s = ms_total * 1e-3 / step_launches
    achieved = BYTES_PER_CELL_UPDATE * cell_updates_per_launch / avg_launch_s / 1e9
    kernel_name = {"fixed": "k_advect_fixed", "fma": "k_step3_fma",
                   "exact": "k_step3_exact"}.get(arith_used, arith_used)
    tpc = load_traffic(kernel_name)

    # ---- end to end through the public API with host buffers -----------------------
    e2e = None
    if not args.no_e2e:
        host_in = torch.empty(int(cells), dtype=torch.float64, pin_memory=True)
        host_out = torch.empty(int(cells), dtype=torch.float64, pin_memory=True)
        up.get_field(host_in)  # a real field as input

        def serial_cycle():
            up.set_field(host_in)
            up.advect(TIME_STEPS, DT)
            up.get_field(host_out)
            up.checksum()

        def timed(fn):
            barrier()
            t = time.perf_counter()
            fn()
            barrier()
            el = time.perf_counter() - t
            te = torch.tensor([el], device="cuda", dtype=torch.float64)
            if dist is not None:
                dist.all_reduce(te, op=dist.ReduceOp.MAX)
            return float(te.item())

        # the public streaming call: every step uploads its field, advects,
        # downloads the result and returns its checksum; the next upload and
        # the previous download overlap each advect
        up.advect_host_stream([host_in] * 2, TIME_STEPS, DT, out=[host_out] * 2)
        el = timed(lambda: up.advect_host_stream([host_in] * args.steps, TIME_STEPS, DT,
                                                 out=[host_out] * args.steps))
        # the same cycle one call after another (copies not overlapped)
        serial_cycle()
        el_serial = timed(lambda: [serial_cycle() for _ in range(args.steps)])
        e2e = {"value": ws * cells * TIME_STEPS * args.steps / el / 1e9, "unit": "GCUPS",
               "h2d_bytes_per_step": int(cells) * 8, "d2h_bytes_per_step": int(cells) * 8 + 8,
               "api": "Upwind.advect_host_stream (fdb_upwind_advect_host_stream)",
               "serial_value": ws * cells * TIME_STEPS * args.steps / el_serial / 1e9,
               "serial_api": "set_field + advect + get_field + checksum per step"}
    # ---- the per-cell FP64 arithmetics beside the headline -----------------------------
    f64_paths = None
    if not args.no_f64_paths:
        f64_paths = {}
        for name in ("fma", "exact"):
            up.set_arith(name)
            up.init_sphere(CENTER, RADIUS, NOISE, SEED)
            up.advect(10, DT)  # warm-up
            stream.synchronize()
            e0.record(stream)
            up.advect(TIME_STEPS, DT)
            e1.record(stream)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            g = cells * TIME_STEPS / (ms * 1e-3) / 1e9
            f64_paths[name] = {"gcups": g, "ms_per_advect": ms,
                               "frac_of_16B_roofline": g * BYTES_PER_CELL_UPDATE / peak}
        f64_paths["note"] = ("FP64 arithmetic per cell: exact = the reference's operation "
                             "order (bit-identical), fma = 1 DMUL + 3 DFMA; one advect of "
                             f"{TIME_STEPS} steps each, device-timed")
        up.set_arith(args.arith, args.depth)
    up.close()

    sharded = None
    if not args.no_sharded:
        # the headline line must survive a failure of this secondary leg (its
        # multi-rank transfers have not run on more than one GPU here)
        try:
            sharded = bench_sharded(max(1, min(args.steps, 3)), 1, ws)
        except Exception as exc:  # noqa: BLE001
            sharded = {"error": f"{type(exc).__name__}: {str(exc)[:300]}"}

    batched = None
    if not args.no_batch:
        batched = bench_batched(max(3, min(args.steps, 5)), 3, stream, rank, ws)
    # the adjoint and recovery legs are single-GPU workloads: rank 0 runs them
    adjoint = None
    if not args.no_adjoint and rank == 0:
        adjoint = bench_adjoint(stream)
    recovery = None
    if not args.no_recovery and rank == 0:
        # batched adjoint: 64 instances of 128^3, seeded velocities in [-1,1]^3,
        # 100 steps, 20 gradient-descent iterations through the autograd Function
        from fidibench_gb300.recovery import recover
        recovery = recover(count=64, n=128, steps=100, iters=20, seed=SEED)
        # beside it, the same workload with the time step read per axis (each
        # axis at Courant number 0.5, the sum up to 1.5): the instances with a
        # sum above 1 amplify their checkerboard mode by up to 2 per step
        from fidibench_gb300.recovery import data_amplification
        lit = data_amplification(count=64, n=128, steps=100, seed=SEED, cfl_rule="per_axis")
        try:
            r = recover(count=64, n=128, steps=100, iters=20, seed=SEED, fd_check=False,
                        cfl_rule="per_axis")
            lit["descent"] = {k: r[k] for k in ("misfit_reduction_max", "misfit_reduction_median",
                                                "field_rel_err_median")}
        except Exception as e:  # noqa: BLE001  (the descent diverges: the library reports it)
            lit["descent"] = {"error": str(e)[:300]}
        recovery["per_axis_cfl"] = lit
        recovery["batched_adjoint_with_velocity"] = bench_batch_adjoint(stream)
    laplacian = None
    if not args.no_laplacian and rank == 0:
        laplacian = bench_laplacian(stream, cpu=not args.no_cpu_baseline)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_sample(one_thread=True)

    if rank == 0:
        line = {
            "metric": "FP64 GCUPS (upwind advection, 512^3 periodic)",
            "value": value, "unit": "GCUPS", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if arith_used != "fixed" else "f64 (i64 block-fixed-point arithmetic)",
            "data": "synthetic", "arith": arith_used, "time_steps_timed": TIME_STEPS,
            "config": bench_config(ws),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_source": peak_kind,
                         "traffic": None if tpc is None else tpc * cell_updates_per_launch,
                         "kernel": kernel_name,
                         "basis": "16 B algorithmic per cell-update"},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "f64_paths": f64_paths,
            "clocks": clk,
            "gpu_launches": launches,
            "sharded": sharded,
            "batched": batched,
            "adjoint": adjoint,
            "batched_adjoint_recovery": recovery,
            "stencil_filter": laplacian,
        }
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
