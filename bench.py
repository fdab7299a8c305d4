"""Throughput of the GB300 Rosenbrock integrator: cell-intervals per second.

Workload (one "step" = one host interval over every cell): the plain ROS3 drop-in
configuration — a seeded synthetic mass-action mechanism of 210 species and 500
reactions, 65,536 cells in groups of 32, T U[200, 310] K, p U[10, 1000] hPa
setting [M], dt = 30 s, rtol 1e-3, atol = rtol * 1e-14, photolysis updated at
every interval start. FP64 throughout. The timed job starts from the initial
state (the cold first interval included) and runs K intervals.

    python bench.py [--steps K] [--warmup W] [--cells C] [--impl ours|reference]

Prints one JSON line. ``value`` is device-resident throughput (state, rate
constants and controller memory in HBM; per interval one photolysis-update
kernel and one integrator launch); ``e2e`` is the same metric through the
public host API (host arrays in, host arrays out, copies timed); ``roofline``
relates the integrator kernel's algorithmic FP64 rate to the FP64 FMA rate
measured on the same GPU in the same run; ``cpu_baseline`` is the oracle (a
NumPy/SciPy restatement of the reference) on the host cores.
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-intervals/s at rtol=1e-3 on 1 GB300 vs plain GPU + CPU ref; adjoint/forward cost"

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per algorithmic
# FLOP of the integrator kernel on this workload, by kernel variant, from ncu
# captures (profiles/): the bench reports this ratio times its own FLOPs per
# launch as `roofline.traffic`. compact: the first two timed launches of
# `bench.py --kernel compact --steps 2 --warmup 3 --no-cpu --e2e-steps 0
# --plain-steps 0` (3.590 TB over 0.799 PFLOP; the traffic is dominated by the
# elimination's U operands, 8 bytes per 2-FLOP update, so it scales with the
# FLOPs). generated: the two timed launches of `bench.py --cells 8192 --steps 2
# --warmup 3 --no-cpu --e2e-steps 0 --plain-steps 0 --no-extras` (167.3 GB over
# 99.9 GFLOP), a case small enough for the capture, scaled by the FLOPs. A
# variant without a calibration reports no traffic.
DRAM_BYTES_PER_FLOP = {"compact": 4.491, "generated": 1.675}
# the integrator kernel of each variant, as ncu names it
KERNEL_NAME = {"generated": "fo_generated_solve_kernel"}


# ---- CPU baseline: the oracle in a spawn pool, one group per worker --------------------

def _cpu_worker(args):
    """Integrate one group of the workload over `intervals` intervals with the
    reference (installed in baseline/_ref) or, without it, the oracle's
    restatement; returns (cells, intervals, seconds, kind)."""
    group, n_cells, intervals = args
    os.environ["OMP_NUM_THREADS"] = os.environ["OPENBLAS_NUM_THREADS"] = "1"
    sys.path.insert(0, str(ROOT))
    from fastode_gb300 import synthetic as syn
    from oracle.pool import group_solver
    wl = syn.plain_large(n_cells=n_cells, intervals=intervals).subset(slice(group * 32, group * 32 + 32))
    kind, step, new_counts, new_memory = group_solver(wl)
    Y, counts, mem = wl.cells.Y0.copy(), new_counts(), new_memory()
    t0 = time.perf_counter()
    for i in range(intervals):
        Y, _ = step(Y, wl.k_at(i), counts, mem)
    return 32, intervals, time.perf_counter() - t0, kind


def cpu_baseline(n_cells, intervals, workers):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    groups = list(range(workers))
    t0 = time.perf_counter()
    with ctx.Pool(workers) as pool:
        res = pool.map(_cpu_worker, [(g, n_cells, intervals) for g in groups])
    wall = time.perf_counter() - t0
    cell_int = sum(c * i for c, i, _, _ in res)
    per_core = statistics.mean(c * i / s for c, i, s, _ in res)
    kinds = {r[3] for r in res}
    return cell_int / wall, per_core, wall, kinds.pop() if len(kinds) == 1 else "mixed"


# ---- clocks during the timed region ----------------------------------------------------

class Clocks:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in Path(self.file.name).read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


# ---- replicas: one process per GPU, no data exchange -------------------------------------

def max_over_ranks(seconds: float, world: int, device=None) -> float:
    """The job's time with N replicas: the slowest rank's (an all-reduce MAX
    over the process group; the identity on one process)."""
    if world <= 1:
        return seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_rank: float, world: int, seconds: float) -> float:
    """Whole-job throughput: every rank processes the same units (weak
    scaling), divided by the slowest rank's time."""
    return units_per_rank * world / seconds


# ---- the GPU arm ---------------------------------------------------------------------

def algorithmic_flops(plan, counts_rows, offsets):
    """FP64 operations the algorithm needs for these Counts rows (per group:
    lu, solves, rhs, jac, steps) times the cells of each group."""
    f = plan.flops_per_attempt()
    n = plan.n
    cells = np.diff(offsets).astype(np.float64)
    c = counts_rows.astype(np.float64)
    steps, lu, solves, rhs, jac = c[:, 0], c[:, 5], c[:, 6], c[:, 3], c[:, 4]
    # per attempt besides LU and solves: stage combinations and the error norm
    per_step = 14 * n
    per_group = lu * f["lu"] + solves * f["solve"] + rhs * f["rhs"] + jac * f["jac"] + steps * per_step
    return float((per_group * cells).sum())


SUBSET_FIXTURE = ROOT / "tests" / "golden" / "ros3_210x500_subset.npz"


class PlainInputs:
    """Host inputs of the 210/500 workload: Y0, the (C, R) rate constants at
    t = 0 and the (intervals, C) diurnal factors, built by the generator
    (synthetic.rate_constants). When the workload is the full 65,536-cell job,
    the cells of the parity subset take the reference's own inputs from its
    fixture (the reference ran on those exact values)."""

    def __init__(self, wl, intervals):
        from fastode_gb300 import synthetic as syn
        self.wl = wl
        self.photo = np.nonzero(wl.sm.photolytic)[0].astype(np.int32)
        self.J = wl.sm.J[self.photo]
        self.k0 = wl.k_at(0)
        self.fac = syn.photolysis_factors(wl.cells, wl.dt, intervals)
        self.Y0 = wl.cells.Y0.copy()
        self.subset = None
        if wl.cells.C == 65536 and SUBSET_FIXTURE.exists():
            f = dict(np.load(SUBSET_FIXTURE))
            c = f["cells"]
            m = min(intervals, int(f["intervals"]))
            self.k0[c] = f["k0"]
            self.fac[:m, c] = f["f"][:m]
            self.Y0[c] = f["Y0"]
            self.subset = f

    def k_at(self, i):
        """(C, R) rate constants of interval i, as the device builds them."""
        k = self.k0.copy()
        k[:, self.photo] = self.J[None, :] * self.fac[i][:, None]
        return k

    def parity(self, counts, status, Y, intervals):
        """The measured run against the reference on the parity subset after
        `intervals` intervals from the initial state."""
        f = self.subset
        if f is None or intervals > int(f["intervals"]):
            return None
        groups = np.asarray(f["groups"])
        gs = int(f["group_size"])
        out = {"groups": len(groups), "intervals": intervals,
               "reference": "tests/golden/ros3_210x500_subset.npz (the reference run on these cells)",
               "counts_equal": bool(np.array_equal(counts[groups], f["counts"][:, intervals - 1])),
               "status_equal": bool(np.array_equal(status[groups], f["status"][:, intervals - 1]))}
        snaps = list(np.asarray(f["snapshots"]))
        if intervals in snaps:
            ref = f["Y_snap"][snaps.index(intervals)]
            got = Y[np.asarray(f["cells"])]
            out["state_max_rel"] = float((np.abs(got - ref) / np.maximum(np.abs(ref), 1e-14)).max())
            out["state_rtol"] = 1e-10
        tight = list(np.asarray(f["tight_snapshots"])) if "tight_snapshots" in f else []
        if intervals in tight and intervals in snaps:
            # accuracy: Sandu digits (device scoring kernel) of the measured
            # run and of the reference's own rtol = 1e-3 run against the
            # reference at rtol = 1e-10, atol = 1e-10 * a on these cells
            from fastode_gb300.scenario import digits
            t = f["Y_tight"][tight.index(intervals)]
            got = Y[np.asarray(f["cells"])]
            d_dev = digits(got, t, 1e-14)[0]
            d_ref = digits(f["Y_snap"][snaps.index(intervals)], t, 1e-14)[0]
            out["accuracy"] = {"against": "the reference's Algorithm(ROS3) at rtol 1e-10, atol 1e-10 * a",
                               "digits": d_dev, "reference_digits": d_ref, "difference": abs(d_dev - d_ref)}
        return out


def run_ours(args, rank, world):
    import ctypes as C
    import torch
    from fastode_gb300 import _abi, build as fbuild, synthetic as syn
    from fastode_gb300.batch import Batch, solve_host

    fbuild.build()
    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    lib = _abi.lib()
    fma_rate = C.c_double()
    _abi.check(lib.fo_fp64_fma_rate(C.byref(fma_rate)), "fo_fp64_fma_rate")

    wl = syn.plain_large(n_cells=args.cells, intervals=args.steps)
    sm, cells = wl.sm, wl.cells
    Cc, R, n = cells.C, sm.R, sm.n
    # Inputs as the reference builds them (synthetic.rate_constants on the
    # host: k at t = 0 and every interval's diurnal factors), uploaded once;
    # on the parity subset the reference's own inputs, read from its fixture.
    # Per interval the device sets the photolysis columns to J * f (one IEEE
    # product, fo_photolysis_factor), so the device integrates exactly k_at(i).
    inputs = PlainInputs(wl, max(args.steps, args.warmup, args.e2e_steps))
    photo = inputs.photo
    d = {name: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for name, v in
         dict(J=inputs.J, rxn=photo, atol=wl.atol, fac=inputs.fac).items()}
    k = torch.from_numpy(np.ascontiguousarray(inputs.k0.T)).to(dev)          # (R, C), cells fastest
    stream = torch.cuda.current_stream(dev)
    sp = C.c_void_p(stream.cuda_stream)

    def photolysis(i):
        _abi.check(lib.fo_photolysis_factor(Cc, len(photo), d["rxn"].data_ptr(), d["J"].data_ptr(),
                                            d["fac"][i].data_ptr(), k.data_ptr(), 1, Cc, sp),
                   "fo_photolysis_factor")

    Y0 = torch.from_numpy(inputs.Y0).to(dev)
    from fastode_gb300 import Algorithm
    batch = Batch(sm.mech, Y0, group_size=32, slots=args.slots,
                  algorithm=Algorithm(kernel=args.kernel, ordering=args.ordering, tile=args.tile))

    def reset(b=batch):
        b.Y.copy_(Y0.t())
        b.memory.zero_()
        b.counts.zero_()
        b.status.zero_()

    for i in range(args.warmup):                     # untimed: the same kernels and shapes
        photolysis(i)
        batch.step(k, wl.dt, d["atol"], wl.rtol)
    torch.cuda.synchronize()
    reset()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    marks = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    n_plain = min(args.plain_steps, args.steps)
    counts_at_plain = torch.empty_like(batch.counts)
    with Clocks(dev.index) as clocks:
        start.record()
        for i in range(args.steps):
            marks[i].record()
            photolysis(i)
            ev[i][0].record()
            batch.step(k, wl.dt, d["atol"], wl.rtol)
            ev[i][1].record()
            if i + 1 == n_plain:
                counts_at_plain.copy_(batch.counts, non_blocking=True)   # 213 KB, device to device
        end.record()
        torch.cuda.synchronize()
    elapsed = start.elapsed_time(end) / 1e3
    interval_ms = [marks[i].elapsed_time(marks[i + 1] if i + 1 < args.steps else end) for i in range(args.steps)]

    # the plain one-group-per-block kernel (FO_VARIANT_PLAIN) on the first
    # intervals of the same job, for the "vs plain GPU" comparison
    plain = None
    if n_plain > 0 and args.kernel != "plain":
        pb = Batch(sm.mech, Y0, group_size=32, slots=args.slots, algorithm=Algorithm(kernel="plain", ordering=args.ordering))
        torch.cuda.synchronize()
        p0, p1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        p0.record()
        for i in range(n_plain):
            photolysis(i)
            pb.step(k, wl.dt, d["atol"], wl.rtol)
        p1.record()
        torch.cuda.synchronize()
        plain_s = p0.elapsed_time(p1) / 1e3
        ours_s = sum(interval_ms[:n_plain]) / 1e3
        plain = {"value": Cc * n_plain / plain_s, "unit": "cell-intervals/s", "intervals": n_plain,
                 "ours_same_intervals": Cc * n_plain / ours_s, "speedup": plain_s / ours_s,
                 "same_counts": bool(np.array_equal(pb.counts.cpu().numpy(), counts_at_plain.cpu().numpy())),
                 "same_counts_scope": f"Counts of every group after the first {n_plain} intervals"}
        del pb
    elapsed = max_over_ranks(elapsed, world, dev)
    solve_ms = [a.elapsed_time(b) for a, b in ev]
    counts = batch.counts.cpu().numpy()
    statuses = batch.statuses()
    flops = algorithmic_flops(batch.plan, counts, batch.offsets_host)
    kernel_s = sum(solve_ms) / 1e3
    achieved = flops / kernel_s / 1e12
    peak = 2.0 * fma_rate.value / 1e12
    value = job_value(Cc * args.steps, world, elapsed)

    # e2e through the public host API: host arrays in and out, copies timed
    e2e_steps = min(args.steps, args.e2e_steps)
    e2e = None
    if e2e_steps > 0:
        from fastode_gb300.batch import HostState, solve_host_intervals
        pinned_k = [torch.from_numpy(inputs.k_at(i)).pin_memory() for i in range(e2e_steps)]
        Y0h = torch.from_numpy(inputs.Y0.copy()).pin_memory()
        alg = Algorithm(kernel=args.kernel, ordering=args.ordering, tile=args.tile)
        # (1) the overlapped host API: the state stays on the device, every
        # interval's rate constants go in and its state and statuses come out,
        # on a second stream while the device integrates
        state = HostState(sm.mech, Cc, n, R, 32, alg, None, args.slots, dev)
        state.overlap_buffers()
        sums = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, state, (h2d, d2h) = solve_host_intervals(
            sm.mech, Y0h, pinned_k, wl.dt, wl.atol, wl.rtol, state=state, group_size=32, slots=args.slots,
            on_result=lambda i, Yh, st: sums.append(float(Yh[0, 0])))   # the host reads every result
        e2e_s = time.perf_counter() - t0
        # (2) one solve_host call per interval, the reference's calling pattern
        state = HostState(sm.mech, Cc, n, R, 32, alg, None, args.slots, dev)
        Yh = Y0h
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h2d1 = d2h1 = 0
        for i in range(e2e_steps):
            Yh, state, moved = solve_host(sm.mech, Yh, pinned_k[i], wl.dt, wl.atol, wl.rtol, state=state,
                                          group_size=32, slots=args.slots)
            h2d1 += moved[0]
            d2h1 += moved[1]
        call_s = time.perf_counter() - t0
        # whole job: every rank runs the same intervals; the slowest rank's time
        e2e_s = max_over_ranks(e2e_s, world, dev)
        call_s = max_over_ranks(call_s, world, dev)
        resident = job_value(Cc * e2e_steps, world, max_over_ranks(sum(interval_ms[:e2e_steps]) / 1e3, world, dev))
        e2e = {"value": job_value(Cc * e2e_steps, world, e2e_s), "unit": "cell-intervals/s", "steps": e2e_steps,
               "h2d_bytes_per_step": h2d // e2e_steps, "d2h_bytes_per_step": d2h // e2e_steps,
               "device_resident_same_intervals": resident,
               "api": "fastode_gb300.batch.solve_host_intervals (host (C,n) state in once, host (C,R) rate "
                      "constants in and the (C,n) state and statuses out every interval, copies overlapped "
                      "with the integration; the first intervals of the job from the initial state)",
               "per_call": {"value": job_value(Cc * e2e_steps, world, call_s), "unit": "cell-intervals/s",
                            "h2d_bytes_per_step": h2d1 // e2e_steps, "d2h_bytes_per_step": d2h1 // e2e_steps,
                            "api": "fastode_gb300.batch.solve_host, one call per interval (state in and out "
                                   "every call)"}}

    out = {
        "metric": METRIC, "value": value, "unit": "cell-intervals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
        "config": {"workload": "ros3-210x500: synthetic 210 species / 500 reactions, 65,536 cells in groups "
                               "of 32, dt=30 s, rtol=1e-3, photolysis per interval" if Cc == 65536 else
                               f"ros3-210x500 with {Cc} cells",
                   "cells": Cc, "group_size": 32, "intervals_timed": args.steps, "dt": wl.dt, "rtol": wl.rtol,
                   "l2": "inputs larger than L2 (state 110 MB + rate constants 262 MB + scratch per interval)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "slots": args.slots or "one block per group"},
        "gpu_launches": 2 * args.steps,
        "statuses": {s: statuses.count(s) for s in set(statuses)},
        "counts_per_group_interval": {
            "attempts": float(counts[:, 0].sum() / len(counts) / args.steps),
            "rejected": float(counts[:, 2].sum() / len(counts) / args.steps)},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak,
                     "traffic": (DRAM_BYTES_PER_FLOP[args.kernel] * flops / args.steps
                                 if args.kernel in DRAM_BYTES_PER_FLOP else None),
                     "traffic_unit": "bytes per launch",
                     "traffic_source": (f"ncu DRAM bytes per algorithmic FLOP of this kernel on this workload "
                                        f"({DRAM_BYTES_PER_FLOP[args.kernel]} B/FLOP, measured on an 8,192-cell case) "
                                        "times this run's FLOPs per launch" if args.kernel in DRAM_BYTES_PER_FLOP else
                                        "not calibrated for this kernel variant"),
                     "kernel": KERNEL_NAME.get(args.kernel, "solve_kernel"),
                     "kernel_ms_per_launch": sum(solve_ms) / len(solve_ms),
                     "peak_source": "fo_fp64_fma_rate: full-warp DFMA kernel, same GPU, same run (the driver's "
                                    "peaks file holds HBM and bf16 only)",
                     "algorithmic_flops_per_launch": flops / args.steps},
        "clocks": clocks.summary(),
        "e2e": e2e,
        "plain_gpu": plain,
        "kernel_variant": args.kernel,
        "generated_module": batch.plan.gen_info,
        "lu": {k: batch.plan.info[k] for k in ("ordering", "lu_fma", "nnz_lu", "solve_fma")},
        "parity": inputs.parity(counts, batch.status.cpu().numpy(), batch.state(), args.steps),
        "interval_ms": {"first": interval_ms[0], "median": float(np.median(interval_ms)),
                        "max": float(max(interval_ms))},
    }
    if rank == 0 and args.cpu_intervals > 0 and not args.no_cpu:
        workers = args.cpu_workers or os.cpu_count()
        thr, per_core, wall, kind = cpu_baseline(args.cells, args.cpu_intervals, workers)
        out["cpu_baseline"] = {"value": thr, "unit": "cell-intervals/s", "cores": workers, "kind": kind,
                               "per_core": per_core,
                               "sample": f"{workers} groups of 32 cells x the first {args.cpu_intervals} "
                                         f"intervals (cold start included), one group per process, "
                                         f"BLAS 1 thread, {wall:.1f} s wall"}
    return out


def _device_rates(lib, sm, cells, dev, sp):
    """(R, C) thermal rate constants computed on the device, plus what the
    photolysis update needs."""
    import ctypes as C
    import torch
    from fastode_gb300 import _abi, synthetic as syn
    Cc, R = cells.C, sm.R
    M = cells.p / (syn.R_GAS * cells.T)
    photo = np.nonzero(sm.photolytic)[0].astype(np.int32)
    d = {name: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for name, v in
         dict(A=sm.A, E=sm.E, power=sm.mech.third_body_power, T=cells.T, M=M).items()}
    k = torch.empty((R, Cc), dtype=torch.float64, device=dev)
    _abi.check(lib.fo_rate_constants(Cc, R, d["A"].data_ptr(), d["E"].data_ptr(), d["power"].data_ptr(),
                                     d["T"].data_ptr(), d["M"].data_ptr(), k.data_ptr(), 1, Cc, sp),
               "fo_rate_constants")
    return k, photo


def run_batched(args):
    """Batched uneven workload: 1,048,576 cells over three synthetic mechanisms
    (60/40, 120/260, 210/500) in one persistent launch per interval, photolysis
    under a diurnal cosine (half the cells dark), dt = 60 s, each interval one
    replay of a captured CUDA graph."""
    import ctypes as C
    import torch
    from fastode_gb300 import _abi, build as fbuild, synthetic as syn
    from fastode_gb300.multi import MultiBatch, Part
    fbuild.build()
    dev = torch.device("cuda", 0)
    lib = _abi.lib()
    sp = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    wls = syn.batched_uneven(n_cells=args.cells, intervals=args.steps)
    from fastode_gb300 import Algorithm
    chosen = [(32, args.kernel, 6) for _ in wls]
    tuning = None
    if args.autotune:
        # per mechanism: group size (8 to 128 cells), kernel and the
        # generated code's register tile, measured on 4,096 of its cells (one
        # untimed and two timed intervals each)
        from fastode_gb300.tune import autotune, candidates, measure_on_device
        from fastode_gb300.plan import plan_for
        tiles = tuple(int(t) for t in str(getattr(args, "tune_tiles", "6")).split(","))
        tuning = []
        for j, wl in enumerate(wls):
            sample = wl.subset(slice(0, min(4096, wl.cells.C)))
            measure = measure_on_device(sample.sm.mech, sample.cells.Y0, sample.k_at, sample.dt, sample.atol,
                                        sample.rtol)
            bp = plan_for(sample.sm.mech)
            smem = {k: bp.smem_items(k) for k in ("pipelined", "plain", "compact")}
            smem["generated"] = 0
            # the generated kernel for groups of up to 32 cells, the compact
            # one above (below 32 cells it measured slower than the generated)
            cands = [c for c in candidates(smem, group_sizes=(8, 16, 32, 64, 128), kernels=("generated", "compact"),
                                           persistent=(True,), tiles=tiles)
                     if (c.kernel == "generated") == (c.group_size <= 32)]
            res = autotune(measure, smem, cands)
            if res.best.kernel != "generated":       # one launch runs one family of kernels
                gen = [(c, v) for c, v in res.table if c.kernel == "generated" and v is not None]
                best = max(gen, key=lambda cv: cv[1])[0] if gen else res.best
            else:
                best = res.best
            chosen[j] = (best.group_size, best.kernel, best.tile)
            tuning.append({"mechanism": wl.name, "sample": f"{sample.cells.C} cells, intervals 1-2 timed",
                           "table": [{"kernel": c.kernel, "group_size": c.group_size, "tile": c.tile,
                                      "cell_intervals_per_s": v} for c, v in res.table],
                           "chosen": {"kernel": best.kernel, "group_size": best.group_size, "tile": best.tile}})
    parts = []
    for wl, (group_size, kernel, tile) in zip(wls, chosen):
        k, photo = _device_rates(lib, wl.sm, wl.cells, dev, sp)
        p = Part(wl.sm.mech, torch.from_numpy(wl.cells.Y0).to(dev), k.t(), wl.atol, wl.rtol, wl.dt,
                 group_size=group_size, algorithm=Algorithm(kernel=kernel, ordering=args.ordering, tile=tile),
                 photolysis=(photo, wl.sm.J[photo], wl.cells.phase))
        parts.append(p)
    kernel = chosen[0][1]
    group_size = sorted({c[0] for c in chosen})
    fma_rate = C.c_double()
    _abi.check(lib.fo_fp64_fma_rate(C.byref(fma_rate)), "fo_fp64_fma_rate")
    mb = MultiBatch(parts)
    mb.capture()
    mb.run(args.warmup, graph=True)
    torch.cuda.synchronize()
    mb.reset()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clocks:
        e0.record()
        mb.run(args.steps, graph=True)
        e1.record()
        torch.cuda.synchronize()
    s = e0.elapsed_time(e1) / 1e3
    total = sum(p.C for p in parts)
    flops = sum(algorithmic_flops(p.plan, p.counts.cpu().numpy(), p.offsets.cpu().numpy()) for p in parts)
    achieved = flops / s / 1e12
    peak = 2.0 * fma_rate.value / 1e12
    per_part = []
    for wl, p in zip(wls, parts):
        c = p.counts.cpu().numpy()
        st = p.status.cpu().numpy()
        per_part.append({"mechanism": wl.name, "cells": p.C, "attempts_per_group_interval":
                         float(c[:, 0].sum() / len(c) / args.steps), "non_converged_groups": int((st != 0).sum()),
                         "plan": {k: v for k, v in p.plan.info.items() if k in ("nnz_lu", "lu_fma", "ordering")}})
    return {"metric": METRIC, "value": total * args.steps / s, "unit": "cell-intervals/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": s / args.steps * 1e3,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic (seeded generator)",
            "config": {"workload": "batched uneven: %d cells over 60/40, 120/260, 210/500, dt=60 s, half dark, "
                                   "one persistent launch per interval replayed as a CUDA graph" % total,
                       "slots": mb.slots, "group_size": group_size, "kernel": kernel},
            "gpu_launches": args.steps * mb.launches_per_interval(), "parts": per_part, "clocks": clocks.summary(),
            "autotune": tuning,
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak,
                         "traffic": (DRAM_BYTES_PER_FLOP[kernel] * flops / args.steps
                                     if kernel in DRAM_BYTES_PER_FLOP else None),
                         "traffic_unit": "bytes per interval (the 210/500 ratio; smaller mechanisms stream less)",
                         "time": "CUDA events around the graph replays of the timed intervals",
                         "peak_source": "fo_fp64_fma_rate, same GPU, same run"}}


def run_adjoint(args):
    """Adjoint cost: (forward + adjoint) / forward for the 210/500 mechanism,
    4,096 cells, 60 intervals of 30 s; loss = sum_i (log(y_i + a) - log(yhat_i + a))^2
    over final states with targets from a perturbed-rate forward run
    (log k + N(0, 0.1)); two central-difference directions (h = 1e-6) of the
    fixed-step replay check the gradient."""
    import torch
    from fastode_gb300 import adjoint as A, build as fbuild, synthetic as syn
    from fastode_gb300.batch import Batch
    fbuild.build()
    dev = torch.device("cuda", 0)
    wl = syn.plain_large(n_cells=args.cells, intervals=args.steps)
    ks = [torch.from_numpy(np.ascontiguousarray(wl.k_at(i).T)).to(dev) for i in range(args.steps)]
    rng = np.random.default_rng(11)
    pert = torch.from_numpy(np.exp(rng.normal(0.0, 0.1, wl.sm.R))).to(dev)[:, None]
    a = 1e-14
    atol = torch.from_numpy(wl.atol).to(dev)

    def forward(kk):
        b = Batch(wl.sm.mech, wl.cells.Y0, group_size=32)
        for i in range(args.steps):
            b.step(kk[i], wl.dt, atol, wl.rtol)
        return b

    target = forward([k * pert for k in ks]).Y.clone()
    forward(ks)                                                    # warm
    torch.cuda.synchronize()
    with Clocks(0) as clocks:
        t0 = time.perf_counter()
        fb = forward(ks)
        torch.cuda.synchronize()
        t_fwd = time.perf_counter() - t0
        for rep in range(2):                                      # a warm-up pass, then the timed one
            t0 = time.perf_counter()
            traj = A.forward_record(wl.sm.mech, wl.cells.Y0, lambda i: ks[i], wl.dt, wl.atol, wl.rtol, args.steps)
            Y = traj.batch.Y
            lam = 2.0 * (torch.log(Y + a) - torch.log(target + a)) / (Y + a)
            lam0, thbar = A.adjoint(traj, lam)
            torch.cuda.synchronize()
            t_fa = time.perf_counter() - t0
    g_th = thbar.sum(dim=1).cpu().numpy()

    def loss(Yend):
        return float(((torch.log(Yend + a) - torch.log(target + a)) ** 2).sum())

    checks = []
    h = 1e-6
    for d in range(args.fd_directions):
        dth = rng.standard_normal(wl.sm.R)
        sc = [torch.from_numpy(np.exp(s * h * dth)).to(dev)[:, None] for s in (1.0, -1.0)]
        fd = (loss(A.replay(traj, ks=[k * sc[0] for k in ks])) - loss(A.replay(traj, ks=[k * sc[1] for k in ks]))) / (2 * h)
        adj = float(np.dot(g_th, dth))
        checks.append({"fd": fd, "adjoint": adj, "rel": abs(fd - adj) / max(abs(fd), 1e-300)})
    return {"metric": "adjoint/forward cost", "value": t_fa / t_fwd, "unit": "ratio", "higher_is_better": False,
            "forward_s": t_fwd, "forward_plus_adjoint_s": t_fa, "max_steps_per_interval": traj.max_steps,
            "clocks": clocks.summary(), "kernel": traj.batch.alg.kernel,
            "time": "wall clock around the forward run and around the recording forward plus the adjoint "
                    "(both synchronized), the second of two passes",
            "config": {"workload": f"adjoint ROS3 210x500, {args.cells} cells, {args.steps} x 30 s, "
                                   "gradients w.r.t. 500 log rate constants and the initial state"},
            "fd_checks": checks,
            "fd_max_rel": max((c["rel"] for c in checks), default=None)}


def run_dae(args):
    """Constrained workload: RODAS3 on 150 differential + 10 algebraic species
    (mass = 0 rows, quasi-steady state), 16,384 cells in groups of 32, 60 s
    intervals, rtol 1e-4, the projection at every call. Forward throughput
    (device-resident, CUDA events around the timed intervals), then the
    adjoint cost ratio on the same run ((forward recorded + adjoint) / plain
    forward, wall clock) with central-difference checks of the gradient. The
    adjoint differentiates the Rosenbrock steps with the recorded step sizes;
    the projection at each interval start is not differentiated (it moves an
    already consistent state by roundoff only)."""
    import torch
    from fastode_gb300 import Algorithm, RODAS3, adjoint as A, build as fbuild, synthetic as syn
    from fastode_gb300.batch import Batch
    fbuild.build()
    dev = torch.device("cuda", 0)
    wl = syn.dae_constrained(n_cells=args.cells, intervals=args.steps + args.warmup)
    ks = [torch.from_numpy(np.ascontiguousarray(wl.k_at(i).T)).to(dev) for i in range(args.steps + args.warmup)]
    atol = torch.from_numpy(wl.atol).to(dev)
    b = Batch(wl.sm.mech, wl.cells.Y0, group_size=32, algorithm=Algorithm(RODAS3), mass=wl.mass)
    for i in range(args.warmup):
        b.step(ks[i], wl.dt, atol, wl.rtol)
    torch.cuda.synchronize()
    b.counts.zero_()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with Clocks(0) as clocks:
        e0.record()
        for i in range(args.steps):
            b.step(ks[args.warmup + i], wl.dt, atol, wl.rtol)
        e1.record()
        torch.cuda.synchronize()
    s = e0.elapsed_time(e1) / 1e3
    statuses = b.statuses()
    c = b.counts.cpu().numpy()
    out = {"metric": METRIC, "value": wl.cells.C * args.steps / s, "unit": "cell-intervals/s", "n_gpus": 1,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": s / args.steps * 1e3,
           "higher_is_better": True, "dtype": "f64", "data": "synthetic (seeded generator)",
           "config": {"workload": f"rodas3-dae 150+10 algebraic / 340 reactions, {wl.cells.C} cells in groups "
                                  f"of 32, dt=60 s, rtol=1e-4, projection every call"},
           "gpu_launches": args.steps, "statuses": {t: statuses.count(t) for t in set(statuses)},
           "counts_per_group_interval": {"attempts": float(c[:, 0].sum() / len(c) / args.steps),
                                         "projection_passes": float(c[:, 10].sum() / len(c) / args.steps)},
           "clocks": clocks.summary()}
    if args.adjoint_intervals > 0:
        m = args.adjoint_intervals
        Y0 = b.Y.t().contiguous()
        kk = ks[args.warmup:args.warmup + m]
        alg = Algorithm(RODAS3)

        def forward():
            fb = Batch(wl.sm.mech, Y0, group_size=32, algorithm=alg, mass=wl.mass)
            for i in range(m):
                fb.step(kk[i], wl.dt, atol, wl.rtol)
            return fb

        forward()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        forward()
        torch.cuda.synchronize()
        t_fwd = time.perf_counter() - t0
        a = 1e-14
        # a warm-up pass, then the timed one: recording forward, then the adjoint
        for rep in range(2):
            t0 = time.perf_counter()
            traj = A.forward_record(wl.sm.mech, Y0, lambda i: kk[i], wl.dt, wl.atol, wl.rtol, m, algorithm=alg,
                                    mass=wl.mass)
            torch.cuda.synchronize()
            t_rec = time.perf_counter() - t0
            Y = traj.batch.Y
            target = (Y * 1.01).clone()
            lam = 2.0 * (torch.log(Y + a) - torch.log(target + a)) / (Y + a)
            t0 = time.perf_counter()
            lam0, thbar = A.adjoint(traj, lam)
            torch.cuda.synchronize()
            t_adj = time.perf_counter() - t0
        t_fa = t_rec + t_adj
        g_th = thbar.sum(dim=1).cpu().numpy()
        rng = np.random.default_rng(13)

        def loss(Yend):
            return float(((torch.log(Yend + a) - torch.log(target + a)) ** 2).sum())

        checks = []
        for d in range(args.fd_directions):
            dth = rng.standard_normal(wl.sm.R)
            sc = [torch.from_numpy(np.exp(sg * 1e-6 * dth)).to(dev)[:, None] for sg in (1.0, -1.0)]
            fd = (loss(A.replay(traj, ks=[k * sc[0] for k in kk])) -
                  loss(A.replay(traj, ks=[k * sc[1] for k in kk]))) / 2e-6
            adj = float(np.dot(g_th, dth))
            checks.append({"fd": fd, "adjoint": adj, "rel": abs(fd - adj) / max(abs(fd), 1e-300)})
        out["adjoint"] = {"metric": "adjoint/forward cost", "value": t_fa / t_fwd, "unit": "ratio",
                          "intervals": m, "forward_s": t_fwd, "forward_plus_adjoint_s": t_fa,
                          "recording_forward_s": t_rec, "adjoint_s": t_adj,
                          "fd_checks": checks, "fd_max_rel": max((c["rel"] for c in checks), default=None)}
    return out


def run_extras(args):
    """The rest of the metric, measured in the same run on the same GPU: the
    batched uneven workload (1,048,576 cells over three mechanisms, one
    persistent launch per interval replayed as a CUDA graph), the adjoint cost
    of the 210/500 mechanism (4,096 cells, 60 intervals) and the constrained
    RODAS3 workload with its adjoint cost. Each entry is its own bench line
    (value, clocks, roofline where it has one); a failure is reported in
    place of the entry."""
    import gc
    from types import SimpleNamespace
    import torch
    extras = {}
    runs = {
        "batched": (run_batched, dict(cells=1048576, steps=10, warmup=3, kernel=args.kernel, ordering=args.ordering,
                                      autotune=True)),
        "adjoint": (run_adjoint, dict(cells=4096, steps=60, fd_directions=4)),
        "dae": (run_dae, dict(cells=16384, steps=30, warmup=3, adjoint_intervals=5, fd_directions=4)),
    }
    for name, (fn, kw) in runs.items():
        gc.collect()
        torch.cuda.empty_cache()
        t0 = time.perf_counter()
        try:
            extras[name] = fn(SimpleNamespace(**kw))
        except Exception as e:                       # report, keep the headline line
            extras[name] = {"error": f"{type(e).__name__}: {e}"}
        extras[name]["wall_s"] = time.perf_counter() - t0
    return extras


def run_reference(args, rank, world):
    """The reference's CPU path on every host core: the reference's own
    Algorithm(ROS3).solve from its installation in baseline/_ref (the oracle's
    restatement when it is not installed); each step advances one group per
    worker by one interval."""
    import multiprocessing as mp
    workers = args.cpu_workers or os.cpu_count()
    ctx = mp.get_context("spawn")
    from oracle.pool import GroupPool
    with GroupPool(ctx, workers, args.cells) as pool:
        kind = pool.kind
        for i in range(args.warmup):
            pool.step()
        pool.reset()
        t0 = time.perf_counter()
        for i in range(args.steps):
            pool.step()
        wall = time.perf_counter() - t0
    value = workers * 32 * args.steps / wall
    return {
        "metric": METRIC, "value": value, "unit": "cell-intervals/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
        "config": {"workload": "ros3-210x500 (sample)", "cells": args.cells, "group_size": 32},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "cell-intervals/s", "cores": workers, "kind": kind,
                         "sample": f"{workers} groups of 32 cells (one per process), each step one interval "
                                   f"of each, from the initial state; "
                                   + ("the unmodified reference installed in baseline/_ref" if kind == "reference"
                                      else "the oracle's restatement of the reference")},
        "e2e": {"value": value, "unit": "cell-intervals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=120)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--cells", type=int, default=65536)
    ap.add_argument("--slots", type=int, default=0)
    ap.add_argument("--kernel", default="generated", choices=["generated", "compact", "pipelined", "plain"],
                    help="generated: the mechanism's own factorization and solves as straight-line code "
                         "(compiled when the plan is made, outside the timed region); the others are "
                         "table-driven")
    ap.add_argument("--tile", type=int, default=6,
                    help="generated kernel: rows and columns of the factorization's register tiles")
    ap.add_argument("--ordering", default="auto", choices=["auto", "refined", "min_fill", "min_degree", "natural"],
                    help="elimination order of the sparse LU (auto: the greedy orders refined by local search)")
    ap.add_argument("--plain-steps", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=12)
    ap.add_argument("--cpu-intervals", type=int, default=30)
    ap.add_argument("--cpu-workers", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="plain", choices=["plain", "batched", "adjoint", "dae"],
                    help="plain: the 210/500 drop-in workload (default, the headline line); batched: the "
                         "three-mechanism persistent launch; adjoint: forward+adjoint cost; dae: the RODAS3 "
                         "constrained workload with its adjoint cost")
    ap.add_argument("--autotune", action="store_true",
                    help="batched workload: choose group size, kernel and register tile per mechanism with the "
                         "autotuner on a sample")
    ap.add_argument("--tune-tiles", default="6",
                    help="batched workload with --autotune: register tiles of the generated code to try, e.g. "
                         "4,6,8 (each one compiles the mechanism once)")
    ap.add_argument("--fd-directions", type=int, default=2,
                    help="central-difference directions checking the adjoint gradient")
    ap.add_argument("--adjoint-intervals", type=int, default=0,
                    help="dae workload: intervals of the adjoint cost measurement (0: none)")
    ap.add_argument("--no-extras", action="store_true",
                    help="plain workload: skip the batched, adjoint and constrained measurements that the "
                         "default run adds to its line")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.workload != "plain" and args.impl == "ours":
        run = {"batched": run_batched, "adjoint": run_adjoint, "dae": run_dae}[args.workload]
        print(json.dumps(run(args)))
        return
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args, rank, world)))
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    out = run_ours(args, rank, world)
    if rank == 0 and world == 1 and not args.no_extras:
        out.update(run_extras(args))
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
