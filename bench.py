#!/usr/bin/env python
"""Headline benchmark: certified Laguerre cells per second on one GB300.

Workload (one step = one pass of the cell engine plus the Lloyd update):
power diagram of 1,000,000 seeds uniform in the unit cube, weights uniform
in [0, 1e-4] (seed 0), clipped to the unit box with the security-radius
loop, FP32 clipping with FP64 re-clip of every cell FP32 cannot certify,
FP64 geometry; the seeds then move to their centroids (CVT Lloyd step,
voronoi/CVT.cpp:133-167).  Every step starts from the seeded positions,
so each step computes the same diagram (the first of the ten Lloyd
iterations of the workload) in both arms.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--ot-n N] [--ot-cpu-n N] [--extras 0|1]

Prints one JSON line.  `value` is cells/s with the seeds resident on the
GPU (CUDA events on the library's stream, L2 flushed between steps);
`e2e` is the same through the C ABI with host arrays (host->device and
device->host copies inside the timed region); `cpu_baseline` times the
CPU restatement of the reference (oracle/) on a bounded sample of the
same diagram on this machine's cores, its grid build amortised over all
the seeds.  --impl reference times that CPU implementation alone on the
same workload.  `c2_lloyd10` runs the workload's ten Lloyd iterations;
`c1` the 100k-seed Voronoi diagram in FP64 with one Lloyd step.  `ot` adds
the optimal-transport half of the headline metric: solve time from zero
weights and from the starts (learned, multilevel, separable) (--ot-n seeds of the clustered mixture,
1,000,000 by default); its `cpu_baseline` times the CPU restatement of the
solver (oracle/ot.py) on --ot-cpu-n seeds of the same mixture with the GPU
solver on the same seeds beside it.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_SEEDS = 1_000_000
# the clipping flop model (per conflict test of a plane against a corner, per
# corner created: Cramer's rule, four 3x3 determinants and three divides)
FLOP_TEST, FLOP_CORNER = 7, 59
# FP32 lanes per SM and SMs of a GB300: the CUDA-core FP32 rate is
# 2 flop x lanes x SMs x clock (no measured FP32 figure exists for the part)
FP32_LANES, N_SM = 128, 152
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch,
# captured with ncu on the 300k-seed diagram with weights on the same scale
# (U[0, 2.2e-4]) and scaled by the seeds processed to this 1M-seed launch:
# the first clipping pass moved 259.6 MB (866 B per cell), the tiled kNN
# 82.7 MB (part of its list writes were still in L2 at the end of the
# smaller launch, so this scaled figure is a lower bound)
CLIP_TRAFFIC_BYTES = 259.6e6 * N_SEEDS / 300_000
KNN_TRAFFIC_BYTES = 82.7e6 * N_SEEDS / 300_000
W_MAX = 1e-4
METRIC = ("Laguerre cells/s (power diagram, 1M seeds, FP32 clip + FP64 re-clip, "
          "Lloyd step from the seeded start)")
WORKLOAD = ("power diagram of 1M seeds uniform in [0,1]^3, weights U[0,1e-4], seed 0; "
            "certified cells (k0 = 20, security radius) clipped to the unit box, "
            "one Lloyd update; every step from the seeded positions")
# identical in both arms: the same diagram, the same per-cell work
CONFIG = {"workload": WORKLOAD, "n_seeds": N_SEEDS, "weights": "U[0,1e-4]", "seed": 0,
          "diagram": "seeded start (first of the workload's 10 Lloyd iterations)",
          "k0": 20, "certification": "security radius 4.1 R^2"}


def make_inputs(n: int, seed: int = 0):
    rng = np.random.default_rng(seed)
    x = rng.random((n, 3))
    w = rng.random(n) * W_MAX
    return x, w


class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples = []
        self._stop = threading.Event()
        self._th = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(
                    ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                     "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0 and out.stdout.strip():
                    self.samples.append([v.strip() for v in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._th = threading.Thread(target=self._run, daemon=True)
        self._th.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        if self._th:
            self._th.join(timeout=10)

    def summary(self) -> dict:
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4)
                          if len(s) > 5 + k and s[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.samples)}


def load_peaks() -> tuple[float, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def fp32_peak() -> tuple[float, str]:
    """FP32 CUDA-core rate in TFLOP/s at the part's maximum SM clock."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            mhz, kind = float(json.load(f)["sm_max_mhz"]), "measured max clock"
    except Exception:
        mhz, kind = 2070.0, "nominal max clock"
    tf = 2 * FP32_LANES * N_SM * mhz * 1e6 / 1e12
    return tf, f"nominal 2 x {FP32_LANES} lanes x {N_SM} SMs at {mhz:.0f} MHz ({kind})"


def cpu_sample(pc, i0: int, m: int, cores: int) -> tuple[float, float]:
    """Seconds for cells [i0, i0 + m) of the prepared diagram plus their
    share of the grid build, and the sample's mean clips per cell."""
    r = pc.range(i0, i0 + m, cores)
    # the Lloyd update of the sample (CVT.cpp:133-167: seeds of empty cells stay)
    m_ = r["vol"][:, None]
    xs = np.where(m_ > 1e-30, r["mg"].reshape(-1, 3) / np.where(m_ > 1e-30, m_, 1.0), 0.0)
    del xs
    return r["seconds"] + pc.build_seconds * m / pc.n, r["mean_clips"]


def cpu_baseline(x: np.ndarray, w: np.ndarray, sample: int) -> dict:
    """The oracle (CPU restatement of the reference path) on cells [0, sample)
    of the same diagram, with every host core."""
    from oracle import oracle
    cores = os.cpu_count() or 1
    pc = oracle.PreparedCells(x, w)
    dt, clips = cpu_sample(pc, 0, sample, cores)
    pc.close()
    return {"value": sample / dt, "unit": "cells/s", "cores": cores, "kind": "port",
            "mean_clips": clips,
            "sample": f"cells 0..{sample} of the {len(x)}-seed power diagram at the seeded "
                      f"start (all seeds as neighbours), oracle/gbv_oracle.c with {cores} "
                      f"threads, {dt:.2f} s incl. the grid build's share"}


def max_over_ranks(x: float) -> float:
    """Maximum of x over the ranks of the process group (x if no group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    dev = (torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl"
           else torch.device("cpu"))
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    x, w = make_inputs(N_SEEDS)
    from oracle import oracle
    cores = os.cpu_count() or 1
    m = args.ref_sample
    pc = oracle.PreparedCells(x, w)
    for s in range(args.warmup):
        cpu_sample(pc, (s * m) % (N_SEEDS - m), m, cores)
    times, clips = [], []
    for s in range(args.steps):
        i0 = ((s + args.warmup) * m) % (N_SEEDS - m)
        dt, cl = cpu_sample(pc, i0, m, cores)
        times.append(dt)
        clips.append(cl)
    pc.close()
    total = sum(times)
    value = m * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "cells/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded numpy)",
        "config": dict(CONFIG),
        "mean_clips": statistics.mean(clips),
        "timing": {"sample_cells_per_step": m, "grid_build_s": pc.build_seconds,
                   "grid_build": "once, amortised: each step adds build_s * m / n"},
        "cpu_baseline": {"value": value, "unit": "cells/s", "cores": cores, "kind": "port",
                         "sample": f"{m} cells per step of the {N_SEEDS}-seed power diagram at "
                                   f"the seeded start, oracle/gbv_oracle.c with {cores} "
                                   f"threads"},
        "e2e": {"value": value, "unit": "cells/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args) -> None:
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    import geogram_gb300 as g
    from geogram_gb300 import _lib
    ctx = g.Context(local)
    lib = _lib.load()
    x_h, w_h = make_inputs(N_SEEDS, seed=rank)
    x0 = torch.from_numpy(x_h).to(dev)
    x = x0.clone()
    w = torch.from_numpy(w_h).to(dev)
    stream = torch.cuda.current_stream(dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        return g.lloyd_iterations(x, 1, w, precision=args.precision, stream=stream, ctx=ctx)

    for _ in range(args.warmup):
        x.copy_(x0)
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = lib.gbv_kernel_launches()
    reports = []
    ev_s = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev_e = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        for s in range(args.steps):
            x.copy_(x0)           # the seeded positions again, outside the events
            flush.fill_(float(s))  # L2 flush (256 MB > 126 MB L2), outside the events
            ev_s[s].record(stream)
            reports.append(step())
            ev_e[s].record(stream)
        torch.cuda.synchronize()
    launches = lib.gbv_kernel_launches() - launches0
    if world > 1:
        dist.barrier()
    step_ms = [a.elapsed_time(b) for a, b in zip(ev_s, ev_e)]
    total_ms = max_over_ranks(sum(step_ms))
    value = world * N_SEEDS * args.steps / (total_ms / 1e3)

    # ---- e2e through the C ABI with host arrays (H2D + compute + D2H),
    # every step from the seeded positions
    e2e_t = []
    for s in range(max(3, args.steps // 2)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        g.lloyd_step(x_h, w_h, precision=args.precision, ctx=ctx)
        e2e_t.append(time.perf_counter() - t0)
    e2e_value = world * N_SEEDS / statistics.mean(e2e_t[1:])

    if rank == 0:
        # ---- the dominant kernel: the first FP32 clipping pass over every
        # cell (clip_kernel<float,64,32>), FP32-pipe bound.  Algorithmic flops
        # = 7 per conflict test + 59 per corner created, counted by the kernel
        # itself; its time from the library's CUDA events around that launch
        rep = reports[-1]
        clip_ms = statistics.median(r["ms_clip_kernel"] for r in reports)
        clip_flop = FLOP_TEST * rep["n_conflict_tests"] + FLOP_CORNER * rep["n_corners_created"]
        clip_tf = clip_flop / (clip_ms / 1e3) / 1e12
        tf_peak, tf_kind = fp32_peak()
        # ---- kNN (HBM): algorithmic bytes per seed = query float4 (16) + k
        # list entries (4 k) + count, last (d2, index) (16) + the Morton
        # counting sort (48), timed by the library's events (grid + kNN)
        k = rep["knn_k"]
        bytes_per_seed = 16 + 4 * k + 16 + 48
        knn_ms = statistics.median(r["ms_knn"] + r["ms_grid"] for r in reports)
        achieved = bytes_per_seed * N_SEEDS / (knn_ms / 1e3) / 1e9
        peak, peak_kind = load_peaks()
        # ---- plain FP64 path on the same seeds, and the error of this mode
        # against it (both modes reproduce the reference's FP64 results)
        torch.cuda.synchronize()
        g.compute_cells_device(x0, w, precision=args.precision, stream=stream, ctx=ctx)
        c32 = g.device_results(ctx)
        g.compute_cells_device(x0, w, precision="fp64", stream=stream, ctx=ctx)
        c64 = g.device_results(ctx)
        t64 = []
        for _ in range(3):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.compute_cells_device(x0, w, precision="fp64", stream=stream, ctx=ctx)
            e1.record(stream)
            torch.cuda.synchronize()
            t64.append(e0.elapsed_time(e1))
        fp64_cps = N_SEEDS / (statistics.median(t64) / 1e3)
        # ---- the FP32-geometry mode (same cells, FP32 volumes / centroids /
        # areas) on the same seeds, and its error against the FP64 path
        t3g = []
        for _ in range(3):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g.compute_cells_device(x0, w, precision="fp32_geometry", stream=stream, ctx=ctx)
            e1.record(stream)
            torch.cuda.synchronize()
            t3g.append(e0.elapsed_time(e1))
        cg = g.device_results(ctx)
        # errors per cell against s_i = max(its FP64 volume, the mean volume)
        s_i = np.maximum(c64["volume"], 1.0 / N_SEEDS)
        cell_of = np.repeat(np.arange(N_SEEDS), np.diff(c64["rowptr"].astype(np.int64)))
        live = c64["volume"] > 0
        geom32 = {
            "cells_per_s": N_SEEDS / (statistics.median(t3g) / 1e3),
            "ms": statistics.median(t3g),
            "speedup_vs_fp64_plain": statistics.median(t64) / statistics.median(t3g),
            "max_vol_err_vs_fp64_per_s": float(
                np.max(np.abs(cg["volume"] - c64["volume"]) / s_i)),
            "max_mg_err_vs_fp64_per_s": float(
                np.max(np.abs(cg["mg"] - c64["mg"]).max(axis=1) / s_i)),
            "max_area_err_vs_fp64_per_s_2_3": float(
                np.max(np.abs(cg["facet_area"] - c64["facet_area"]) / s_i[cell_of] ** (2 / 3))),
            "median_rel_vol_err_vs_fp64": float(np.median(
                np.abs(cg["volume"][live] - c64["volume"][live]) / c64["volume"][live])),
            "neighbour_lists_identical": bool(
                np.array_equal(cg["rowptr"], c64["rowptr"]) and
                np.array_equal(cg["neighbors"], c64["neighbors"])),
        }
        t32 = statistics.median(r["ms_total"] for r in reports)
        rel_vol = float(np.max(np.abs(c32["volume"] - c64["volume"]) /
                               np.maximum(np.abs(c64["volume"]), 1e-300)))
        abs_mg = float(np.max(np.abs(c32["mg"] - c64["mg"])))
        same_nbr = bool(np.array_equal(c32["rowptr"], c64["rowptr"]) and
                        np.array_equal(c32["neighbors"], c64["neighbors"]))
        cpu = cpu_baseline(x_h, w_h, args.cpu_sample)
        line = {
            "metric": METRIC, "value": value, "unit": "cells/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64",
            "data": "synthetic (seeded numpy, uniform seeds and weights)",
            "config": dict(CONFIG),
            "mean_clips": rep["mean_clips"],
            "timing": {"precision": args.precision, "l2": "flushed between steps (256 MB write)",
                       "seeds": "reset to the seeded positions before each step, outside "
                                "the timed region",
                       "parallelism": "replicas only" if world > 1 else "1 GPU"},
            "roofline": {"kernel": "clip_kernel<float,64,32> (first clipping pass, all cells)",
                         "bound": "fp32", "achieved": clip_tf, "peak": tf_peak,
                         "unit": "TFLOP/s", "frac": clip_tf / tf_peak, "peak_kind": tf_kind,
                         "ms": clip_ms, "flop": clip_flop,
                         "counts": {"conflict_tests": rep["n_conflict_tests"],
                                    "corners_created": rep["n_corners_created"],
                                    "flop_per_test": FLOP_TEST,
                                    "flop_per_corner": FLOP_CORNER},
                         "traffic": CLIP_TRAFFIC_BYTES},
            "roofline_knn": {"kernel": "grid + knn_tile_kernel + flagged exact queries",
                             "bound": "hbm", "achieved": achieved, "peak": peak,
                             "unit": "GB/s", "frac": achieved / peak,
                             "peak_kind": peak_kind + " (hbm_gbs)", "ms": knn_ms,
                             "bytes_per_seed": bytes_per_seed, "k": k,
                             "traffic": KNN_TRAFFIC_BYTES},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "cells/s",
                    "h2d_bytes_per_step": 32 * N_SEEDS, "d2h_bytes_per_step": 24 * N_SEEDS},
            "gpu_launches": int(launches),
            "clocks": clk.summary(),
            "phases_ms": {kk: round(statistics.median(r[kk] for r in reports), 3)
                          for kk in ("ms_grid", "ms_knn", "ms_clip", "ms_clip_kernel",
                                     "ms_retry", "ms_total")},
            "cells": {kk: rep[kk] for kk in ("n_recheck_fp64", "n_more_k", "n_overflow",
                                             "n_exact", "n_knn_exact", "mean_clips",
                                             "max_clips", "nnz", "knn_k")},
            "fp64_plain": {"cells_per_s": fp64_cps, "ms": statistics.median(t64),
                           "speedup_of_this_mode": statistics.median(t64) / t32,
                           "max_rel_vol_err_vs_fp64": rel_vol, "max_abs_mg_err_vs_fp64": abs_mg,
                           "neighbour_lists_identical": same_nbr},
            "fp32_geometry": geom32,
        }
        if args.extras:
            line["c2_lloyd10"] = run_lloyd10(x0, w, args.precision, stream, ctx, flush)
            line["c1"] = run_c1(ctx, stream)
        if args.ot_n > 0:
            line["ot"] = run_ot(args.ot_n, ctx)
            if args.ot_cpu_n > 0:
                try:
                    line["ot"]["cpu_baseline"] = ot_cpu_baseline(args.ot_cpu_n, ctx)
                except Exception as e:  # a reported baseline: never lose the line for it
                    line["ot"]["cpu_baseline"] = {"error": f"{type(e).__name__}: {e}"}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()


def run_lloyd10(x0, w, precision: str, stream, ctx, flush) -> dict:
    """The workload as written: ten Lloyd iterations from the seeded start,
    each timed with CUDA events (L2 flushed before each)."""
    import torch
    import geogram_gb300 as g
    x = x0.clone()
    ms, clips = [], []
    for _ in range(10):
        flush.fill_(2.0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = g.lloyd_iterations(x, 1, w, precision=precision, stream=stream, ctx=ctx)
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
        clips.append(round(r["mean_clips"], 3))
    return {"iterations": 10, "total_ms": sum(ms), "ms_per_iteration": [round(v, 3) for v in ms],
            "mean_clips_per_iteration": clips,
            "cells_per_s": 10 * len(x0) / (sum(ms) / 1e3)}


def run_c1(ctx, stream) -> dict:
    """100k seeds uniform in the unit cube (seed 0), Voronoi (zero weights),
    FP64, k0 = 20 with security-radius growth, one Lloyd step: GPU time, and
    the CPU restatement on all its cells with every host core."""
    import torch
    import geogram_gb300 as g
    from oracle import oracle
    n = 100_000
    xh = np.random.default_rng(0).random((n, 3))
    x0 = torch.from_numpy(xh).cuda()
    x = x0.clone()
    ms = []
    for s in range(8):
        x.copy_(x0)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = g.lloyd_iterations(x, 1, None, precision="fp64", stream=stream, ctx=ctx)
        e1.record(stream)
        torch.cuda.synchronize()
        if s >= 3:
            ms.append(e0.elapsed_time(e1))
    cores = os.cpu_count() or 1
    pc = oracle.PreparedCells(xh, None)
    out = pc.range(0, n, cores)
    cpu_s = out["seconds"] + pc.build_seconds
    pc.close()
    gpu_ms = statistics.median(ms)
    return {"workload": "Voronoi of 100k seeds U[0,1]^3 (seed 0), FP64, k0 = 20 + security "
                        "radius, one Lloyd step",
            "gpu_ms": gpu_ms, "gpu_cells_per_s": n / (gpu_ms / 1e3),
            "mean_clips": r["mean_clips"],
            "cpu_baseline": {"kind": "port", "cores": cores, "seconds": cpu_s,
                             "cells_per_s": n / cpu_s, "mean_clips": out["mean_clips"],
                             "sample": "all 100k cells, grid build included"}}


def gaussian_mixture(n: int, k: int, sigma: float, rng: np.random.Generator) -> np.ndarray:
    """n seeds from k isotropic Gaussians (means uniform in [0.2, 0.8]^3,
    standard deviation sigma), rejected outside the unit cube."""
    mu = rng.uniform(0.2, 0.8, (k, 3))
    out, have = [], 0
    while have < n:
        c = rng.integers(0, k, n)
        p = mu[c] + sigma * rng.standard_normal((n, 3))
        p = p[((p > 0.0) & (p < 1.0)).all(1)]
        out.append(p)
        have += len(p)
    return np.concatenate(out)[:n]


def run_ot(n: int, ctx) -> dict:
    """Semi-discrete OT to the uniform measure on the unit cube (nu_i = 1/n)
    of n seeds from an 8-component Gaussian mixture (sigma 0.05, seed 0),
    damped Newton + FP64 CG to a relative mass error of 1e-6: from zero
    weights and from the learned start.  Wall time on the host around each
    solve (everything runs on the GPU; the learned start includes its
    features, network and solve)."""
    import torch
    import geogram_gb300 as g
    from geogram_gb300.warmstart import WarmStartModel
    x = torch.tensor(gaussian_mixture(n, 8, 0.05, np.random.default_rng(0)), device="cuda")
    model = WarmStartModel.load()

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rep = fn()
        torch.cuda.synchronize()
        return rep, time.perf_counter() - t0

    keys = ("newton_iters", "cell_calls", "cg_iters", "halvings", "converged", "mass_error_inf")
    w = torch.zeros(n, dtype=torch.float64, device="cuda")
    rp, tp = timed(lambda: g.ot_solve_device(x, w, tol=1e-6, ctx=ctx))
    w2 = torch.empty(n, dtype=torch.float64, device="cuda")
    rl, tl = timed(lambda: model.solve(x, w2, tol=1e-6, ctx=ctx))
    w3 = torch.empty(n, dtype=torch.float64, device="cuda")
    rv, tv = timed(lambda: g.ot_solve_levels_device(x, w3, ratio=8, min_level=20000, tol=1e-6,
                                                    ctx=ctx))

    def separable():
        w4 = g.ot_separable_start_device(x, ctx=ctx)
        return g.ot_solve_device(x, w4, tol=1e-6, ctx=ctx)
    rs, ts = timed(separable)
    plain = {k: rp[k] for k in keys}
    plain["seconds"] = tp
    learned = {k: rl[k] for k in keys}
    learned.update(seconds=tl, start_ms=rl["ms_start"], start_scale=rl["start_scale"])
    levels = {k: rv[k] for k in keys}
    levels.update(seconds=tv, levels=rv["levels"], start_scale=rv["start_scale"])
    sep = {k: rs[k] for k in keys}
    sep.update(seconds=ts, start_scale=rs["start_scale"])
    return {"workload": f"OT of {n} seeds, 8-component Gaussian mixture (means U[0.2,0.8]^3, "
                        "sigma 0.05, seed 0) to the uniform measure on the unit cube, "
                        "relative mass error 1e-6",
            "n": n, "plain": plain, "learned_start": learned, "speedup": tp / tl,
            "multilevel": levels, "multilevel_speedup": tp / tv,
            "separable_start": sep, "separable_speedup": tp / ts}


def ot_cpu_baseline(n: int, ctx) -> dict:
    """The OT restatement (oracle/ot.py: exact Laguerre cells, damped Newton,
    Jacobi PCG) on the host with every core, on a bounded sample: n seeds of
    the same mixture; the GPU solver on the same seeds beside it."""
    import torch
    import geogram_gb300 as g
    from oracle import ot
    cores = os.cpu_count() or 1
    x = gaussian_mixture(n, 8, 0.05, np.random.default_rng(0))
    t0 = time.perf_counter()
    _, info = ot.newton(x, tol=1e-6, nthreads=cores)
    t_cpu = time.perf_counter() - t0
    xd = torch.tensor(x, device="cuda")
    wd = torch.zeros(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    rep = g.ot_solve_device(xd, wd, tol=1e-6, ctx=ctx)
    torch.cuda.synchronize()
    t_gpu = time.perf_counter() - t0
    return {"kind": "restatement", "cores": cores, "n": n, "seconds": t_cpu,
            "newton_iters": info["iters"], "converged": info["converged"],
            "gpu_seconds_same_seeds": t_gpu, "gpu_newton_iters": rep["newton_iters"],
            "sample": f"OT of {n} seeds of the same mixture (seed 0) to mass error 1e-6, "
                      f"oracle/ot.py on oracle/gbv_oracle.c with {cores} threads"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--precision", default="fp32")
    ap.add_argument("--cpu-sample", type=int, default=200_000)
    ap.add_argument("--ref-sample", type=int, default=50_000)
    ap.add_argument("--ot-n", type=int, default=1_000_000,
                    help="seeds of the optimal-transport comparison (0: skip)")
    ap.add_argument("--extras", type=int, default=1,
                    help="1: add the ten-iteration workload and the 100k Voronoi line")
    ap.add_argument("--ot-cpu-n", type=int, default=2000,
                    help="seeds of the CPU optimal-transport baseline sample (0: skip)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
