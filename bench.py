"""Benchmark of the SIPG DG operator apply (dune-fem's GalerkinOperator apply).

Workload (one "step" = one operator apply w = A u over the whole grid):
3-D unit cube, 64^3 hexahedra, DG Q3 Legendre (64 dofs/cell, 16,777,216
dofs), SIPG Laplacian with penalty 10 (p+1)^2 = 160, (p+2)^3 = 125 Gauss points
per cell, weak homogeneous Dirichlet, FP64 dof vector i.i.d. uniform[-1,1]
from seed 20261203 (synthetic, seeded).  u and w (268 MB together) exceed the
129 MB L2, so no flush is done between applies.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbfem|reference]

Prints one JSON line.  --impl reference times the CPU restatement of the
reference's algorithm (oracle/, dense per-element evaluation, all host
threads) on a bounded sample of cells per step.
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
sys.path.insert(0, os.path.join(ROOT, "dune-fem_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

CELLS = (64, 64, 64)
ORDER = 3
QUAD = ORDER + 2
SEED = 20261203
METRIC = "SIPG apply DoF/s"
UNIT = "DoF/s"
BYTES_PER_DOF = 16.0          # read u (8) + write w (8), geometry recomputed, tables on chip
FLOP_PER_DOF = 402.0          # sum-factorised SIPG Q3, q=5 (volume + faces)
CONFIG = {"workload": "SIPG DG Q3 apply, 3-D unit cube 64^3 hexes, 16.8M dofs, q=5, penalty 160, FP64",
          "cells": list(CELLS), "order": ORDER, "quad_points": QUAD, "dofs": 64 ** 3 * 64,
          "l2": "inputs exceed L2 (u + w = 268 MB > 129 MB), no flush"}


def load_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True,
                                     timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if "Active" in s[3 + i]
                          and not s[3 + i].startswith("Not")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, world):
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return x


def cpu_sample_rate(prob, u, seconds, nthreads):
    """DoF/s of the oracle apply on a bounded sample: contiguous cell ranges
    (whole z-slabs) until `seconds` of CPU work have passed."""
    w = np.zeros(prob.ndofs)
    slab = CELLS[0] * CELLS[1]
    done_cells = 0
    t0 = time.perf_counter()
    c0 = 0
    while True:
        c1 = min(c0 + slab, prob.ncells)
        prob.apply_cells(u, w, c0, c1, nthreads=nthreads)
        done_cells += c1 - c0
        c0 = c1 % prob.ncells
        el = time.perf_counter() - t0
        if el >= seconds:
            break
    return done_cells * prob.nloc / el, done_cells


def run_reference(args, world, rank):
    if rank != 0:
        return
    import oracle
    prob = oracle.DGProblem(CELLS, ORDER, quad_points=QUAD)
    u = np.random.default_rng(SEED).uniform(-1.0, 1.0, prob.ndofs)
    nthreads = os.cpu_count() or 1
    per_step = max(0.05, min(2.0, 90.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        cpu_sample_rate(prob, u, per_step, nthreads)
    rates, cells = [], 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        r, c = cpu_sample_rate(prob, u, per_step, nthreads)
        rates.append(r)
        cells += c
    el = time.perf_counter() - t0
    value = cells * prob.nloc / el
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": CONFIG, "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": "per step: whole 64x64-cell z-slabs of the 64^3 grid applied by the "
                                       "oracle (dense per-element evaluation as dune-fem's GalerkinOperator) "
                                       "for ~%.2f s" % per_step},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_gpu(args, world, rank, local):
    import gbfem
    peaks, peak_kind = load_peaks()
    op = gbfem.DGOperator(CELLS, ORDER, quad_points=QUAD)
    n = op.size
    u_h = np.random.default_rng(SEED + rank).uniform(-1.0, 1.0, n)
    u = gbfem.DeviceArray.from_numpy(u_h)
    w = gbfem.DeviceArray(n)
    import torch
    torch.cuda.set_device(local)
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream
    for _ in range(args.warmup):
        op(u, w, sptr)
    torch.cuda.synchronize()
    barrier(world)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            op(u, w, sptr)
        e1.record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ms = e0.elapsed_time(e1)
    ms = allreduce_max(ms, world)
    ms_step = ms / args.steps
    value = world * n / (ms_step * 1e-3)

    # end to end through the host-buffer C-ABI call: H2D of u, apply, D2H of w per step
    uh = torch.from_numpy(u_h).pin_memory()
    wh = torch.empty(n, dtype=torch.float64).pin_memory()
    uh_np, wh_np = uh.numpy(), wh.numpy()
    e2e_steps = max(3, min(args.steps, 50))
    op.apply_host(uh_np, wh_np)
    torch.cuda.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        op.apply_host(uh_np, wh_np)
    el = time.perf_counter() - t0
    el = allreduce_max(el, world)
    e2e_value = world * n * e2e_steps / el
    if rank != 0:
        return

    fp64_peak, fp32_peak = gbfem.measure_fma_peaks()
    achieved_gbs = BYTES_PER_DOF * n / (ms_step * 1e-3) / 1e9
    achieved_tflops = FLOP_PER_DOF * n / (ms_step * 1e-3) / 1e12
    traffic = None
    prof = os.path.join(ROOT, "profiles", "dg_apply_q3_64cube_f64.json")
    if os.path.exists(prof):
        with open(prof) as f:
            traffic = json.load(f).get("dram_bytes_per_launch")
    # CPU baseline: the oracle on this host's cores, bounded sample (~15 s)
    import oracle
    prob = oracle.DGProblem(CELLS, ORDER, quad_points=QUAD)
    nthreads = os.cpu_count() or 1
    cpu_rate, cpu_cells = cpu_sample_rate(prob, u_h, 15.0, nthreads)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded uniform[-1,1] dofs)",
            "config": dict(CONFIG, parallelism="replicas" if world > 1 else "single GPU"),
            "gpu_launches": args.steps,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n,
                    "steps": e2e_steps, "path": "gbfem_operator_apply_host (pinned host buffers)"},
            "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": achieved_gbs / peaks["hbm_gbs"], "traffic": traffic,
                         "peak_source": peak_kind, "algorithmic_bytes_per_dof": BYTES_PER_DOF},
            "fp64_pipe": {"achieved_tflops": achieved_tflops, "peak_tflops_measured": fp64_peak,
                          "frac": achieved_tflops / fp64_peak if fp64_peak else None,
                          "algorithmic_flop_per_dof": FLOP_PER_DOF, "fp32_peak_tflops_measured": fp32_peak},
            "cpu_baseline": {"value": cpu_rate, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": "%d cells (whole z-slabs) of the 64^3 grid applied by the oracle "
                                       "(dense per-element evaluation as dune-fem's GalerkinOperator), ~15 s"
                                       % cpu_cells},
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gbfem", choices=["gbfem", "reference"])
    args = ap.parse_args()
    world, rank, local = dist_init() if args.impl == "gbfem" else (
        int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank, local)


if __name__ == "__main__":
    main()
