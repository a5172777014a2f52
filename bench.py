"""Benchmark of the SIPG DG operator apply (dune-fem's GalerkinOperator apply).

Workload (one "step" = one operator apply w = A u over the whole grid):
3-D unit cube, 64^3 hexahedra, DG Q3 Legendre (64 dofs/cell, 16,777,216
dofs), SIPG Laplacian with penalty 10 (p+1)^2 = 160, (p+2)^3 = 125 Gauss points
per cell, weak homogeneous Dirichlet, FP64 dof vector i.i.d. uniform[-1,1]
from seed 20261203 (synthetic, seeded).  u and w (268 MB together) exceed the
129 MB L2, so no flush is done between applies.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gbfem|reference]

Prints one JSON line.  Its "solve" object is the metric's second half: the
time to relative residual 1e-10 of the mixed FP32-in-FP64 solve against FP64
block-Jacobi CG on the variable-kappa SIPG Q3 problem at 64^3 (about a
minute; --no-solve skips it).  --impl reference times the CPU restatement of the
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
FLOP_PER_DOF = 402.0          # sum-factorised SIPG Q3, q=5 (volume + faces), the algorithmic count
# flops the closed-form kernels execute per cell (n = 4, constant kappa, no
# mass, no advection; an FMA counts 2), divided by n^3:
#  traces: 3 n^2 lines x (even/odd partial sums of v and P: 4 FMA + 2 MUL,
#          u_0 enters both even sums as is; 4 adds for the two faces) = 48 x 14
#  fluxes: 6 n^2 face points x 2 (J = v- - v+, P- - P+)             = 96 x 2
#  lines:  n^2 lines per axis x (4 adds + 2 x (5 structural nonzeros of M_d
#          + 7 face-expansion FMAs))                                = 48 x 28
KERNEL_FLOP_PER_DOF = (48 * 14 + 96 * 2 + 48 * (4 + 2 * (5 + 7))) / 64.0  # = 34.5
# FP64 instructions per dof, which is what the FP64 pipe issues (an add takes
# the slot of an FMA): (48 x 10 + 96 x 2 + 48 x 16) / 64
KERNEL_FP64_INSTR_PER_DOF = (48 * 10 + 96 * 2 + 48 * 16) / 64.0  # = 22.5
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


def allreduce_max(x, world, device="cuda"):
    """Max over ranks of a per-rank time (the replicas' job time)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([x], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return x


def fma_peaks():
    """FP64 and FP32 FMA-pipe peaks (TFLOP/s) of the current GPU, from the
    benchmark-only microbenchmark library built beside libgbfem."""
    import ctypes as C
    L = C.CDLL(os.path.join(ROOT, "dune-fem_gb300", "lib", "libgbfem_bench.so"))
    L.gbfem_bench_fma_peaks.argtypes = [C.POINTER(C.c_double), C.POINTER(C.c_double)]
    a, b = C.c_double(), C.c_double()
    rc = L.gbfem_bench_fma_peaks(C.byref(a), C.byref(b))
    if rc != 0:
        raise RuntimeError("FMA peak microbenchmark failed: CUDA error %d" % rc)
    return a.value, b.value


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


SOLVE_CELLS, SOLVE_ORDER, SOLVE_SEED = 64, 3, 1


def solve_comparison():
    """The solve half of the metric: time to relative residual ||f - A u|| /
    ||f|| <= 1e-10 on the variable-kappa SIPG Q3 problem at 64^3 (the
    learned-preconditioner configuration's grid and coefficient field, kappa
    seed 1; f = 1, u = 0 weak Dirichlet), each arm from u = 0 including its
    preconditioner set-up:
    - fp64: FP64 CG with FP64 block Jacobi, stopping on the unpreconditioned
      residual (the reference's CG stops on <r, B r>, which here leaves a
      true residual near 1.6e-9);
    - mixed: FP64 FGMRES on the full kappa around an FP32 inner CG on the
      cellwise-kappa operator (kappa's cell means) with the scaled shared-block
      Jacobi; the outer residual is FP64.
    Reports times, iterations, the true residuals (FP64 apply on the GPU),
    the mixed solution's max-norm difference from the FP64 one and the clocks
    of each arm."""
    import torch
    import gbfem
    N, p = SOLVE_CELLS, SOLVE_ORDER
    cells = (N, N, N)
    modes = gbfem.fourier_modes(SOLVE_SEED, 256, 0.1, 1.0)
    k64 = gbfem.project(cells, p, gbfem.FN_EXP_FOURIER, modes=modes)
    k32 = gbfem.project(cells, p, gbfem.FN_EXP_FOURIER, modes=modes, precision=gbfem.F32)
    f = gbfem.project(cells, p, gbfem.FN_CONSTANT, params=(1.0,), scale_by_volume=True)
    op64 = gbfem.DGOperator(cells, p, kappa=k64)
    op32c = gbfem.DGOperator(cells, p, precision=gbfem.F32, kappa_cell=gbfem.cell_means(k32, p))
    fh = f.numpy()
    fn = float(np.linalg.norm(fh))

    def true_rel(u):
        au = gbfem.DeviceArray(op64.size)
        op64(u, au)
        return float(np.linalg.norm(fh - au.numpy()) / fn)

    out = {"workload": "SIPG Q3 %d^3 (%d dofs), -div(kappa grad u) = 1, u = 0 weak, log kappa ~ 256 Fourier "
                       "modes (std 1, corr 0.1), seed %d; to ||f - A u|| / ||f|| <= 1e-10" % (N, op64.size, SOLVE_SEED),
           "unit": "s"}
    u_mix = gbfem.DeviceArray(op64.size)
    u_mix.clear()
    with ClockSampler(0) as clk_m:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pcs = gbfem.Preconditioner.scaled_block_jacobi(op32c)
        torch.cuda.synchronize()
        t_setup = time.perf_counter() - t0
        info = gbfem.solve_mixed(op64, op32c, pcs, f, u_mix, tolerance=1e-10, inner_tolerance=1e-2,
                                 max_outer=300, outer="fgmres", outer_restart=30, graph_chunk=16)
        torch.cuda.synchronize()
        t_mix = time.perf_counter() - t0
    out["mixed"] = {"time_s": t_mix, "setup_s": t_setup, "converged": bool(info.converged),
                    "outer_iterations": info.outer_iterations, "inner_iterations": info.iterations,
                    "stagnated": bool(info.stagnated), "true_rel_residual": true_rel(u_mix),
                    "method": "FP64 FGMRES(30) outer on the full kappa; FP32 CG inner (rel. tol 1e-2, device-resident "
                              "loop in graph chunks of 16) on the cellwise-kappa one-kernel closed form with the "
                              "scaled shared-block Jacobi",
                    "clocks": clk_m.summary()}
    del pcs
    u64 = gbfem.DeviceArray(op64.size)
    u64.clear()
    with ClockSampler(0) as clk_d:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pc64 = gbfem.Preconditioner.block_jacobi(op64)
        torch.cuda.synchronize()
        t_setup64 = time.perf_counter() - t0
        inv = gbfem.KrylovInverseOperator("cg", tolerance=1e-10, error_measure=gbfem.RELATIVE_RESIDUAL,
                                          max_iterations=20000)
        inv.bind(op64, pc64)
        # CG's recursively updated residual drifts from f - A u (here by about
        # 1e-9 ||f||), so a cycle that stops at 1e-10 can end above it: the
        # solve is applied again from its iterate (a new cycle starts from the
        # true residual f - A u, cg.hh:36-47) until the true residual is below
        # the tolerance; the true-residual checks are inside the timed region
        cycles, iters, rel = [], 0, None
        for _ in range(4):
            inv(f, u64)
            i64 = inv.info()
            iters += abs(i64["iterations"])
            rel = true_rel(u64)
            cycles.append({"iterations": i64["iterations"], "true_rel_residual": rel})
            if rel <= 1e-10 or not i64["converged"]:
                break
        torch.cuda.synchronize()
        t64 = time.perf_counter() - t0
    out["fp64"] = {"time_s": t64, "setup_s": t_setup64, "converged": bool(rel <= 1e-10),
                   "iterations": iters, "cycles": cycles, "true_rel_residual": rel,
                   "method": "FP64 CG + FP64 block Jacobi (dense cell blocks), stop on the unpreconditioned residual, "
                             "restarted from the iterate while the true residual is above the tolerance",
                   "clocks": clk_d.summary()}
    a, b = u_mix.numpy(), u64.numpy()
    out["mixed_vs_fp64_rel_max_diff"] = float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    out["speedup_mixed_vs_fp64"] = t64 / t_mix
    return out


def profiled_traffic(path):
    """DRAM bytes of one headline apply from the committed ncu summary:
    (both kernels: trace pass + main kernel, main kernel alone, launch-list
    share of the main kernel), or (None, None, None) without the file."""
    if not os.path.exists(path):
        return None, None, None
    with open(path) as f:
        d = json.load(f)
    main = d.get("dram_bytes_per_launch")
    t = d.get("trace_kernel") or {}
    step = None
    if main is not None and "dram_read" in t and "dram_write" in t:
        step = int(main + t["dram_read"] + t["dram_write"])
    share = (d.get("launch_list_share") or {}).get("dg_const_kernel")
    return step, main, share


def time_applies(op, u, w, steps, stream):
    import torch
    sptr = stream.cuda_stream
    for _ in range(3):
        op(u, w, sptr)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        op(u, w, sptr)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def run_gpu(args, world, rank, local):
    import gbfem
    peaks, peak_kind = load_peaks()
    # default algorithm: constant kappa -> the closed form of the q=5 quadrature
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
    # the same call with the kernels reading / writing the host buffers in
    # place over NVLink-C2C instead of the copy pipeline
    op.set_host_transfer(True)
    op.apply_host(uh_np, wh_np)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        op.apply_host(uh_np, wh_np)
    e2e_in_place = world * n * e2e_steps / allreduce_max(time.perf_counter() - t0, world)
    op.set_host_transfer(False)
    if rank != 0:
        return

    # the Gauss-point quadrature kernel on the same input (variable-kappa path), for reference
    opq = gbfem.DGOperator(CELLS, ORDER, quad_points=QUAD, algorithm=gbfem.ALGO_QUADRATURE)
    wq = gbfem.DeviceArray(n)
    ms_quad = time_applies(opq, u, wq, max(3, min(args.steps, 20)), stream)
    wa, wb = w.numpy(), wq.numpy()
    quad_rel = float(np.max(np.abs(wa - wb)) / np.max(np.abs(wb)))
    op32 = gbfem.DGOperator(CELLS, ORDER, quad_points=QUAD, precision=gbfem.F32)
    u32 = gbfem.convert(u, gbfem.F32)
    w32 = gbfem.DeviceArray(n, gbfem.F32)
    ms_f32 = time_applies(op32, u32, w32, max(3, min(args.steps, 50)), stream)
    op32t = gbfem.DGOperator(CELLS, ORDER, quad_points=QUAD, precision=gbfem.F32, algorithm=gbfem.ALGO_TRACE_PASS)
    ms_f32_two = time_applies(op32t, u32, w32, max(3, min(args.steps, 50)), stream)
    del opq, wq, op32, op32t, u32, w32

    fp64_peak, fp32_peak = fma_peaks()
    achieved_gbs = BYTES_PER_DOF * n / (ms_step * 1e-3) / 1e9
    achieved_tflops = KERNEL_FLOP_PER_DOF * n / (ms_step * 1e-3) / 1e12
    traffic, traffic_main, main_share = profiled_traffic(
        os.path.join(ROOT, "profiles", "dg_trace_const_q3_64cube_f64.json"))
    # CPU baseline: the oracle on this host's cores, bounded sample (~15 s)
    import oracle
    prob = oracle.DGProblem(CELLS, ORDER, quad_points=QUAD)
    nthreads = os.cpu_count() or 1
    cpu_rate, cpu_cells = cpu_sample_rate(prob, u_h, 15.0, nthreads)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded uniform[-1,1] dofs)",
            "config": CONFIG,
            "gpu_launches": 2 * args.steps,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n,
                    "steps": e2e_steps,
                    "path": "gbfem_operator_apply_host (page-locked host buffers; copy in, trace pass, apply and "
                            "copy out pipelined over 16 z-slabs on four streams, replayed as one CUDA graph)",
                    "in_place_c2c_value": e2e_in_place},
            "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                         "frac": achieved_gbs / peaks["hbm_gbs"], "traffic": traffic,
                         "peak_source": peak_kind, "algorithmic_bytes_per_dof": BYTES_PER_DOF,
                         "scope": "one apply: trace pass + main kernel (achieved and traffic alike)",
                         "main_kernel": {"name": "dg_const_kernel", "traffic": traffic_main,
                                         "launch_list_share": main_share,
                                         "frac_at_share": (achieved_gbs / main_share / peaks["hbm_gbs"])
                                         if main_share else None}},
            "fp64_pipe": {"achieved_tflops": achieved_tflops, "peak_tflops_measured": fp64_peak,
                          "frac": achieved_tflops / fp64_peak if fp64_peak else None,
                          "kernel_flop_per_dof": KERNEL_FLOP_PER_DOF,
                          "kernel_fp64_instructions_per_dof": KERNEL_FP64_INSTR_PER_DOF,
                          "issue_frac": (KERNEL_FP64_INSTR_PER_DOF * n / (ms_step * 1e-3) / 1e12) / (fp64_peak / 2)
                          if fp64_peak else None,
                          "sum_factorised_quadrature_flop_per_dof": FLOP_PER_DOF,
                          "fp32_peak_tflops_measured": fp32_peak},
            "algorithm": "constant-kappa closed form of the q=5 Gauss quadrature (exact for these integrands; "
                         "trace pre-pass + 1-D stiffness along lines + identity tangential face mass); "
                         "2 kernel launches per apply",
            "quadrature_kernel": {"value": n / (ms_quad * 1e-3), "unit": UNIT, "ms_per_step": ms_quad,
                                  "rel_max_diff_vs_default": quad_rel,
                                  "note": "sum-factorised evaluation at the 125 Gauss points (the variable-kappa path)"},
            "fp32_apply": {"value": n / (ms_f32 * 1e-3), "unit": UNIT, "ms_per_step": ms_f32,
                           "hbm_frac": 8.0 * n / (ms_f32 * 1e-3) / 1e9 / peaks["hbm_gbs"],
                           "kernel": "dg_cell_kernel (one kernel, no trace buffer; 8 B/dof algorithmic)",
                           "two_kernel_ms_per_step": ms_f32_two},
            "cpu_baseline": {"value": cpu_rate, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": "%d cells (whole z-slabs) of the 64^3 grid applied by the oracle "
                                       "(dense per-element evaluation as dune-fem's GalerkinOperator), ~15 s"
                                       % cpu_cells},
            "clocks": clk.summary()}
    if not args.no_solve:
        line["solve"] = solve_comparison()
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------
# Secondary workloads (the other problem configurations; one JSON line each).
# ----------------------------------------------------------------------------
def _timed(fn):
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    out = fn()
    torch.cuda.synchronize()
    return out, time.perf_counter() - t0


def q1_rhs(N):
    """Load vector of f = (2 pi^2 + 1) sin(pi x) sin(pi y) for Q1 (3x3 Gauss), zero Dirichlet rows."""
    h = 1.0 / N
    g, w = np.polynomial.legendre.leggauss(3)
    g, w = 0.5 * (g + 1), 0.5 * w
    b = np.zeros((N + 1, N + 1))
    ex = np.arange(N)
    for qy in range(3):
        for qx in range(3):
            X = (ex[None, :] + g[qx]) * h
            Y = (ex[:, None] + g[qy]) * h
            fv = (2 * np.pi ** 2 + 1) * np.sin(np.pi * X) * np.sin(np.pi * Y) * w[qx] * w[qy] * h * h
            for ky in range(2):
                for kx in range(2):
                    phi = (g[qx] if kx else 1 - g[qx]) * (g[qy] if ky else 1 - g[qy])
                    b[ky:ky + N, kx:kx + N] += fv * phi
    b[0, :] = b[-1, :] = b[:, 0] = b[:, -1] = 0.0
    return b.ravel()


def workload_q1cg(args):
    """2-D -lap u + u = f, 64x64 Q1, Dirichlet, diagonal-preconditioned CG to 1e-10 relative."""
    import gbfem
    import oracle
    N = 64
    op = gbfem.Q1Operator((N, N), diffusion=1.0, mass=1.0)
    pc = gbfem.Preconditioner.diagonal(op)
    b = q1_rhs(N)
    inv = gbfem.KrylovInverseOperator("cg", tolerance=1e-10)
    inv.bind(op, pc)
    bd = gbfem.DeviceArray.from_numpy(b)
    u = gbfem.DeviceArray(op.size)
    times = []
    for _ in range(args.warmup + args.steps):
        u.clear()
        _, t = _timed(lambda: inv(bd, u))
        times.append(t)
    t = float(np.median(times[args.warmup:]))
    # e2e: host rhs in, host solution out
    def e2e():
        bd2 = gbfem.DeviceArray.from_numpy(b)
        u2 = gbfem.DeviceArray(op.size)
        u2.clear()
        inv(bd2, u2)
        return u2.numpy()
    it_manufactured = inv.iterations()
    x, te = _timed(e2e)
    xs = np.linspace(0, 1, N + 1)
    X, Y = np.meshgrid(xs, xs)
    err = float(np.max(np.abs(x - (np.sin(np.pi * X) * np.sin(np.pi * Y)).ravel())))
    # the manufactured rhs is (to 1e-14) an eigenvector of the diagonally
    # preconditioned operator on this uniform grid, so CG stops after one
    # iteration (the oracle too); a seeded random interior rhs times the loop
    br = np.random.default_rng(SEED).uniform(-1, 1, b.size)
    br.reshape(N + 1, N + 1)[[0, -1], :] = 0.0
    br.reshape(N + 1, N + 1)[:, [0, -1]] = 0.0
    brd = gbfem.DeviceArray.from_numpy(br)
    rt = []
    for _ in range(args.warmup + args.steps):
        u.clear()
        _, tt = _timed(lambda: inv(brd, u))
        rt.append(tt)
    it_rand = inv.iterations()
    t_rand = float(np.median(rt[args.warmup:]))
    # the same solve with the device-resident loop (scalars on the device,
    # 32 iterations per CUDA-graph launch, one host read per launch)
    invg = gbfem.KrylovInverseOperator("cg", tolerance=1e-10, graph_chunk=32)
    invg.bind(op, pc)
    gt = []
    for _ in range(args.warmup + args.steps):
        u.clear()
        _, tt = _timed(lambda: invg(brd, u))
        gt.append(tt)
    t_graph = float(np.median(gt[args.warmup:]))
    it_graph = invg.iterations()
    # and a small 3-D DG solve (16^3 Q2 SIPG, block-Jacobi CG), where the
    # per-iteration host synchronisations are a large share of the iteration
    opd = gbfem.DGOperator((16, 16, 16), 2, mass=0.1)
    pcd = gbfem.Preconditioner.block_jacobi(opd)
    fd = gbfem.DeviceArray.from_numpy(np.random.default_rng(SEED).uniform(-1, 1, opd.size))
    ud = gbfem.DeviceArray(opd.size)
    dg_small = {}
    for name, chunk in (("host_loop", 0), ("graph32", 32)):
        invd = gbfem.KrylovInverseOperator("cg", tolerance=1e-10, graph_chunk=chunk)
        invd.bind(opd, pcd)
        dt = []
        for _ in range(args.warmup + args.steps):
            ud.clear()
            _, tt = _timed(lambda: invd(fd, ud))
            dt.append(tt)
        tm = float(np.median(dt[args.warmup:]))
        dg_small[name] = {"ms": 1e3 * tm, "iterations": invd.iterations(),
                          "us_per_iteration": 1e6 * tm / max(1, invd.iterations())}
    dg = oracle.q1_apply((N, N), None, 1.0, 1.0, diag_only=True)
    t0 = time.perf_counter()
    it_ref, x_ref, _ = oracle.cg(lambda v: oracle.q1_apply((N, N), v, 1.0, 1.0), b, prec=lambda r: r / dg,
                                 epsilon=1e-10, max_iter=100000)
    t_ref = time.perf_counter() - t0
    return {"metric": "Q1 64x64 diag-PCG solve time to 1e-10", "value": 1e3 * t, "unit": "ms",
            "higher_is_better": False, "iterations": it_manufactured, "oracle_iterations": it_ref,
            "max_nodal_error_vs_exact": err, "rel_diff_vs_oracle": float(np.max(np.abs(x - x_ref)) / np.max(np.abs(x_ref))),
            "random_rhs": {"ms": 1e3 * t_rand, "iterations": it_rand,
                           "us_per_iteration": 1e6 * t_rand / max(1, it_rand)},
            "random_rhs_graph32": {"ms": 1e3 * t_graph, "iterations": it_graph,
                                   "us_per_iteration": 1e6 * t_graph / max(1, it_graph)},
            "dg_16cube_q2_bj_cg": dg_small,
            "e2e": {"value": 1e3 * te, "unit": "ms", "h2d_bytes_per_step": 8 * b.size, "d2h_bytes_per_step": 8 * b.size},
            "cpu_baseline": {"value": 1e3 * t_ref, "unit": "ms", "cores": 1, "kind": "port",
                             "sample": "whole solve: oracle CG (cg.hh restated) + oracle Q1 apply"},
            "dtype": "f64", "config": {"workload": "Q1 CG 64x64, -lap u + u = f, Dirichlet, diagonal preconditioner"}}


def workload_rk3(args):
    """3-D periodic advection-diffusion, 128^3 Q2, SSP-RK3 CFL 0.2, FP64 and FP32."""
    import gbfem
    N, p = 128, 2
    steps = args.rk_steps
    kw = dict(diffusion=1e-3, velocity=(1.0, 0.5, 0.25), periodic=(1, 1, 1), weak_dirichlet=False)
    # Time step: TimeProvider with CFL factor 0.2 on the operator's estimate
    # h / (|b| (2p+1)), capped by the SIPG stability bound 2 / rho(M^{-1} A)
    # (SSP-RK3 is stable on [-2.51, 0]; rho from 30 device power iterations).
    opr = gbfem.DGOperator((N, N, N), p, **kw)
    est, ub = gbfem.time_step_estimate(opr, power_iterations=30)
    dt_adv, dt_stab = 0.2 * est, ub
    rho = 2.0 / ub
    del opr
    res = {}
    for prec, name in ((gbfem.F64, "f64"), (gbfem.F32, "f32")):
        op = gbfem.DGOperator((N, N, N), p, precision=prec, **kw)
        u = gbfem.project((N, N, N), p, gbfem.FN_GAUSSIAN, params=(0.5, 0.5, 0.5, 0.1), precision=prec)
        gbfem.RK3(op).step(u, min(dt_adv, dt_stab))  # warm-up step (then restart from the initial condition)
        u = gbfem.project((N, N, N), p, gbfem.FN_GAUSSIAN, params=(0.5, 0.5, 0.5, 0.1), precision=prec)
        tp = gbfem.TimeProvider(cfl=0.2)
        ode = gbfem.ExplicitRungeKuttaSolver(op, tp, estimate=(est, ub))  # the FP64 estimate for both
        ode.initialize(u)
        tp.init()
        dt = tp.deltaT()

        def loop():
            for _ in range(steps):
                ode.solve(u)
                tp.next()
        _, t = _timed(loop)
        res[name] = (t, u.numpy().astype(np.float64))
        del ode, op
    ndofs = N ** 3 * (p + 1) ** 3
    err = float(np.max(np.abs(res["f32"][1] - res["f64"][1])) / np.max(np.abs(res["f64"][1])))
    return {"metric": "SSP-RK3 128^3 Q2 advection-diffusion, time per step", "value": 1e3 * res["f64"][0] / steps,
            "unit": "ms/step", "higher_is_better": False, "steps": steps, "dt": dt, "dt_advective_cfl_0.2": dt_adv,
            "time_loop": "TimeProvider(cfl=0.2) + ExplicitRungeKuttaSolver (SSP-RK3)",
            "dt_stability": dt_stab, "spectral_radius_minv_a": rho,
            "f64_max_abs": float(np.max(np.abs(res["f64"][1]))),
            "f32_ms_per_step": 1e3 * res["f32"][0] / steps,
            "f64_dof_stage_per_s": 3 * ndofs * steps / res["f64"][0],
            "f32_dof_stage_per_s": 3 * ndofs * steps / res["f32"][0],
            "f32_vs_f64_rel_max_error": err, "dtype": "f64 (and f32)",
            "config": {"workload": "DG Q2 128^3 periodic, b=(1,0.5,0.25), eps=1e-3, Gaussian bump w=0.1, CFL 0.2"}}


def residual_floor(op64, f, x):
    """How far FP64 storage of the solution lets ||f - A u|| / ||f|| fall.
    du changes every dof of x by one unit in the last place (seeded random
    sign), the smallest change an FP64 vector can make; ||A du|| / ||f|| is
    then the residual change that FP64 rounding of u alone causes.  When it is
    as large as the residual reached, no FP64 vector is measurably closer to
    the solution, and the stagnation is this floor, not a solver defect.
    Also reports the residual of x + du (both evaluated by the FP64 apply)."""
    import gbfem
    fh = f.numpy()
    fn = float(np.linalg.norm(fh))
    sign = np.where(np.random.default_rng(17).random(x.size) < 0.5, -1.0, 1.0)
    du = np.spacing(x) * sign
    a_du = gbfem.DeviceArray(op64.size)
    op64(gbfem.DeviceArray.from_numpy(du), a_du)
    res = {}
    for name, v in (("u", x), ("u_plus_ulp", x + du)):
        au = gbfem.DeviceArray(op64.size)
        op64(gbfem.DeviceArray.from_numpy(v), au)
        res[name] = float(np.linalg.norm(fh - au.numpy()) / fn)
    return {"rel_residual_of_u": res["u"], "rel_residual_of_u_plus_ulp": res["u_plus_ulp"],
            "one_ulp_change_rel_residual": float(np.linalg.norm(a_du.numpy()) / fn),
            "note": "||A du|| / ||f|| for du = one ulp of every dof of u (random sign): the residual change "
                    "the FP64 representation of u alone causes"}


def workload_mixed(args):
    """3-D SIPG -div(kappa grad u) = 1, 96^3 Q4 (or --cells, --mixed-order), log-Gaussian kappa; the
    mixed-precision solves against FP64 block-Jacobi CG."""
    import gbfem
    N, p = args.cells, args.mixed_order
    cells = (N, N, N)
    modes = gbfem.fourier_modes(args.seed, 256, 0.1, 1.0)
    k64 = gbfem.project(cells, p, gbfem.FN_EXP_FOURIER, modes=modes)
    k32 = gbfem.project(cells, p, gbfem.FN_EXP_FOURIER, modes=modes, precision=gbfem.F32)
    f = gbfem.project(cells, p, gbfem.FN_CONSTANT, params=(1.0,), scale_by_volume=True)
    op64 = gbfem.DGOperator(cells, p, kappa=k64)
    op32 = gbfem.DGOperator(cells, p, precision=gbfem.F32, kappa=k32)
    out = {"metric": "SIPG Q%d variable-kappa solve time to 1e-10 (mixed FP32-in-FP64 vs FP64 CG)" % p,
           "unit": "s", "higher_is_better": False, "dtype": "f64 outer / f32 inner",
           "config": {"workload": "SIPG Q%d %d^3, -div(kappa grad u) = 1, u = 0 weak, log kappa ~ 256 Fourier modes "
                                  "(std 1, corr 0.1), seed %d" % (p, N, args.seed), "dofs": op64.size}}
    variants = set(args.mixed_variants.split(","))
    pc32, t_setup32 = None, 0.0
    if variants & {"refinement", "fgmres"}:
        (pc32, t_setup32) = _timed(lambda: gbfem.Preconditioner.block_jacobi(op64, gbfem.F32))
    u = gbfem.DeviceArray(op64.size)
    u.clear()
    t_mixed = float("inf")
    info = None
    x_mixed = None
    best = {}  # variant -> time of the solves that converged or reached the FP64 rounding floor

    def consider(name, inf, t):
        nonlocal x_mixed
        if inf.converged or inf.stagnated:
            best[name] = t
            if min(best.values()) == t:
                x_mixed = u.numpy()
    if not args.skip_refinement and "refinement" in variants:
        info, t_mixed = _timed(lambda: gbfem.solve_mixed(op64, op32, pc32, f, u, tolerance=1e-10,
                                                         inner_tolerance=args.inner_tol, max_outer=60))
        out.update({"value": t_mixed, "mixed_refinement_s": t_mixed, "mixed_setup_s": t_setup32,
                    "mixed_converged": bool(info.converged),
                    "mixed_rel_residual": info.residual, "mixed_inner_iterations": info.iterations,
                    "mixed_operator_applies": info.operator_applies,
                    "mixed_outer_iterations": info.outer_iterations, "mixed_stagnated": bool(info.stagnated)})
        consider("refinement", info, t_mixed)
    # flexible FP64 outer Krylov (FGMRES) with the FP32 inner solve as its
    # preconditioner: converges where plain refinement stalls on cond(A) eps32
    if "fgmres" in variants:
        u.clear()
        infog, t_fg = _timed(lambda: gbfem.solve_mixed(op64, op32, pc32, f, u, tolerance=1e-10,
                                                       inner_tolerance=args.fgmres_inner_tol, max_outer=300,
                                                       outer="fgmres", outer_restart=30))
        out.update({"mixed_fgmres_s": t_fg, "mixed_fgmres_converged": bool(infog.converged),
                    "mixed_fgmres_rel_residual": infog.residual, "mixed_fgmres_inner_iterations": infog.iterations,
                    "mixed_fgmres_outer_iterations": infog.outer_iterations,
                    "mixed_fgmres_stagnated": bool(infog.stagnated)})
        consider("fgmres", infog, t_fg)
    del pc32
    # the flexible outer solve with scaled FP16 block-Jacobi storage (half the
    # preconditioner traffic of the FP32 inner iteration)
    if "f16" in variants:
        (pc16, t_setup16) = _timed(lambda: gbfem.Preconditioner.block_jacobi(op64, gbfem.F16))
        u.clear()
        info16, t_mixed16 = _timed(lambda: gbfem.solve_mixed(op64, op32, pc16, f, u, tolerance=1e-10,
                                                             inner_tolerance=args.fgmres_inner_tol, max_outer=300,
                                                             outer="fgmres", outer_restart=30))
        out.update({"mixed_f16_blocks_fgmres_s": t_mixed16, "mixed_f16_setup_s": t_setup16,
                    "mixed_f16_outer_iterations": info16.outer_iterations,
                    "mixed_f16_converged": bool(info16.converged), "mixed_f16_rel_residual": info16.residual,
                    "mixed_f16_inner_iterations": info16.iterations, "mixed_f16_stagnated": bool(info16.stagnated)})
        consider("fgmres_f16_blocks", info16, t_mixed16)
        del pc16
    # the FP32 inner operator with kappa replaced by its cell means: the
    # closed-form kernel applies it exactly (cheaper than the Gauss-point
    # kernel); the FP64 FGMRES still iterates on the full kappa
    # ("cellkappa" runs both preconditioners below, "scaledbj" only the second)
    if variants & {"cellkappa", "scaledbj"}:
        kbar = gbfem.cell_means(k32, p)
        op32c = gbfem.DGOperator(cells, p, precision=gbfem.F32, kappa_cell=kbar)
    if "cellkappa" in variants:
        (pc16c, t_setup16c) = _timed(lambda: gbfem.Preconditioner.block_jacobi(op32c, gbfem.F16))
        u.clear()
        infoc, t_c = _timed(lambda: gbfem.solve_mixed(op64, op32c, pc16c, f, u, tolerance=1e-10,
                                                      inner_tolerance=args.fgmres_inner_tol, max_outer=300,
                                                      outer="fgmres", outer_restart=30,
                                                      graph_chunk=args.inner_graph_chunk))
        out.update({"mixed_cellkappa_f16_fgmres_s": t_c, "mixed_cellkappa_setup_s": t_setup16c,
                    "mixed_cellkappa_converged": bool(infoc.converged),
                    "mixed_cellkappa_rel_residual": infoc.residual,
                    "mixed_cellkappa_inner_iterations": infoc.iterations,
                    "mixed_cellkappa_outer_iterations": infoc.outer_iterations,
                    "mixed_cellkappa_stagnated": bool(infoc.stagnated)})
        consider("fgmres_cellkappa_f16_blocks", infoc, t_c)
        del pc16c
    if variants & {"cellkappa", "scaledbj"}:
        # the same with the scaled shared-block Jacobi (27 kappa = 1 blocks)
        pcs = gbfem.Preconditioner.scaled_block_jacobi(op32c)
        u.clear()
        infos, t_s = _timed(lambda: gbfem.solve_mixed(op64, op32c, pcs, f, u, tolerance=1e-10,
                                                      inner_tolerance=args.fgmres_inner_tol, max_outer=300,
                                                      outer="fgmres", outer_restart=30,
                                                      graph_chunk=args.inner_graph_chunk))
        out.update({"mixed_cellkappa_scaledbj_fgmres_s": t_s, "mixed_cellkappa_scaledbj_converged": bool(infos.converged),
                    "mixed_cellkappa_scaledbj_rel_residual": infos.residual,
                    "mixed_cellkappa_scaledbj_inner_iterations": infos.iterations,
                    "mixed_cellkappa_scaledbj_outer_iterations": infos.outer_iterations,
                    "mixed_cellkappa_scaledbj_stagnated": bool(infos.stagnated)})
        consider("fgmres_cellkappa_scaled_bj", infos, t_s)
        del pcs, op32c
    if best:
        name = min(best, key=best.get)
        out["value"], out["value_from"] = best[name], name
    if x_mixed is not None:
        out["fp64_floor"] = residual_floor(op64, f, x_mixed)
    if not args.skip_fp64:
        (pc64, t_setup64) = _timed(lambda: gbfem.Preconditioner.block_jacobi(op64))
        inv = gbfem.KrylovInverseOperator("cg", tolerance=1e-10, max_iterations=args.fp64_max_iter)
        inv.bind(op64, pc64)
        u.clear()
        _, t64 = _timed(lambda: inv(f, u))
        i64 = inv.info()
        x64 = u.numpy()
        # the FP64 CG stops on <r, B r> (preconditioned); its true relative
        # residual is the accuracy the mixed solves are compared at
        au = gbfem.DeviceArray(op64.size)
        op64(u, au)
        fh = f.numpy()
        out["fp64_true_rel_residual"] = float(np.linalg.norm(fh - au.numpy()) / np.linalg.norm(fh))
        del au
        out.update({"fp64_cg_s": t64, "fp64_setup_s": t_setup64, "fp64_converged": i64["converged"],
                    "fp64_iterations": i64["iterations"], "speedup_mixed_vs_fp64": t64 / out["value"] if out.get("value") else None,
                    "mixed_vs_fp64_rel_max_diff": (None if x_mixed is None else
                                                   float(np.max(np.abs(x_mixed - x64)) / np.max(np.abs(x64))))})
    return out


def workload_learned(args):
    """SIPG Q3 variable kappa (cells^3), CNN preconditioner trained on the
    solver's own (residual, error) pairs for args.train_seeds kappa seeds,
    evaluated on args.eval_seeds held-out seeds against FP64 CG."""
    import gbfem
    import learned
    N, p = args.cells, args.order
    net = gbfem.CNN(p, N, seed=2026)
    log = (lambda m: print(m, file=sys.stderr, flush=True)) if args.verbose else None
    t0 = time.perf_counter()
    if args.loss == "projected":
        args.form = "twolevel"
        net.scale = 1.0
        losses = learned.train_projected(net, N, p, list(range(args.train_seeds)), steps_per_pair=args.train_steps,
                                         lr=args.lr, log=log)
    elif args.loss == "anorm":
        losses = learned.train_anorm(net, N, p, list(range(args.train_seeds)), steps_per_pair=args.train_steps,
                                     lr=args.lr, log=log, form=args.form)
    else:
        losses = learned.train(net, N, p, list(range(args.train_seeds)), steps_per_pair=args.train_steps,
                               lr=args.lr, log=log, form=args.form)
    t_train = time.perf_counter() - t0
    if args.save_net:
        net.save(args.save_net)
    diag = learned.diagnose(net, N, p, 100000, form=args.form)
    evals = [learned.evaluate(net, N, p, 100000 + s, plain=not args.skip_plain, form=args.form,
                              plain_max_iterations=args.plain_max_iter)
             for s in range(args.eval_seeds)]
    def mean(key, field):
        v = [e[key][field] for e in evals if key in e]
        return float(np.mean(v)) if v else None
    out = {"metric": "SIPG Q%d variable-kappa solve time to 1e-10: learned/mixed vs plain FP64 CG" % p, "unit": "s",
           "higher_is_better": False, "dtype": "f64 outer / f32 inner / bf16 network",
           "config": {"workload": "SIPG Q%d %d^3 (%d dofs), -div(kappa grad u) = 1, log kappa ~ 256 Fourier modes; "
                                  "%d training seeds, %d held-out seeds" % (p, N, N ** 3 * (p + 1) ** 3,
                                                                          args.train_seeds, args.eval_seeds)},
           "value": mean("mixed_learned", "time_s"),
           "train_s": t_train, "train_steps": len(losses), "loss_first": losses[0], "loss_last": losses[-1],
           "loss_last_mean20": float(np.mean(losses[-20:])), "form": args.form, "loss": args.loss,
           "a_norm_error_ratio": diag,
           "evals": evals}
    for k in ("plain_cg", "bj_cg", "learned_fcg", "mixed_bj", "mixed_learned"):
        out[k + "_mean_time_s"] = mean(k, "time_s")
        out[k + "_mean_iterations"] = mean(k, "iterations")
    if out.get("plain_cg_mean_time_s") and out.get("mixed_learned_mean_time_s"):
        out["speedup_mixed_learned_vs_plain_fp64_cg"] = out["plain_cg_mean_time_s"] / out["mixed_learned_mean_time_s"]
    if out.get("bj_cg_mean_time_s") and out.get("learned_fcg_mean_time_s"):
        out["speedup_learned_fcg_vs_bj_cg"] = out["bj_cg_mean_time_s"] / out["learned_fcg_mean_time_s"]
    return out


def workload_kernels(args):
    """CUDA-event timings of the building blocks of one Krylov iteration on the
    variable-kappa SIPG problem (order args.order, args.cells^3)."""
    import torch
    import gbfem
    import learned
    N, p = args.cells, args.order
    op64, op32, k64, k32, f = learned.sipg_problem(N, p, args.seed)
    n = op64.size
    stream = torch.cuda.current_stream()
    sptr = stream.cuda_stream

    def ev(fn, reps=10):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    u64 = gbfem.DeviceArray.from_numpy(np.random.default_rng(0).uniform(-1, 1, n))
    w64 = gbfem.DeviceArray(n)
    u32 = gbfem.convert(u64, gbfem.F32)
    w32 = gbfem.DeviceArray(n, gbfem.F32)
    out = {"metric": "Krylov building blocks, ms", "unit": "ms", "cells": N, "order": p, "dofs": n}
    out["apply_f64_quadrature_kappa"] = ev(lambda: op64(u64, w64, sptr))
    out["apply_f32_quadrature_kappa"] = ev(lambda: op32(u32, w32, sptr))
    opc = gbfem.DGOperator((N, N, N), p)
    out["apply_f64_const"] = ev(lambda: opc(u64, w64, sptr))
    opc32 = gbfem.DGOperator((N, N, N), p, precision=gbfem.F32)
    out["apply_f32_const"] = ev(lambda: opc32(u32, w32, sptr))
    t0 = time.perf_counter()
    bj64 = gbfem.Preconditioner.block_jacobi(op64)
    torch.cuda.synchronize()
    out["bj64_setup_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    bj32 = gbfem.Preconditioner.block_jacobi(op32, gbfem.F32)
    torch.cuda.synchronize()
    out["bj32_setup_s"] = time.perf_counter() - t0
    out["bj64_apply"] = ev(lambda: bj64(u64, w64, sptr))
    out["bj32_apply"] = ev(lambda: bj32(u32, w32, sptr))
    bj16 = gbfem.Preconditioner.block_jacobi(op32, gbfem.F16)
    out["bj16_apply"] = ev(lambda: bj16(u32, w32, sptr))
    del bj16
    # the cellwise-kappa FP32 operator and its scaled shared-block Jacobi
    opc = gbfem.DGOperator((N, N, N), p, precision=gbfem.F32, kappa_cell=gbfem.cell_means(k32, p))
    out["apply_f32_cellkappa"] = ev(lambda: opc(u32, w32, sptr))
    sbj = gbfem.Preconditioner.scaled_block_jacobi(opc)
    out["scaled_bj_apply"] = ev(lambda: sbj(u32, w32, sptr))
    del sbj, opc
    out["dot_f64_host_result"] = ev(lambda: gbfem.dot(u64, w64, sptr))
    out["axpy_f64"] = ev(lambda: gbfem.axpy(0.5, u64, w64, sptr))
    for name, op, pc, fv in (("cg_iter_f64_bj", op64, bj64, f), ("cg_iter_f32_bj", op32, bj32, gbfem.convert(f, gbfem.F32))):
        x = gbfem.DeviceArray(n, op.precision)
        inv = gbfem.KrylovInverseOperator("cg", tolerance=1e-30, max_iterations=50)
        inv.bind(op, pc)
        x.clear()
        inv(fv, x)
        out[name] = inv.info()["time_ms"] / 50.0
    if N % 8 == 0 and p <= 4:
        net = gbfem.CNN(p, N, seed=1)
        net.set_kappa(k64)
        out["cnn_forward_f64"] = ev(lambda: net.forward(u64, w64))
        out["cnn_train_step_f32"] = ev(lambda: net.train_step(u32, w32, 1e-4), reps=5)
    return out


def workload_apply_kappa(args):
    """The variable-kappa Gauss-point apply (cells^3, Q_order, q = order+2) in
    FP32 and FP64: the operator of the mixed solve's inner and outer loops."""
    import gbfem
    import torch
    N, p = args.cells, args.order
    cells = (N, N, N)
    modes = gbfem.fourier_modes(args.seed, 256, 0.1, 1.0)
    out = {"metric": "variable-kappa SIPG apply DoF/s (Gauss-point kernel)", "unit": "DoF/s", "higher_is_better": True,
           "config": {"workload": "SIPG Q%d %d^3, log-Gaussian kappa (256 Fourier modes)" % (p, N)}}
    stream = torch.cuda.current_stream()
    for prec, name in ((gbfem.F32, "f32"), (gbfem.F64, "f64")):
        k = gbfem.project(cells, p, gbfem.FN_EXP_FOURIER, modes=modes, precision=prec)
        op = gbfem.DGOperator(cells, p, precision=prec, kappa=k)
        u0 = np.random.default_rng(SEED).uniform(-1, 1, op.size)
        u = gbfem.DeviceArray.from_numpy(u0.astype(np.float32) if prec == gbfem.F32 else u0)
        w = gbfem.DeviceArray(op.size, prec)
        ms = time_applies(op, u, w, max(3, min(args.steps, 20)), stream)
        out[name] = {"ms": ms, "dof_per_s": op.size / (ms * 1e-3)}
        del op, k, u, w
    out["value"] = out["f32"]["dof_per_s"]
    out["dtype"] = "f32 (and f64)"
    return out


def workload_apply_f32(args):
    """The constant-coefficient FP32 apply (cells^3, Q_order) alone, --steps
    times after 3 warm-up applies, with no other GPU work: the command the
    kernel profiles under profiles/ are taken from.  --algorithm 0 is the
    default (one kernel for p <= 3), 2 the two-kernel trace-pass form;
    --kappa-cell uses a seeded kappa per cell."""
    import gbfem
    import torch
    N, p = args.cells, args.order
    cells = (N, N, N)
    kc = None
    if args.kappa_cell:
        kc = gbfem.DeviceArray.from_numpy(
            np.exp(np.random.default_rng(args.seed).uniform(-2, 2, N ** 3)).astype(np.float32))
    op = gbfem.DGOperator(cells, p, precision=gbfem.F32, algorithm=args.algorithm, kappa_cell=kc)
    u = gbfem.DeviceArray.from_numpy(np.random.default_rng(SEED).uniform(-1, 1, op.size).astype(np.float32))
    w = gbfem.DeviceArray(op.size, gbfem.F32)
    stream = torch.cuda.current_stream()
    ms = time_applies(op, u, w, max(1, args.steps), stream)
    return {"metric": "FP32 SIPG apply DoF/s", "unit": "DoF/s", "higher_is_better": True,
            "value": op.size / (ms * 1e-3), "ms_per_step": ms, "dtype": "f32",
            "hbm_frac_8B_per_dof": 8.0 * op.size / (ms * 1e-3) / 1e9 / load_peaks()[0]["hbm_gbs"],
            "config": {"workload": "SIPG Q%d %d^3 FP32 apply, algorithm %d%s" %
                                   (p, N, args.algorithm, ", kappa per cell" if kc is not None else "")}}


def workload_scaled_bj(args):
    """The scaled shared-block Jacobi apply of the cellwise-kappa FP32
    operator (cells^3, Q_order, seeded kappa per cell) on both engines of its
    tile products: tcgen05 tensor cores (3xTF32) and FP32 FMA; --steps applies
    after 3 warm-up applies, CUDA events."""
    import gbfem
    import torch
    N, p = args.cells, args.order
    nc = N ** 3
    kc = gbfem.DeviceArray.from_numpy(np.exp(np.random.default_rng(args.seed).uniform(-2, 2, nc)).astype(np.float32))
    op = gbfem.DGOperator((N, N, N), p, precision=gbfem.F32, kappa_cell=kc)
    r = gbfem.DeviceArray.from_numpy(np.random.default_rng(SEED).uniform(-1, 1, op.size).astype(np.float32))
    z = gbfem.DeviceArray(op.size, gbfem.F32)
    stream = torch.cuda.current_stream()
    out = {"metric": "scaled block-Jacobi apply", "unit": "ms", "higher_is_better": False, "dtype": "f32",
           "config": {"workload": "scaled shared-block Jacobi, SIPG Q%d %d^3 (%d dofs), kappa per cell" % (p, N, op.size)}}
    res = {}
    for engine in ("tensor", "fma"):
        pc = gbfem.Preconditioner.scaled_block_jacobi(op, engine=engine)
        ms = time_applies(pc, r, z, max(1, args.steps), stream)
        res[engine] = z.numpy()
        out[engine] = {"ms": ms, "hbm_frac_8B_per_dof": 8.0 * op.size / (ms * 1e-3) / 1e9 / load_peaks()[0]["hbm_gbs"],
                       "status": pc.status() if engine == "tensor" else 0}
        del pc
    out["value"] = out["tensor"]["ms"]
    out["tensor_vs_fma_rel_max_diff"] = float(np.max(np.abs(res["tensor"] - res["fma"])) / np.max(np.abs(res["fma"])))
    return out


def workload_cnn(args):
    """The learned preconditioner's network on cells^3 DG Q_order: forward
    (z = S rms NN(r/rms)) and forward + loss + backward, each --steps times
    after 3 warm-ups, CUDA events, on both engines of the 3x3x3 convolutions
    (tcgen05 with TMA loads, and mma.sync); the command the convolution
    profiles under profiles/ are taken from."""
    import gbfem
    import torch
    N, p = args.cells, args.order
    nloc = (p + 1) ** 3
    n = N ** 3 * nloc
    rng = np.random.default_rng(args.seed)
    kappa = np.zeros(n)
    kappa[::nloc] = np.exp(rng.normal(0, 1, N ** 3))
    r = gbfem.DeviceArray.from_numpy(rng.uniform(-1, 1, n))
    t = gbfem.DeviceArray.from_numpy(rng.uniform(-1, 1, n))
    z = gbfem.DeviceArray(n)
    stream = torch.cuda.current_stream()
    out = {"metric": "learned-preconditioner network time", "unit": "ms", "higher_is_better": False, "dtype": "bf16",
           "config": {"workload": "4-level 3-D U-net, 32 channels, DG Q%d %d^3 (%d dofs)" % (p, N, n)}}
    steps = max(1, args.steps)
    for engine in ("tensor", "mma"):
        net = gbfem.CNN(p, N, seed=1)
        net.set_conv_engine(engine)
        net.set_kappa(gbfem.DeviceArray.from_numpy(kappa))
        res = {}
        for name, fn in (("forward", lambda: net.forward(r, z)),
                         ("forward_backward", lambda: gbfem.check(gbfem.lib().gbfem_cnn_loss_grad(
                             net.handle, gbfem.F64, r.ptr, t.ptr, None, None)))):
            for _ in range(3):
                fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            res[name + "_ms"] = e0.elapsed_time(e1) / steps
        res["status"] = net.status()
        out[engine] = res
        del net
    out["value"] = out["tensor"]["forward_ms"]
    return out


def workload_forms(args):
    """The general-form path against the built-in operator on the same
    problem: Bratu -lap u = 5 e^u (SIPG Q2, weak u = 0) on cells^3 as
    NonlinearDGOperator (hand-written reaction kernel) and as a run-time
    compiled Form (flux g, source -5 e^u, dual-number Jacobian): apply and
    Jacobian-apply times (CUDA events, --steps after 3 warm-ups), their
    relative difference, and the Newton solve (Eisenstat-Walker, GMRES,
    block Jacobi of each Jacobian) matrix-free and with each Jacobian
    assembled into the block-sparse matrix."""
    import gbfem
    import integrands
    import torch
    N, p = args.cells, 2
    cells = (N, N, N)
    builtin = gbfem.NonlinearDGOperator(cells, p, reaction=(0.0, 0.0, -5.0))
    form = integrands.Form(flux="for (int k = 0; k < 3; ++k) F[0][k] = g[0][k];", source="s[0] = -5.0 * exp(u[0]);",
                           dirichlet="")
    generated = integrands.FormOperator(form, cells, p)
    n = builtin.size
    rng = np.random.default_rng(SEED)
    u = gbfem.DeviceArray.from_numpy(0.3 * rng.uniform(-1, 1, n))
    du = gbfem.DeviceArray.from_numpy(rng.uniform(-1, 1, n))
    w = gbfem.DeviceArray(n)
    stream = torch.cuda.current_stream()
    steps = max(1, args.steps)
    out = {"metric": "Bratu on a generated form vs the built-in operator", "unit": "ms", "higher_is_better": False,
           "dtype": "f64", "config": {"workload": "Bratu -lap u = 5 e^u, SIPG Q2 %d^3 (%d dofs), u = 0 weak" % (N, n)}}
    res = {}
    for name, op in (("builtin", builtin), ("form", generated)):
        jac = op.jacobian(u)
        r = {"apply_ms": time_applies(op, u, w, steps, stream)}
        res[name] = w.numpy()
        r["jacobian_apply_ms"] = time_applies(jac, du, w, steps, stream)
        res[name + "_j"] = w.numpy()
        for assembled in (False, True):
            newton = gbfem.NewtonInverseOperator(tolerance=1e-9, forcing="eisenstatwalker", linear_tolerance=1e-10,
                                                 linear_method="gmres", linear_restart=50, max_iterations=100,
                                                 preconditioner=gbfem.PC_BLOCK_JACOBI, assembled=assembled)
            newton.bind(op)
            rhs = gbfem.DeviceArray(n)
            rhs.clear()
            x = gbfem.DeviceArray(n)
            x.clear()
            newton(rhs, x)  # warm-up
            x.clear()
            _, t = _timed(lambda: newton(rhs, x))
            info = newton.info()
            key = "newton_assembled" if assembled else "newton_matrix_free"
            r[key] = {"s": t, "newton_iterations": info["iterations"], "linear_iterations": info["linear_iterations"],
                      "converged": info["converged"]}
            res[name + "_x" + ("a" if assembled else "")] = x.numpy()
            del newton
        out[name] = r
        del jac
    def rel(a, b):
        return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    out["apply_rel_diff"] = rel(res["form"], res["builtin"])
    out["jacobian_rel_diff"] = rel(res["form_j"], res["builtin_j"])
    out["solution_rel_diff"] = rel(res["form_x"], res["builtin_x"])
    out["assembled_vs_matrix_free_rel_diff"] = rel(res["form_xa"], res["form_x"])
    out["value"] = out["form"]["apply_ms"]
    return out


def workload_mixed_solve(args):
    """The mixed arm of the headline line's solve object alone (64^3 Q3,
    kappa seed 1, f = 1, to ||f - A u|| / ||f|| <= 1e-10): FP64 FGMRES(30) on
    the full kappa around the FP32 inner CG (device-resident, graph chunks of
    16) on the cellwise-kappa one-kernel apply with the tcgen05 scaled block
    Jacobi.  --max-outer bounds the outer iterations (a short window for
    kernel launch lists)."""
    import gbfem
    import torch
    N, p = SOLVE_CELLS, SOLVE_ORDER
    cells = (N, N, N)
    modes = gbfem.fourier_modes(SOLVE_SEED, 256, 0.1, 1.0)
    k64 = gbfem.project(cells, p, gbfem.FN_EXP_FOURIER, modes=modes)
    k32 = gbfem.project(cells, p, gbfem.FN_EXP_FOURIER, modes=modes, precision=gbfem.F32)
    f = gbfem.project(cells, p, gbfem.FN_CONSTANT, params=(1.0,), scale_by_volume=True)
    op64 = gbfem.DGOperator(cells, p, kappa=k64)
    op32c = gbfem.DGOperator(cells, p, precision=gbfem.F32, kappa_cell=gbfem.cell_means(k32, p))
    u = gbfem.DeviceArray(op64.size)
    u.clear()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    pcs = gbfem.Preconditioner.scaled_block_jacobi(op32c)
    info = gbfem.solve_mixed(op64, op32c, pcs, f, u, tolerance=1e-10, inner_tolerance=1e-2,
                             max_outer=args.max_outer, outer="fgmres", outer_restart=30, graph_chunk=16)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    inner = abs(info.iterations)
    return {"metric": "mixed solve time to relative residual 1e-10", "unit": "s", "higher_is_better": False,
            "value": t, "dtype": "f64/f32", "outer_iterations": info.outer_iterations, "inner_iterations": inner,
            "converged": bool(info.converged), "ms_per_inner_iteration": t / max(1, inner) * 1e3,
            "config": {"workload": "SIPG Q3 %d^3 (%d dofs), variable kappa (seed %d), mixed FGMRES arm; max outer %d"
                                   % (N, op64.size, SOLVE_SEED, args.max_outer)}}


def workload_newton(args):
    """Bratu problem -lap u = lambda e^u (lambda = 5, SIPG Q2, weak u = 0) on
    cells^3 by Newton with block-Jacobi CG for each Jacobian; with and without
    Eisenstat-Walker forcing.  CPU baseline: the oracle's restated Newton loop
    with the oracle's Jacobian and a dense solve on a 3^3 grid."""
    import gbfem
    N, p = args.cells, 2
    cells = (N, N, N)
    reaction = (0.0, 0.0, -5.0)
    op = gbfem.NonlinearDGOperator(cells, p, reaction=reaction)
    rhs = gbfem.DeviceArray(op.size)
    rhs.clear()
    w = gbfem.DeviceArray(op.size)
    out = {"metric": "Bratu Newton solve time to |S(u)| < 1e-9 (SIPG Q2, lambda = 5)", "unit": "s",
           "higher_is_better": False, "dtype": "f64",
           "config": {"workload": "Bratu -lap u = 5 e^u, SIPG Q2 %d^3, u = 0 weak; Newton + block-Jacobi CG" % N,
                      "dofs": op.size}}
    runs = (("none", "cg"), ("eisenstatwalker", "gmres"))
    for forcing, method in runs:
        # the forcing term bounds the true residual |J dw - r| <= eta |r|: GMRES
        # (right preconditioning) measures that one, preconditioned CG does not
        newton = gbfem.NewtonInverseOperator(tolerance=1e-9, forcing=forcing, linear_tolerance=1e-10,
                                             linear_method=method, linear_restart=50, max_iterations=100,
                                             preconditioner=gbfem.PC_BLOCK_JACOBI)
        newton.bind(op)
        w.clear()
        newton(rhs, w)  # warm-up (allocations, first Jacobian)
        w.clear()
        _, t = _timed(lambda: newton(rhs, w))
        info = newton.info()
        out["forcing_" + forcing] = {"s": t, "linear_method": method, "newton_iterations": info["iterations"],
                                     "linear_iterations": info["linear_iterations"], "residual": info["residual"],
                                     "converged": info["converged"]}
    done = [v["s"] for v in (out["forcing_none"], out["forcing_eisenstatwalker"]) if v["converged"]]
    out["value"] = min(done) if done else None
    out["max_u"] = float(np.max(w.numpy()))
    # oracle on 3^3 (dense Jacobian solves)
    import oracle
    import nonlinear_oracle as no
    prob = oracle.DGProblem((3, 3, 3), p)
    P = no.NonlinearProblem(prob, reaction)
    t0 = time.perf_counter()
    _, io = no.newton(P.apply, lambda ww, r, tol: (np.linalg.solve(P.jacobian_matrix(ww), r), 1),
                      np.zeros(prob.ndofs), np.zeros(prob.ndofs), tolerance=1e-9)
    out["cpu_baseline"] = {"value": time.perf_counter() - t0, "unit": "s", "cores": 1, "kind": "port",
                           "sample": "3^3 cells Q2: oracle Newton, dense Jacobian from the oracle apply, numpy solve",
                           "newton_iterations": io["iterations"]}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gbfem", choices=["gbfem", "reference"])
    ap.add_argument("--workload", default="apply",
                    choices=["apply", "q1cg", "rk3", "mixed", "learned", "kernels", "newton", "apply_kappa",
                             "apply_f32", "scaled_bj", "cnn", "forms", "mixed_solve"])
    ap.add_argument("--rk-steps", type=int, default=100)
    ap.add_argument("--cells", type=int, default=96)
    ap.add_argument("--order", type=int, default=3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--inner-tol", type=float, default=1e-3)
    ap.add_argument("--fgmres-inner-tol", type=float, default=1e-2)
    ap.add_argument("--fp64-max-iter", type=int, default=20000)
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-refinement", action="store_true")
    ap.add_argument("--mixed-variants", default="refinement,fgmres,f16,cellkappa")
    ap.add_argument("--mixed-order", type=int, default=4)
    ap.add_argument("--inner-graph-chunk", type=int, default=0)
    ap.add_argument("--train-seeds", type=int, default=256)
    ap.add_argument("--eval-seeds", type=int, default=32)
    ap.add_argument("--train-steps", type=int, default=2)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--skip-plain", action="store_true")
    ap.add_argument("--save-net", default="")
    ap.add_argument("--form", default="additive", choices=["additive", "twolevel"])
    ap.add_argument("--loss", default="projected", choices=["projected", "anorm", "mse"])
    ap.add_argument("--plain-max-iter", type=int, default=0)
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--no-solve", action="store_true", help="skip the solve comparison of the headline line")
    ap.add_argument("--algorithm", type=int, default=0)
    ap.add_argument("--kappa-cell", action="store_true")
    ap.add_argument("--max-outer", type=int, default=300)
    args = ap.parse_args()
    if args.workload != "apply":
        fn = {"q1cg": workload_q1cg, "rk3": workload_rk3, "mixed": workload_mixed,
              "learned": workload_learned, "kernels": workload_kernels, "newton": workload_newton,
              "apply_kappa": workload_apply_kappa, "apply_f32": workload_apply_f32,
              "scaled_bj": workload_scaled_bj, "cnn": workload_cnn, "forms": workload_forms,
              "mixed_solve": workload_mixed_solve}[args.workload]
        line = fn(args)
        line.update({"n_gpus": 1, "data": "synthetic"})
        print(json.dumps(line), flush=True)
        return
    world, rank, local = dist_init() if args.impl == "gbfem" else (
        int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")), 0)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank, local)


if __name__ == "__main__":
    main()
