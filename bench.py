#!/usr/bin/env python3
"""Benchmark of the GB300 Krylov solve path (one JSON line on stdout).

Default workload (one GPU): the 128^3 jittered-hex pressure-Poisson system
(2,097,152 cells, 14,581,760 stored entries, random cell numbering, RHS
U[-1,1]) solved by DIC-preconditioned CG to ||r|| < 1e-8 ||b|| from x0 = 0,
in binary64 and in mixed precision (binary32 inner iterations, binary64
true residual / reductions / solution).  A step is one complete solve:
reset x = 0 and r1 = b, form the preconditioner, iterate to the tolerance.

  value     mixed-precision solves/s with every input resident in HBM
  e2e       the same solve through tfs_solve() with page-locked host arrays:
            val, b, x copied in and x, r1 copied out inside every step
  roofline  the dominant kernels against the measured HBM copy bandwidth:
            the binary32 DIC application (level sweeps) for DIC workloads,
            else the binary32 SpMV; roofline_spmv is always the SpMV (the
            metric's SpMV GB/s)
  cpu_baseline  the oracle (the reference's sequential solver restated in C)
            on one host core, same system, one full binary64 DIC-CG solve

--impl reference times the reference's CPU solver (the oracle restatement;
no Fortran compiler exists on either machine) on all host cores, one
independent single-threaded solve per core (run_reference says how a step
is bounded).  Its processes build the same seeded system with the host-only
generator libtfs_synth.so and never load the GPU solver library.

Multi-GPU (torchrun): replicas only -- every rank solves its own seeded system
(seed + rank) with no collective on the data path; the step time is the max
over ranks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import itertools
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path[:0] = [str(REPO), str(REPO / "t-flows_gb300")]

METRIC = "CG/BiCG solves/s, p99 latency, SpMV GB/s: mixed vs FP64 at 1e-8 residual"
UNIT = "solves/s"
REL_TOL = 1e-8
BASE_SEED = 20261203

WORKLOADS = {
    # name: (kind, n, method, prec, description)
    "poisson128_dic_cg": (0, 128, 0, 2, "128^3 jittered-hex pressure Poisson, DIC-CG"),
    "poisson32_diag_cg": (0, 32, 0, 1, "32^3 jittered-hex pressure Poisson, diagonal CG"),
    "convdiff160_diag_bicg": (1, 160, 1, 1, "160^3 jittered-hex upwind convection-diffusion, diagonal BiCG"),
    "convdiff160_diag_cgs": (1, 160, 2, 1, "160^3 jittered-hex upwind convection-diffusion, diagonal CGS"),
}
SERVE_WORKLOAD = "serving_trace"
SERVE_DESC = ("Poisson arrivals at 400/s (seeded): 70% pressure solves (jittered-hex Poisson, "
              "diagonal CG, tol 1e-6 or 1e-8 relative at 50/50, limit 2000), 30% transport solves "
              "(upwind convection-diffusion, diagonal BiCG with the call sites' limit of 10 "
              "iterations, Compute_Scalar.f90:615-618); cells log-uniform in [10k, 2M] over a pool of "
              "resident systems; 150 GB device budget")
BATCH_WORKLOAD = "batched256_poisson_cg"
BATCH_DESC = ("256 independent jittered-hex pressure-Poisson systems, cells log-uniform in "
              "[5k, 500k] (k x k x m meshes), jitter U(0, 25%), own seed and permutation each; "
              "diagonal CG, all in one persistent cluster launch")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------- dist

class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ---------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- helpers

def measured_peak_gbs() -> tuple[float, str]:
    p = REPO / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# Binary32 CG SpMV kernels by tfs_stats.spmv_kernel (W: the slice width).
SPMV_KERNEL_NAMES = {
    0: ("k_mx_spmv_pq", "direct: per-row dependent loads"),
    1: ("k_spmv_pq_pipe<float,true,W>", "software-pipelined: next row's columns loaded during the gathers"),
}


def ncu_traffic(workload: str, kernel: str) -> float | None:
    """Per-launch DRAM bytes of `kernel` from the committed ncu summary."""
    p = REPO / "profiles" / "traffic.json"
    try:
        d = json.loads(p.read_text())
        return float(d[workload][kernel]["dram_bytes_per_launch"])
    except Exception:
        return None


def pct(v: list[float], q: float) -> float:
    s = sorted(v)
    if not s:
        return float("nan")
    k = min(len(s) - 1, max(0, int(round(q / 100.0 * (len(s) - 1)))))
    return s[k]


def workload_config(args, n: int, nnz: int) -> dict:
    """The `config` of a single-system workload, identical in both arms."""
    kind, nside, method, prec, desc = WORKLOADS[args.workload]
    world = int(os.environ.get("WORLD_SIZE", "1"))
    return {"workload": args.workload, "description": desc, "cells": n, "nnz": nnz,
            "solver": ["CG", "BiCG", "CGS"][method], "prec": ["none", "diag", "DIC"][prec],
            "stop": "||b-Ax|| < 1e-8 ||b||, x0 = 0", "niter_limit": args.niter,
            "l2": "inputs larger than L2 (matrix + vectors > 129 MB)" if nnz > 4000000
                  else "inputs smaller than L2 (L2-resident system)",
            "parallelism": f"replicas x{world}"}


# ---------------------------------------------------------------- our arm

def run_ours(args, dist: Dist) -> dict | None:
    import numpy as np

    import tflows
    from tflows.lib import TFS_FP64, TFS_MIXED, check, load_library
    from tflows.matrix_mod import ptr

    lib = load_library()
    check(lib.tfs_use_device(dist.local_rank), "tfs_use_device")
    kind, nside, method, prec, desc = WORKLOADS[args.workload]
    t0 = time.perf_counter()
    s = tflows.SynthSystem(kind, nside, jitter=0.2, seed=BASE_SEED + dist.rank)
    log(f"[bench] system {desc}: n={s.n} nnz={s.nnz} ({time.perf_counter() - t0:.1f}s)")
    t0 = time.perf_counter()
    import tflows.lib as L
    opts = {L.TFS_OPT_LAUNCH: 1 if args.eager else 0}
    for kv in args.option:
        name, value = kv.split("=")
        opts[getattr(L, "TFS_OPT_" + name.upper())] = int(value)
    sol = tflows.Solver(s.matrix(), options=opts)
    log(f"[bench] registered: {sol.stats()['n_levels']} levels ({time.perf_counter() - t0:.1f}s)")
    # Launch shapes of the single-solve kernels, picked on this system
    # (tfs_autotune) before anything is timed.
    tune = None
    if not args.no_autotune:
        tune = sol.autotune(s.val, TFS_MIXED, prec, 5)
        log(f"[bench] autotune: {tune}")
    n, nnz = s.n, s.nnz
    tol = REL_TOL * float(np.linalg.norm(s.b))
    h = sol.h

    def dalloc(nbytes):
        p = C.c_void_p()
        check(lib.tfs_device_alloc(nbytes, C.byref(p)), "tfs_device_alloc")
        return p.value

    def halloc(nbytes, dtype, count):
        p = C.c_void_p()
        check(lib.tfs_host_alloc(nbytes, C.byref(p)), "tfs_host_alloc")
        buf = (C.c_char * nbytes).from_address(p.value)
        return p.value, np.frombuffer(buf, dtype=dtype, count=count)

    d_val, d_b, d_x, d_r, d_zero = dalloc(8 * nnz), dalloc(8 * n), dalloc(8 * n), dalloc(8 * n), dalloc(8 * n)
    zeros = np.zeros(n)
    check(lib.tfs_copy(h, C.c_void_p(d_val), s.val.ctypes.data_as(C.c_void_p), 8 * nnz), "copy")
    check(lib.tfs_copy(h, C.c_void_p(d_b), s.b.ctypes.data_as(C.c_void_p), 8 * n), "copy")
    check(lib.tfs_copy(h, C.c_void_p(d_zero), zeros.ctypes.data_as(C.c_void_p), 8 * n), "copy")
    check(lib.tfs_sync(h), "sync")

    def step_resident():
        check(lib.tfs_copy(h, C.c_void_p(d_x), C.c_void_p(d_zero), 8 * n), "copy")
        check(lib.tfs_copy(h, C.c_void_p(d_r), C.c_void_p(d_b), 8 * n), "copy")
        return sol.solve_device(method, d_val, d_x, d_r, prec, args.niter, tol)

    def read_x():
        x = np.empty(n)
        check(lib.tfs_copy(h, x.ctypes.data_as(C.c_void_p), C.c_void_p(d_x), 8 * n), "copy")
        check(lib.tfs_sync(h), "sync")
        return x

    results = {}
    timed_launches = 0
    clock_info = None
    modes = [m for m in ((TFS_FP64, "fp64"), (TFS_MIXED, "mixed")) if m[1] in args.modes.split(",")]
    for mode, name in modes:
        sol.set_precision(mode)
        for _ in range(args.warmup):
            res = step_resident()
        dist.barrier()
        lat, launches = [], 0
        sampler = ClockSampler(dist.local_rank) if name == "mixed" else None
        if sampler:
            sampler.__enter__()
        check(lib.tfs_timer_start(h), "timer")
        for _ in range(args.steps):
            res = step_resident()
            st = sol.stats()
            lat.append(st["solve_ms"])
            launches += st["kernel_launches"]
        ms = C.c_double()
        check(lib.tfs_timer_stop(h, C.byref(ms)), "timer")
        if sampler:
            sampler.__exit__(None, None, None)
            clock_info = sampler.summary()
        dist.barrier()
        total_ms = dist.max(ms.value)
        st = sol.stats()
        results[name] = {
            "solves_per_s": dist.sum(args.steps) / (total_ms / 1e3),
            "ms_per_solve": total_ms / args.steps,
            "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
            "iterations": res.niter, "fin_res": res.fin_res, "status": res.status,
            "true_residuals": st["true_residuals"],
            "spmv_in_solve_us": (st["spmv_ns_total"] / max(1, st["spmv_launches"])) / 1e3,
            "sweep_in_solve_us": (st["sweep_ns_total"] / max(1, st["sweep_launches"])) / 1e3,
            "_x": read_x(),
        }
        if name == "mixed":
            timed_launches = launches
        log(f"[bench] {name}: {results[name]['solves_per_s']:.2f} solves/s, "
            f"{res.niter} it, p50 {results[name]['p50_ms']:.2f} ms")

    # SpMV alone (CUDA events, back-to-back launches on the resident matrix).
    spmv64_ms = sol.time_spmv(s.val, TFS_FP64, args.spmv_reps)
    spmv32_ms = sol.time_spmv(s.val, TFS_MIXED, args.spmv_reps)
    # The same SpMV on the same matrix in RCM row order (the layout of the
    # solves without DIC): the gathers of a warp's 32 rows then share
    # sectors, where the DIC level order scatters them.
    spmv_rcm = None
    if prec == 2:
        with tflows.Solver(s.matrix()) as sol_rcm:
            r32 = sol_rcm.time_spmv(s.val, TFS_MIXED, args.spmv_reps)
            r64 = sol_rcm.time_spmv(s.val, TFS_FP64, args.spmv_reps)
        spmv_rcm = {"fp32_us": round(r32 * 1e3, 2), "fp64_us": round(r64 * 1e3, 2),
                    "fp32_gbs": round((8 * nnz + 12 * n + 4) / (r32 * 1e-3) / 1e9, 1),
                    "fp64_gbs": round((12 * nnz + 20 * n + 4) / (r64 * 1e-3) / 1e9, 1)}
    bytes64 = 12 * nnz + 20 * n + 4
    bytes32 = 8 * nnz + 12 * n + 4
    # DIC application alone (both sweeps), when the workload uses DIC.
    prec32_ms = sol.time_prec(s.val, TFS_MIXED, args.spmv_reps) if prec == 2 else None
    prec_bytes32 = 8 * nnz + 24 * n
    # Device stamps of one binary32 DIC application's level launches: how a
    # level step splits into the hand-off between launches (the wait for the
    # previous level's completion) and the launch's own work.
    level_split = None
    if prec == 2 and sol.stats()["dic_kernel"] == 0:
        prof = sol.profile_prec(s.val, TFS_MIXED)
        work = [p["end_us"] - p["start_us"] for p in prof]
        gaps = [b["start_us"] - a["end_us"] for a, b in zip(prof, prof[1:])]
        level_split = {"launches": len(prof), "span_us": round(prof[-1]["end_us"] - prof[0]["start_us"], 2),
                       "work_us": round(sum(work), 2), "handoff_us": round(sum(gaps), 2),
                       "per_launch": [[p["launch"], round(p["start_us"], 2), round(p["end_us"], 2)] for p in prof],
                       "how": "tfs_profile_prec: global timer when each launch's blocks passed their dependency "
                              "wait (earliest) and finished (latest); hand-off = next start - this end"}

    # End to end through tfs_solve with page-locked host arrays (headline arithmetic).
    e2e = None
    if not args.no_e2e:
        sol.set_precision(modes[-1][0])
        p_val, h_val = halloc(8 * nnz, np.float64, nnz)
        p_x, h_x = halloc(8 * n, np.float64, n)
        p_r, h_r = halloc(8 * n, np.float64, n)
        h_val[:] = s.val
        e2e_ms = []
        for i in range(args.warmup + args.steps):
            h_x[:] = 0.0
            h_r[:] = s.b
            t = time.perf_counter()
            res = sol.solve(method, h_val, h_x, h_r, prec, args.niter, tol)
            if i >= args.warmup:
                e2e_ms.append((time.perf_counter() - t) * 1e3)
        e2e_total = dist.max(sum(e2e_ms))
        e2e = {"value": dist.sum(args.steps) / (e2e_total / 1e3), "unit": UNIT,
               "h2d_bytes_per_step": 8 * nnz + 16 * n, "d2h_bytes_per_step": 16 * n,
               "p50_ms": pct(e2e_ms, 50), "p99_ms": pct(e2e_ms, 99),
               "timing": "host wall clock around each tfs_solve call (copies included)"}
        for p in (p_val, p_x, p_r):
            lib.tfs_host_free(C.c_void_p(p))

    # The rows after the solve path, on the same mesh (outside the timed
    # region): Matrix_Mod_Topology built on the device against the host
    # builder, and the face-loop assembly on the device against the oracle.
    next_rows = None
    if dist.rank == 0 and not args.no_next_rows:
        next_rows = measure_next_rows(lib, sol, s, dalloc)
        next_rows["reference_meshes"] = measure_reference_meshes()
        next_rows["process_pattern"] = measure_process_pattern(lib)
    for p in (d_val, d_b, d_x, d_r, d_zero):
        lib.tfs_device_free(C.c_void_p(p))

    # CPU baseline and the error of both GPU solutions against the oracle.
    cpu = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        from oracle import tfs_oracle as O
        # A probe of a few iterations sizes the sample: one full solve (and
        # the error of the GPU solutions against it) when that takes at most
        # about a minute on one core, else a bounded run of iterations scaled
        # to the binary64 GPU solve's iteration count.
        probe = 8
        xp, rp = np.zeros(n), s.b.copy()
        t = time.perf_counter()
        O.solve(method, n, s.row, s.col, s.dia, s.val, xp, rp, prec, probe, tol)
        t_it = (time.perf_counter() - t) / probe
        gpu_its = (results.get("fp64") or next(iter(results.values())))["iterations"]
        if t_it * gpu_its <= 60.0:
            xo, ro = np.zeros(n), s.b.copy()
            t = time.perf_counter()
            it, ini, fin = O.solve(method, n, s.row, s.col, s.dia, s.val, xo, ro, prec, args.niter, tol)
            cpu_s = time.perf_counter() - t
            cpu = {"value": 1.0 / cpu_s, "unit": UNIT, "cores": 1, "kind": "port",
                   "sample": f"one full binary64 solve ({it} iterations, {cpu_s:.1f} s) of the same "
                             f"system on 1 host core; {os.cpu_count()} cores present",
                   "oracle_iterations": it}
            for name in results:
                x = results[name]["_x"]
                results[name]["rel_err_vs_oracle"] = float(np.linalg.norm(x - xo) / np.linalg.norm(xo))
                results[name]["iterations_vs_oracle"] = f"{results[name]['iterations']} vs {it}"
        else:
            k = max(probe, int(20.0 / max(t_it, 1e-9)))
            xp, rp = np.zeros(n), s.b.copy()
            t = time.perf_counter()
            O.solve(method, n, s.row, s.col, s.dia, s.val, xp, rp, prec, k, tol)
            per_it = (time.perf_counter() - t) / k
            cpu_s = per_it * gpu_its
            cpu = {"value": 1.0 / cpu_s, "unit": UNIT, "cores": 1, "kind": "port",
                   "sample": f"{k} binary64 iterations ({per_it * k:.1f} s) of the same system on 1 host "
                             f"core, scaled to the {gpu_its} iterations of the binary64 GPU solve (a full "
                             f"oracle solve would take about {cpu_s:.0f} s); {os.cpu_count()} cores present"}
    for name in results:
        results[name].pop("_x", None)

    peak, peak_src = measured_peak_gbs()
    achieved = bytes32 / (spmv32_ms * 1e-3) / 1e9
    st_k = sol.stats()
    kname, kdesc = SPMV_KERNEL_NAMES.get(st_k["spmv_kernel"], ("k_mx_spmv_pq", "direct"))
    kname = kname.replace("W", str(st_k["sell_width"]))
    roof_spmv = {"kernel": f"{kname} (binary32 SELL-32 SpMV + (p,q), {kdesc})", "bound": "hbm",
                 "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                 "frac": round(achieved / peak, 4), "peak_source": f"{peak_src} hbm_gbs",
                 "algorithmic_bytes_per_launch": bytes32,
                 "traffic": ncu_traffic(args.workload, kname.split("<")[0]),
                 "timing": "CUDA events, back-to-back launches on the handle's stream"}
    roof = roof_spmv
    if prec32_ms is not None:
        # The level sweeps are the dominant kernels of DIC-CG: one "launch" is
        # one preconditioner application (all level kernels of both sweeps).
        ach = prec_bytes32 / (prec32_ms * 1e-3) / 1e9
        roof = {"kernel": "k_sweep_level + k_sweep_tail1 (one binary32 DIC application: "
                          "forward levels, fused tails, backward levels)",
                "bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                "frac": round(ach / peak, 4), "peak_source": f"{peak_src} hbm_gbs",
                "algorithmic_bytes_per_launch": prec_bytes32,
                "us_per_application": round(prec32_ms * 1e3, 2), "level_split": level_split,
                "traffic": ncu_traffic(args.workload, "dic_application"),
                "timing": "CUDA events, back-to-back applications on the handle's stream"}
    mixed = results.get("mixed") or results["fp64"]
    fp64 = results.get("fp64") or mixed
    line = {
        "metric": METRIC, "value": round(mixed["solves_per_s"], 4), "unit": UNIT,
        "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(mixed["ms_per_solve"], 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner / f64 outer",
        "data": "synthetic (seeded jittered-hex mesh, random cell numbering, RHS U[-1,1])",
        "config": workload_config(args, n, nnz),
        "options": {kv.split("=")[0]: int(kv.split("=")[1]) for kv in args.option} or None,
        "p50_ms": round(mixed["p50_ms"], 4), "p99_ms": round(mixed["p99_ms"], 4),
        "fp64": results.get("fp64"), "mixed": results.get("mixed"),
        "mixed_over_fp64": round(mixed["solves_per_s"] / fp64["solves_per_s"], 4),
        "spmv": {"fp64_us": round(spmv64_ms * 1e3, 2), "fp32_us": round(spmv32_ms * 1e3, 2),
                 "fp64_gbs": round(bytes64 / (spmv64_ms * 1e-3) / 1e9, 1),
                 "fp32_gbs": round(achieved, 1), "timing": "CUDA events, back-to-back launches",
                 "rcm_order": dict(spmv_rcm, fp32_frac=round(spmv_rcm["fp32_gbs"] / peak, 4),
                                   layout="the same matrix in RCM row order (no DIC levels)")
                              if spmv_rcm else None},
        "roofline": roof, "roofline_spmv": roof_spmv, "autotune": tune, "next_rows": next_rows,
        "e2e": e2e, "gpu_launches": int(timed_launches),
        "clocks": clock_info,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    sol.close()
    return line if dist.rank == 0 else None


def measure_next_rows(lib, sol, s, dalloc) -> dict:
    """Device topology build and device face assembly of the workload's mesh
    (interior faces), each checked bit for bit against its CPU counterpart
    and timed beside it."""
    import numpy as np
    from oracle import tfs_oracle as O
    from tflows.lib import check
    from tflows.matrix_mod import Matrix_Mod_Topology, Matrix_Mod_Topology_Device

    faces = s.faces_c
    Matrix_Mod_Topology_Device(64, np.zeros((0, 2), np.int32))      # warm-up
    t = time.perf_counter()
    dev = Matrix_Mod_Topology_Device(s.n, faces)
    topo_dev_ms = (time.perf_counter() - t) * 1e3
    t = time.perf_counter()
    host = Matrix_Mod_Topology(s.n, faces)
    topo_host_ms = (time.perf_counter() - t) * 1e3
    topo_same = bool(np.array_equal(dev.col, host.col) and np.array_equal(dev.pos, host.pos)
                     and np.array_equal(dev.mir, host.mir) and np.array_equal(dev.row, host.row)
                     and np.array_equal(dev.dia, host.dia))
    # Assembly: pressure-like coefficients per face, an inertial cell term.
    rng = np.random.default_rng(BASE_SEED)
    nf = len(faces)
    a = rng.uniform(0.5, 1.5, nf)
    cell = rng.uniform(0.0, 1e-3, s.n)
    sol.faces_register(faces, dev.pos)
    d_a, d_c, d_v = dalloc(8 * nf), dalloc(8 * s.n), dalloc(8 * s.nnz)
    zeros = np.zeros(s.nnz)
    h = sol.h
    check(lib.tfs_copy(h, C.c_void_p(d_a), a.ctypes.data_as(C.c_void_p), 8 * nf), "copy")
    check(lib.tfs_copy(h, C.c_void_p(d_c), cell.ctypes.data_as(C.c_void_p), 8 * s.n), "copy")
    times = []
    for rep in range(4):
        check(lib.tfs_copy(h, C.c_void_p(d_v), zeros.ctypes.data_as(C.c_void_p), 8 * s.nnz), "copy")
        check(lib.tfs_timer_start(h), "timer")
        check(lib.tfs_assemble_faces_device(h, C.c_void_p(d_a), C.c_void_p(d_a), C.c_void_p(d_a),
                                            C.c_void_p(d_a), C.c_void_p(d_c), C.c_void_p(d_v)), "assemble")
        ms = C.c_double()
        check(lib.tfs_timer_stop(h, C.byref(ms)), "timer")
        if rep:
            times.append(ms.value)
    val = np.empty(s.nnz)
    check(lib.tfs_copy(h, val.ctypes.data_as(C.c_void_p), C.c_void_p(d_v), 8 * s.nnz), "copy")
    check(lib.tfs_sync(h), "sync")
    for p in (d_a, d_c, d_v):
        lib.tfs_device_free(C.c_void_p(p))
    t = time.perf_counter()
    want = O.assemble_faces(s.n, faces.reshape(-1), dev.pos.reshape(-1), dev.dia, a, a, a, a, cell, zeros)
    asm_cpu_ms = (time.perf_counter() - t) * 1e3
    return {
        "topology_device_ms": round(topo_dev_ms, 2), "topology_host_ms": round(topo_host_ms, 2),
        "topology_identical": topo_same,
        "assemble_device_ms": round(statistics.median(times), 4), "assemble_oracle_ms": round(asm_cpu_ms, 2),
        "assemble_identical": bool(np.array_equal(val, want)),
        "timing": "topology: host wall clock around the synchronous calls (the device build includes "
                  "its scratch allocation and the copies of faces in and arrays out); assembly: CUDA "
                  "events on the handle's stream, median of 3 after a warm-up",
    }


def measure_reference_meshes() -> dict:
    """DIC-CG on the reference's own test meshes (Gambit files of its Tests/
    directory, committed as tests/golden/gambit_*.npz): binary64 and mixed
    solves against the oracle, in the meshes' own cell numbering."""
    import numpy as np
    from oracle import tfs_oracle as O
    from tflows import TFS_CG, TFS_FP64, TFS_MIXED, Solver
    from tflows import gambit as G

    out = {}
    for name in ("chan", "plain50"):
        s = G.system_from_fixture(REPO / "tests" / "golden" / f"gambit_{name}.npz")
        tol = 1e-8 * float(np.linalg.norm(s.b))
        xo, ro = np.zeros(s.n), s.b.copy()
        t = time.perf_counter()
        it, ini, fin = O.solve(0, s.n, s.row, s.col, s.dia, s.val, xo, ro, 2, 5000, tol)
        cpu_ms = (time.perf_counter() - t) * 1e3
        row = {"cells": s.n, "nnz": s.nnz, "oracle_iterations": it, "oracle_ms": round(cpu_ms, 2)}
        for mode, tag in ((TFS_FP64, "fp64"), (TFS_MIXED, "mixed")):
            with Solver(s.matrix(), precision=mode) as sol:
                ms = []
                for rep in range(4):
                    x, r = np.zeros(s.n), s.b.copy()
                    res = sol.solve(TFS_CG, s.val, x, r, 2, 5000, tol)
                    if rep:
                        ms.append(sol.stats()["solve_ms"])
                st = sol.stats()
                row[tag] = {"iterations": res.niter, "status": res.status,
                            "device_ms": round(statistics.median(ms), 3),
                            "rel_err_vs_oracle": float(np.linalg.norm(x - xo) / np.linalg.norm(xo)),
                            "dic_levels": st["n_levels"]}
        out[name] = row
    out["timing"] = ("device time of one tfs_solve (CUDA events inside the library, median of 3 "
                     "after a warm-up); oracle: one binary64 solve on one host core")
    return out


def measure_process_pattern(lib, calls: int = 20) -> dict:
    """The solver calls T-FlowS's Process makes, replayed on the reference's
    own meshes through the Fortran-shaped entry points with host arrays:
    per outer iteration a pressure-correction solve Bicg(A, pp, b, PREC, 40,
    PP%STol) (Compute_Pressure_Simple.f90:190-193) and a momentum solve
    Cg(A, u, b, PREC, 10, U%STol) (NewUVW.f90:592-599), with the settings of
    the Flow_over_plain deck (T-FlowS.cmn: ic preconditioning, absolute
    tolerances 1e-6).  Each call uploads the matrix values, b and x and
    reads x and r1 back, as the drop-in does; the right-hand side changes
    from call to call (seeded U[-1,1]) and x starts from zero.  The mesh's
    pressure matrix stands in for both systems (the momentum matrix needs
    the flow field).  Timed against the oracle making the same calls on one
    host core; every binary64 GPU call is checked against the oracle's."""
    import numpy as np
    from oracle import tfs_oracle as O
    from tflows import TFS_FP64, TFS_MIXED
    from tflows import gambit as G
    out = {}
    kinds = (("pressure_bicg", 1, 40), ("momentum_cg", 0, 10))
    for name in ("chan", "plain50"):
        s = G.system_from_fixture(REPO / "tests" / "golden" / f"gambit_{name}.npz")
        rng = np.random.default_rng(BASE_SEED)
        rhs = [rng.uniform(-1.0, 1.0, s.n) for _ in range(calls)]
        P = lambda a, t: a.ctypes.data_as(C.POINTER(t))
        row = {"cells": s.n, "nnz": s.nnz, "calls": 2 * calls,
               "settings": "prec 2 (ic), tol 1e-6 absolute, pressure BiCG limit 40, momentum CG limit 10"}
        # the oracle, one host core
        ref, t_cpu = {}, []
        for j in range(calls):
            for kname, method, lim in kinds:
                x, r = np.zeros(s.n), rhs[j].copy()
                t = time.perf_counter()
                it, _, _ = O.solve(method, s.n, s.row, s.col, s.dia, s.val, x, r, 2, lim, 1e-6)
                t_cpu.append(time.perf_counter() - t)
                ref[(kname, j)] = (x, it)
        row["oracle_ms_per_call"] = round(statistics.mean(t_cpu) * 1e3, 4)
        for mode, tag in ((TFS_FP64, "fp64"), (TFS_MIXED, "mixed")):
            lib.tfs_set_default_precision(mode)
            t_gpu, errs, its, its_ref = [], [], [], []
            for rep in range(2):             # the first pass builds the handle and its graphs
                t_gpu, errs, its, its_ref = [], [], [], []
                for j in range(calls):
                    for kname, method, lim in kinds:
                        x, r = np.zeros(s.n), rhs[j].copy()
                        niter = C.c_int32(lim)
                        ini, fin = C.c_double(0.0), C.c_double(0.0)
                        fn = lib.tfs_bicg if method == 1 else lib.tfs_cg
                        t = time.perf_counter()
                        st = fn(s.n, s.nnz, P(s.row, C.c_int32), P(s.col, C.c_int32), P(s.dia, C.c_int32),
                                P(s.val, C.c_double), P(x, C.c_double), P(r, C.c_double), 2, C.byref(niter),
                                1e-6, C.byref(ini), C.byref(fin))
                        t_gpu.append(time.perf_counter() - t)
                        if st not in (0, 4):
                            raise RuntimeError(f"{fn.__name__}: status {st}")
                        xo, it = ref[(kname, j)]
                        its.append(niter.value)
                        its_ref.append(it)
                        errs.append(float(np.linalg.norm(x - xo) / max(np.linalg.norm(xo), 1e-300)))
            row[tag] = {"ms_per_call": round(statistics.mean(t_gpu) * 1e3, 4),
                        "p99_ms": round(pct([t * 1e3 for t in t_gpu], 99), 4),
                        "speedup_vs_oracle_1core": round(statistics.mean(t_cpu) / statistics.mean(t_gpu), 3),
                        "iterations_equal_to_oracle": sum(1 for a, b in zip(its, its_ref) if a == b),
                        "max_abs_iteration_difference": max(abs(a - b) for a, b in zip(its, its_ref)),
                        "max_rel_err_vs_oracle": max(errs)}
        lib.tfs_set_default_precision(TFS_FP64)
        out[name] = row
    out["timing"] = ("host wall clock around each tfs_bicg / tfs_cg call (value, b, x uploads and x, r1 "
                     "read-back included; handle and graphs built in an untimed first pass) and around each "
                     "oracle call on one host core")
    return out


# ---------------------------------------------------------------- shared by the legs

def cg_iteration_bytes(n: int, nnz: int, mixed: bool) -> int:
    """Algorithmic bytes of one diagonal-CG iteration: the matrix once (values
    and column indices), the row geometry, and every distinct vector read or
    written once (p, q, r, x, the diagonal: 12 nnz + 76 n + 4 in binary64).
    Mixed: 4-byte values and vectors in the iteration, the binary32
    correction e in place of x (8 nnz + 40 n + 4); its binary64 true
    residuals are not counted, so the mixed figure is a lower bound."""
    return 8 * nnz + 40 * n + 4 if mixed else 12 * nnz + 76 * n + 4


def _pinned(lib, nbytes, dtype, count):
    import numpy as np
    from tflows.lib import check
    p = C.c_void_p()
    check(lib.tfs_host_alloc(max(1, nbytes), C.byref(p)), "tfs_host_alloc")
    buf = (C.c_char * max(1, nbytes)).from_address(p.value)
    return p.value, np.frombuffer(buf, dtype=dtype, count=count)


def _oracle_one(arg):
    """One oracle solve of a seeded system (spawned worker)."""
    sys.path[:0] = [str(REPO), str(REPO / "t-flows_gb300")]
    import numpy as np
    from oracle import tfs_oracle as O
    from tflows.synth import SynthSystem
    kind, nx, ny, nz, jit, sd, method, prec, niter, tol_rel = arg
    s = SynthSystem(kind, nx, ny, nz, jitter=jit, seed=sd)
    x, r = np.zeros(s.n), s.b.copy()
    t = time.perf_counter()
    it, _, _ = O.solve(method, s.n, s.row, s.col, s.dia, s.val, x, r, prec, niter,
                       tol_rel * float(np.linalg.norm(s.b)))
    return x, it, time.perf_counter() - t


def oracle_pool(jobs):
    """Oracle solves on the host cores (spawned processes: a forked pool would
    inherit the CUDA context)."""
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
        return pool.map(_oracle_one, jobs)


# ---------------------------------------------------------------- serving leg

def serving_leg(args, dist: Dist, n_pool: int, n_requests: int) -> dict:
    """Replay a seeded Poisson-arrival trace through the request server, each
    arithmetic twice: operands resident on the device (tfs_server_submit) and
    end to end from page-locked host arrays (tfs_server_submit_host: val, b
    and x copied in and x, r1 copied out by every request).  Latency =
    submit -> completion."""
    import concurrent.futures as cf

    import numpy as np

    import tflows
    from tflows.lib import TFS_BICG, TFS_CG, TFS_FP64, TFS_MIXED, check, load_library
    from tflows.synth import serving_pool_specs, uniform

    lib = load_library()
    check(lib.tfs_use_device(dist.local_rank), "tfs_use_device")
    seed = BASE_SEED + 7 + dist.rank
    specs = serving_pool_specs(n_pool, seed)
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        systems = list(ex.map(lambda sp: tflows.SynthSystem(sp[0], sp[1], sp[2], sp[3], jitter=0.2,
                                                            seed=sp[4]), specs))
    log(f"[bench] serving pool: {len(systems)} systems, {sum(s.n for s in systems)} cells "
        f"({time.perf_counter() - t0:.1f}s)")

    def dalloc(nbytes):
        p = C.c_void_p()
        check(lib.tfs_device_alloc(nbytes, C.byref(p)), "tfs_device_alloc")
        return p.value

    slots = args.serve_slots
    dev, host, pinned = [], [], []
    for s in systems:
        d = {"val": dalloc(8 * s.nnz), "b": dalloc(8 * s.n),
             "x": [dalloc(8 * s.n) for _ in range(slots)], "r": [dalloc(8 * s.n) for _ in range(slots)]}
        check(lib.tfs_memcpy(C.c_void_p(d["val"]), s.val.ctypes.data_as(C.c_void_p), 8 * s.nnz), "copy")
        check(lib.tfs_memcpy(C.c_void_p(d["b"]), s.b.ctypes.data_as(C.c_void_p), 8 * s.n), "copy")
        dev.append(d)
        pv, hv = _pinned(lib, 8 * s.nnz, np.float64, s.nnz)
        hv[:] = s.val
        hx = [_pinned(lib, 8 * s.n, np.float64, s.n) for _ in range(slots)]
        hr = [_pinned(lib, 8 * s.n, np.float64, s.n) for _ in range(slots)]
        pinned += [pv] + [q[0] for q in hx + hr]
        host.append({"val": hv, "x": [q[1] for q in hx], "r": [q[1] for q in hr]})
    # The trace: exponential inter-arrival times, request kind from the pool.
    gaps = [-math.log(1.0 - uniform(seed, 41, j)) / args.serve_rate for j in range(n_requests)]
    arrivals = list(itertools.accumulate(gaps))
    reqs = []
    for j in range(n_requests):
        k = min(n_pool - 1, int(uniform(seed, 42, j) * n_pool))
        tol_rel = 1e-6 if uniform(seed, 43, j) < 0.5 else 1e-8
        reqs.append((arrivals[j], k, tol_rel))
    bnorm = [float(np.linalg.norm(s.b)) for s in systems]

    def method_of(k):
        # pressure: diagonal CG (limit 2000); transport: diagonal BiCG with the
        # call sites' limit of 10 iterations (Compute_Scalar.f90:615-618)
        return (TFS_CG, 2000) if specs[k][0] == 0 else (TFS_BICG, 10)

    def replay(mode, on_host):
        budget = int(args.serve_budget_gb * 1e9)
        lat, qd, runm, its, status = [], [], [], [], []
        bytes_alg = 0
        with tflows.Server(budget, max_inflight=args.serve_inflight, device=dist.local_rank) as srv:
            ids = [srv.add_system(s.n, s.row, s.col, s.dia) for s in systems]

            def submit(k, slot, niter, tol):
                method = method_of(k)[0]
                if on_host:
                    h = host[k]
                    h["r"][slot][:] = systems[k].b
                    return srv.submit_host(ids[k], method, 1, h["val"], h["x"][slot], h["r"][slot],
                                           niter, tol, mode=mode, x0_zero=True)
                d = dev[k]
                return srv.submit(ids[k], method, 1, d["val"], d["x"][slot], d["r"][slot], niter, tol,
                                  mode=mode, d_b=d["b"], x0_zero=True)

            # Warm every system once (layout, graphs), outside the trace.
            for t in [submit(k, 0, 10, 0.0) for k in range(len(systems))]:
                srv.wait(t)
            pending = {}            # (system, slot) -> ticket still using it
            next_slot = [0] * len(systems)
            tickets = []
            start = time.perf_counter()
            for (t_arr, k, tol_rel) in reqs:
                now = time.perf_counter() - start
                if t_arr > now:
                    time.sleep(t_arr - now)
                slot = next_slot[k] % slots
                next_slot[k] += 1
                if (k, slot) in pending:       # slot still in use: wait for it
                    tickets.append((pending[(k, slot)][1], srv.wait(pending.pop((k, slot))[0])))
                t = submit(k, slot, method_of(k)[1], tol_rel * bnorm[k])
                pending[(k, slot)] = (t, k)
            for t, k in pending.values():
                tickets.append((k, srv.wait(t)))
            span = time.perf_counter() - start
            stats = srv.stats()
        for k, res in tickets:
            lat.append(res["latency_ms"]); qd.append(res["queued_ms"]); runm.append(res["run_ms"])
            its.append(res["niter"]); status.append(res["status"])
            it_done = min(res["niter"], method_of(k)[1])
            bytes_alg += it_done * cg_iteration_bytes(systems[k].n, systems[k].nnz, mode == TFS_MIXED)
        out = {"solves_per_s": len(tickets) / span, "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99),
               "mean_ms": statistics.mean(lat), "queue_p99_ms": pct(qd, 99), "run_p50_ms": pct(runm, 50),
               "requests": len(tickets), "span_s": span, "failed": sum(1 for x in status if x != 0),
               "evictions": stats["evictions"], "peak_running": stats["peak_running"],
               "resident_gb": stats["resident_bytes"] / 1e9, "_bytes": bytes_alg}
        return out

    results, clock_info = {}, None
    for mode, name in ((TFS_FP64, "fp64"), (TFS_MIXED, "mixed")):
        dist.barrier()
        sampler = ClockSampler(dist.local_rank) if mode == TFS_MIXED else None
        if sampler:
            sampler.__enter__()
        results[name] = replay(mode, False)
        if sampler:
            sampler.__exit__(None, None, None)
            clock_info = sampler.summary()
        results[name + "_e2e"] = replay(mode, True)
        log(f"[bench] serving {name}: {results[name]['solves_per_s']:.1f} solves/s, "
            f"p50 {results[name]['p50_ms']:.2f} ms, p99 {results[name]['p99_ms']:.2f} ms; end to end "
            f"{results[name + '_e2e']['solves_per_s']:.1f} solves/s, p99 {results[name + '_e2e']['p99_ms']:.2f} ms")
    # Error against the oracle: one request of each of the 4 smallest systems,
    # both arithmetics, tolerance 1e-8 (transport: the 10-iteration limit).
    sample = sorted(range(n_pool), key=lambda k: systems[k].n)[:4]
    jobs = [(specs[k][0], specs[k][1], specs[k][2], specs[k][3], 0.2, specs[k][4], method_of(k)[0], 1,
             method_of(k)[1], 1e-8) for k in sample]
    refs = oracle_pool(jobs) if dist.rank == 0 and not args.no_cpu_baseline else None
    errs = {"fp64": [], "mixed": []}
    if refs is not None:
        with tflows.Server(int(args.serve_budget_gb * 1e9), device=dist.local_rank) as srv:
            for k, (xo, it, _) in zip(sample, refs):
                sid = srv.add_system(systems[k].n, systems[k].row, systems[k].col, systems[k].dia)
                for mode, name in ((TFS_FP64, "fp64"), (TFS_MIXED, "mixed")):
                    h = host[k]
                    h["r"][0][:] = systems[k].b
                    srv.wait(srv.submit_host(sid, method_of(k)[0], 1, h["val"], h["x"][0], h["r"][0],
                                             method_of(k)[1], 1e-8 * bnorm[k], mode=mode, x0_zero=True))
                    errs[name].append(float(np.linalg.norm(h["x"][0] - xo) / np.linalg.norm(xo)))
    for d in dev:
        for q in [d["val"], d["b"]] + d["x"] + d["r"]:
            lib.tfs_device_free(C.c_void_p(q))
    for q in pinned:
        lib.tfs_host_free(C.c_void_p(q))
    peak, peak_src = measured_peak_gbs()
    for name in ("fp64", "mixed"):
        r = results[name]
        ach = r.pop("_bytes") / r["span_s"] / 1e9
        r["roofline"] = {"bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(ach / peak, 4), "peak_source": f"{peak_src} hbm_gbs",
                         "note": "algorithmic bytes of every request's iterations over the trace's wall "
                                 "span (a lower bound: idle gaps between arrivals included)"}
        results[name + "_e2e"].pop("_bytes")
        r["rel_err_vs_oracle_max"] = max(errs[name]) if errs[name] else None
    mixed, fp64 = results["mixed"], results["fp64"]
    return {
        "workload": SERVE_WORKLOAD, "description": SERVE_DESC, "pool": len(systems),
        "cells": sum(s.n for s in systems), "requests": len(reqs), "rate_per_s": args.serve_rate,
        "max_inflight": args.serve_inflight, "budget_gb": args.serve_budget_gb,
        "mixed": mixed, "fp64": fp64,
        "e2e": {"value": round(results["mixed_e2e"]["solves_per_s"], 3), "unit": UNIT,
                "p50_ms": round(results["mixed_e2e"]["p50_ms"], 3),
                "p99_ms": round(results["mixed_e2e"]["p99_ms"], 3),
                "fp64_value": round(results["fp64_e2e"]["solves_per_s"], 3),
                "fp64_p99_ms": round(results["fp64_e2e"]["p99_ms"], 3),
                "h2d_bytes_per_request": "8 nnz + 16 n of the request's system",
                "d2h_bytes_per_request": "16 n",
                "timing": "host wall clock over the trace; every request copies val, b, x in and x, r1 "
                          "out from page-locked host arrays on its system's stream"},
        "mixed_over_fp64": round(mixed["solves_per_s"] / fp64["solves_per_s"], 3),
        "mixed_over_fp64_e2e": round(results["mixed_e2e"]["solves_per_s"] /
                                     results["fp64_e2e"]["solves_per_s"], 3),
        "error_sample": f"one request of each of the {len(sample)} smallest pool systems per arithmetic "
                        f"(tol 1e-8 relative; transport solves stop at their 10-iteration limit) against "
                        f"the oracle",
        "clocks": clock_info,
    }


def run_serving(args, dist: Dist) -> dict | None:
    leg = serving_leg(args, dist, args.serve_pool, args.serve_requests)
    mixed = leg["mixed"]
    line = {
        "metric": METRIC, "value": round(dist.sum(mixed["solves_per_s"]), 3), "unit": UNIT,
        "n_gpus": dist.world, "steps": leg["requests"], "warmup": leg["pool"],
        "ms_per_step": round(mixed["mean_ms"], 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 inner / f64 outer",
        "data": "synthetic (seeded jittered-hex meshes, random cell numbering, RHS U[-1,1], seeded trace)",
        "config": serving_config(args),
        "p50_ms": round(mixed["p50_ms"], 3), "p99_ms": round(mixed["p99_ms"], 3),
        "roofline": mixed["roofline"], "gpu_launches": None, "clocks": leg.pop("clocks"), "e2e": leg["e2e"],
        "serving": leg,
    }
    return line if dist.rank == 0 else None


def serving_config(args) -> dict:
    world = int(os.environ.get("WORLD_SIZE", "1"))
    return {"workload": SERVE_WORKLOAD, "description": SERVE_DESC, "pool": args.serve_pool,
            "requests": args.serve_requests, "rate_per_s": args.serve_rate,
            "max_inflight": args.serve_inflight, "budget_gb": args.serve_budget_gb,
            "parallelism": f"replicas x{world}"}


# ---------------------------------------------------------------- batched leg

def batch_specs(n_sys: int, seed: int) -> list[tuple[int, int, int, float, int]]:
    from tflows.synth import batched_poisson_specs
    return batched_poisson_specs(n_sys, seed)


def batched_leg(args, dist: Dist, n_sys: int, steps: int, warmup: int) -> dict:
    """n_sys uneven systems (the first n_sys of the seeded 256-system
    specification): the batched cluster solve in binary64 and mixed
    precision against the plain binary64 single-system path (one graph-
    captured tfs_solve_device per system), with operands resident on the
    device, and end to end through tfs_batch_solve with page-locked host
    arrays."""
    import concurrent.futures as cf

    import numpy as np

    import tflows
    from tflows.lib import TFS_CG, TFS_FP64, TFS_MIXED, check, load_library

    lib = load_library()
    check(lib.tfs_use_device(dist.local_rank), "tfs_use_device")
    specs = batch_specs(256, BASE_SEED + dist.rank)[:n_sys]
    t0 = time.perf_counter()

    def make(spec):
        nx, ny, nz, jit, sd = spec
        lib.tfs_use_device(dist.local_rank)
        s = tflows.SynthSystem(0, nx, ny, nz, jitter=jit, seed=sd)
        return s, tflows.Solver(s.matrix())

    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 1)) as ex:
        pairs = list(ex.map(make, specs))
    systems = [p[0] for p in pairs]
    solvers = [p[1] for p in pairs]
    n_rows = sum(s.n for s in systems)
    nnz_all = sum(s.nnz for s in systems)
    log(f"[bench] batch of {len(systems)} systems, {n_rows} cells, {nnz_all} entries "
        f"({time.perf_counter() - t0:.1f}s to build and register)")

    def dalloc(nbytes):
        p = C.c_void_p()
        check(lib.tfs_device_alloc(nbytes, C.byref(p)), "tfs_device_alloc")
        return p.value

    d_val, d_b, d_x, d_r, d_zero = [], [], [], [], []
    for s, sv in zip(systems, solvers):
        d_val.append(dalloc(8 * s.nnz)); d_b.append(dalloc(8 * s.n)); d_x.append(dalloc(8 * s.n))
        d_r.append(dalloc(8 * s.n)); d_zero.append(dalloc(8 * s.n))
        z = np.zeros(s.n)
        check(lib.tfs_copy(sv.h, C.c_void_p(d_val[-1]), s.val.ctypes.data_as(C.c_void_p), 8 * s.nnz), "copy")
        check(lib.tfs_copy(sv.h, C.c_void_p(d_b[-1]), s.b.ctypes.data_as(C.c_void_p), 8 * s.n), "copy")
        check(lib.tfs_copy(sv.h, C.c_void_p(d_zero[-1]), z.ctypes.data_as(C.c_void_p), 8 * s.n), "copy")
        check(lib.tfs_sync(sv.h), "sync")
    tols = np.array([REL_TOL * float(np.linalg.norm(s.b)) for s in systems])
    nsys = len(systems)
    batch = tflows.Batch(solvers)
    ptrs = lambda a: (C.c_void_p * len(a))(*a)
    reset_dst = ptrs(d_x + d_r)
    reset_src = ptrs(d_zero + d_b)
    reset_bytes = (C.c_size_t * (2 * nsys))(*([8 * s.n for s in systems] * 2))

    def batch_step(mode):
        check(lib.tfs_batch_copy(batch.b, 2 * nsys, reset_dst, reset_src, reset_bytes), "tfs_batch_copy")
        return batch.solve_device(TFS_CG, 1, d_val, d_x, d_r, args.niter, tols, mode=mode)

    # Autotune the cluster shape on the workload itself (one solve per shape).
    tune = {}
    for cl in (4, 8, 16):
        for tpb in (256, 512):
            try:
                batch.configure(cl, tpb)
                batch_step(TFS_MIXED)
                t = time.perf_counter()
                batch_step(TFS_MIXED)
                tune[(cl, tpb)] = time.perf_counter() - t
            except Exception as e:  # a shape that cannot be resident
                log(f"[bench] cluster {cl} x {tpb}: {e}")
    best = min(tune, key=tune.get)
    batch.configure(*best)
    log(f"[bench] autotuned cluster {best[0]} x {best[1]} threads: "
        + ", ".join(f"{k[0]}x{k[1]}={v * 1e3:.1f}ms" for k, v in sorted(tune.items())))

    def read_xs():
        out = []
        for k, (s, sv) in enumerate(zip(systems, solvers)):
            x = np.empty(s.n)
            check(lib.tfs_copy(sv.h, x.ctypes.data_as(C.c_void_p), C.c_void_p(d_x[k]), 8 * s.n), "copy")
            check(lib.tfs_sync(sv.h), "sync")
            out.append(x)
        return out

    results, xs_by, clock_info = {}, {}, None
    peak, peak_src = measured_peak_gbs()
    for mode, name in ((TFS_FP64, "batched_fp64"), (TFS_MIXED, "batched_mixed")):
        for _ in range(warmup):
            res = batch_step(mode)
        dist.barrier()
        sampler = ClockSampler(dist.local_rank) if mode == TFS_MIXED else None
        if sampler:
            sampler.__enter__()
        t = time.perf_counter()
        lat = []
        for _ in range(steps):
            res = batch_step(mode)
            lat.append(res.ms)
        wall = time.perf_counter() - t
        if sampler:
            sampler.__exit__(None, None, None)
            clock_info = sampler.summary()
        dist.barrier()
        wall = dist.max(wall)
        its = [int(v) for v in res.niter]
        alg = sum(min(it, args.niter) * cg_iteration_bytes(s.n, s.nnz, mode == TFS_MIXED)
                  for it, s in zip(its, systems))
        dev_ms = statistics.mean(lat)
        ach = alg / (dev_ms * 1e-3) / 1e9
        results[name] = {"solves_per_s": dist.sum(nsys * steps) / wall,
                         "ms_per_batch": wall / steps * 1e3,
                         "device_ms_per_batch": dev_ms,
                         "iterations_total": int(sum(its)), "iterations_max": int(max(its)),
                         "failed": int((res.status != 0).sum()),
                         "roofline": {"kernel": f"k_batch<CG,{'float' if mode == TFS_MIXED else 'double'}> "
                                                f"(+ k_batch_gather): whole solves, one {best[0]}-CTA "
                                                f"cluster per system",
                                      "bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
                                      "frac": round(ach / peak, 4), "peak_source": f"{peak_src} hbm_gbs",
                                      "algorithmic_bytes_per_launch": alg,
                                      "timing": "CUDA events around the gather and the persistent launch"}}
        xs_by[name] = read_xs()
        log(f"[bench] {name}: {results[name]['solves_per_s']:.1f} solves/s "
            f"({dev_ms:.2f} ms device, {ach:.0f} GB/s algorithmic)")

    # Plain binary64 path: one graph-captured single-system solve per system.
    for sv in solvers:
        sv.set_precision(TFS_FP64)

    def plain_pass():
        its = 0
        for k, sv in enumerate(solvers):
            check(lib.tfs_copy(sv.h, C.c_void_p(d_x[k]), C.c_void_p(d_zero[k]), 8 * systems[k].n), "copy")
            check(lib.tfs_copy(sv.h, C.c_void_p(d_r[k]), C.c_void_p(d_b[k]), 8 * systems[k].n), "copy")
            r = sv.solve_device(TFS_CG, d_val[k], d_x[k], d_r[k], 1, args.niter, float(tols[k]))
            its += r.niter
        return its
    plain_pass()
    t = time.perf_counter()
    plain_steps = max(1, steps // 5)
    for _ in range(plain_steps):
        its = plain_pass()
    wall = dist.max(time.perf_counter() - t)
    results["plain_fp64"] = {"solves_per_s": dist.sum(nsys * plain_steps) / wall,
                             "ms_per_pass": wall / plain_steps * 1e3, "iterations_total": its}
    log(f"[bench] plain fp64: {results['plain_fp64']['solves_per_s']:.1f} solves/s")

    # End to end: tfs_batch_solve with page-locked host arrays (copies of
    # every system's val, b, x in and x, r1 out inside each step).
    h_val, h_x, h_r, pinned = [], [], [], []
    for s in systems:
        pv, v = _pinned(lib, 8 * s.nnz, np.float64, s.nnz)
        v[:] = s.val
        px, x = _pinned(lib, 8 * s.n, np.float64, s.n)
        pr, r = _pinned(lib, 8 * s.n, np.float64, s.n)
        h_val.append(v); h_x.append(x); h_r.append(r); pinned += [pv, px, pr]
    e2e_ms = []
    for i in range(warmup + steps):
        for k, s in enumerate(systems):
            h_x[k][:] = 0.0
            h_r[k][:] = s.b
        t = time.perf_counter()
        batch.solve(TFS_CG, 1, h_val, h_x, h_r, args.niter, tols, mode=TFS_MIXED)
        if i >= warmup:
            e2e_ms.append((time.perf_counter() - t) * 1e3)
    for q in pinned:
        lib.tfs_host_free(C.c_void_p(q))
    e2e_total = dist.max(sum(e2e_ms))
    e2e = {"value": round(dist.sum(nsys * steps) / (e2e_total / 1e3), 3), "unit": UNIT,
           "h2d_bytes_per_step": int(sum(8 * s.nnz + 16 * s.n for s in systems)),
           "d2h_bytes_per_step": int(sum(16 * s.n for s in systems)),
           "p50_ms_per_batch": round(pct(e2e_ms, 50), 3),
           "timing": "host wall clock around each tfs_batch_solve (copies included), mixed precision"}

    # Error against the oracle on a sample: every eighth system.
    sample = list(range(0, nsys, 8))
    errs = {}
    if dist.rank == 0 and not args.no_cpu_baseline:
        t = time.perf_counter()
        refs = oracle_pool([(0, *specs[k][:3], specs[k][3], specs[k][4], 0, 1, args.niter, REL_TOL)
                            for k in sample])
        log(f"[bench] batch oracle sample: {len(sample)} systems ({time.perf_counter() - t:.1f}s)")
        for name in ("batched_fp64", "batched_mixed"):
            e = [float(np.linalg.norm(xs_by[name][k] - xo) / np.linalg.norm(xo))
                 for k, (xo, it, _) in zip(sample, refs)]
            results[name]["rel_err_vs_oracle_max"] = max(e)
        errs = {"systems": len(sample), "oracle_iterations": [int(it) for _, it, _ in refs]}
    batch.close()
    for sv in solvers:
        sv.close()
    for q in d_val + d_b + d_x + d_r + d_zero:
        lib.tfs_device_free(C.c_void_p(q))
    mixed = results["batched_mixed"]
    return {
        "workload": BATCH_WORKLOAD, "description": BATCH_DESC, "systems": nsys, "cells": n_rows,
        "nnz": nnz_all, "solver": "CG", "prec": "diag", "stop": "||b-Ax|| < 1e-8 ||b|| per system, x0 = 0",
        "cluster": best[0], "threads_per_cta": best[1], "steps": steps,
        "batched_mixed": mixed, "batched_fp64": results["batched_fp64"], "plain_fp64": results["plain_fp64"],
        "mixed_batched_over_plain_fp64": round(mixed["solves_per_s"] / results["plain_fp64"]["solves_per_s"], 3),
        "e2e": e2e, "error_sample": errs,
        "autotune_ms": {f"{k[0]}x{k[1]}": round(v * 1e3, 2) for k, v in tune.items()},
        "gpu_launches": 2 * steps, "clocks": clock_info,
    }


def batched_config(args) -> dict:
    world = int(os.environ.get("WORLD_SIZE", "1"))
    return {"workload": BATCH_WORKLOAD, "description": BATCH_DESC, "systems": args.batch_systems,
            "solver": "CG", "prec": "diag", "stop": "||b-Ax|| < 1e-8 ||b|| per system, x0 = 0",
            "niter_limit": args.niter, "l2": "inputs larger than L2", "parallelism": f"replicas x{world}"}


def run_batched(args, dist: Dist) -> dict | None:
    leg = batched_leg(args, dist, args.batch_systems, args.steps, args.warmup)
    mixed = leg["batched_mixed"]
    line = {
        "metric": METRIC, "value": round(mixed["solves_per_s"], 3), "unit": UNIT,
        "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(mixed["ms_per_batch"], 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner / f64 outer",
        "data": "synthetic (seeded jittered-hex meshes, random cell numbering, RHS U[-1,1])",
        "config": batched_config(args), "roofline": mixed["roofline"], "e2e": leg["e2e"],
        "gpu_launches": leg.pop("gpu_launches"), "clocks": leg.pop("clocks"), "batched": leg,
    }
    if dist.rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = batched_cpu_baseline(batch_specs(args.batch_systems, BASE_SEED), args)
    return line if dist.rank == 0 else None


def _batched_cpu_one(spec):
    sys.path[:0] = [str(REPO), str(REPO / "t-flows_gb300")]
    import numpy as np
    import tflows
    from oracle import tfs_oracle as O
    nx, ny, nz, jit, sd = spec
    s = tflows.SynthSystem(0, nx, ny, nz, jitter=jit, seed=sd)
    x, r = np.zeros(s.n), s.b.copy()
    tol = REL_TOL * float(np.linalg.norm(s.b))
    t = time.perf_counter()
    it, _, _ = O.solve(0, s.n, s.row, s.col, s.dia, s.val, x, r, 1, 5000, tol)
    return time.perf_counter() - t, s.n, it


def batched_cpu_baseline(specs, args) -> dict:
    """The oracle on all host cores, one system per core, on a sample of the
    batch; scaled to all systems by their share of n^(4/3) (work ~ n x iterations)."""
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    sample = specs[:cores]
    ctx = mp.get_context("spawn")
    t = time.perf_counter()
    with ctx.Pool(cores) as pool:
        out = pool.map(_batched_cpu_one, sample)
    wall = time.perf_counter() - t
    w = lambda spec: (spec[0] * spec[1] * spec[2]) ** (4.0 / 3.0)
    scale = sum(w(sp) for sp in specs) / sum(w(sp) for sp in sample)
    est = wall * scale
    return {"value": round(len(specs) / est, 4), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"the first {len(sample)} systems of the batch, one single-threaded binary64 "
                      f"diagonal-CG solve per core ({wall:.1f} s wall), scaled to the {len(specs)} "
                      f"systems by sum(n^(4/3))"}


# ---------------------------------------------------------------- reference arm

_REF = {}


def _ref_init(kind, nside, seed):
    # The reference arm builds its inputs with the host-only generator
    # (libtfs_synth.so) and solves them with the oracle: the GPU solver
    # library is never loaded in these processes.
    sys.path[:0] = [str(REPO), str(REPO / "t-flows_gb300")]
    from tflows.synth import SynthSystem
    _REF["s"] = SynthSystem(kind, nside, jitter=0.2, seed=seed)


def _ref_solve(arg):
    """One single-threaded binary64 solve of the workload's system by the
    oracle, stopped after `iters` iterations (or at the tolerance)."""
    import numpy as np
    from oracle import tfs_oracle as O
    method, prec, iters, tol = arg
    s = _REF["s"]
    x, r = np.zeros(s.n), s.b.copy()
    t = time.perf_counter()
    it, _, _ = O.solve(method, s.n, s.row, s.col, s.dia, s.val, x, r, prec, iters, tol)
    return time.perf_counter() - t, it


def run_reference_other(args) -> dict:
    """Reference arm of the batched and serving workloads: the oracle on all
    host cores, one single-threaded binary64 solve per core, every step a
    sample of `cores` systems (batch) or requests (trace) of the workload."""
    import multiprocessing as mp
    from tflows.synth import serving_pool_specs, uniform
    cores = os.cpu_count() or 1
    if args.workload == BATCH_WORKLOAD:
        specs = batch_specs(args.batch_systems, BASE_SEED)
        jobs_all = [(0, *sp[:3], sp[3], sp[4], 0, 1, args.niter, REL_TOL) for sp in specs]
        config = batched_config(args)
        what = "systems of the batch"
    else:
        seed = BASE_SEED + 7
        pool = serving_pool_specs(args.serve_pool, seed)
        jobs_all = []
        for j in range(args.serve_requests):
            k = min(args.serve_pool - 1, int(uniform(seed, 42, j) * args.serve_pool))
            tol_rel = 1e-6 if uniform(seed, 43, j) < 0.5 else 1e-8
            kind, nx, ny, nz, sd = pool[k]
            method, niter = (0, 2000) if kind == 0 else (1, 10)
            jobs_all.append((kind, nx, ny, nz, 0.2, sd, method, 1, niter, tol_rel))
        config = serving_config(args)
        what = "requests of the trace"
    step_s, done = [], 0
    with mp.get_context("spawn").Pool(cores) as p:
        for i in range(args.warmup + args.steps):
            jobs = [jobs_all[(i * cores + c) % len(jobs_all)] for c in range(cores)]
            t = time.perf_counter()
            p.map(_oracle_one, jobs)
            if i >= args.warmup:
                step_s.append(time.perf_counter() - t)
                done += cores
    value = done / sum(step_s)
    cpu = {"value": round(value, 4), "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"each step: {cores} {what}, one whole single-threaded binary64 solve per core "
                     f"(consecutive {what} step after step)"}
    return {
        "impl": "reference", "metric": METRIC, "value": cpu["value"], "unit": UNIT, "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(statistics.mean(step_s) * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (same seeded systems as our arm)", "config": config, "cpu_baseline": cpu,
        "e2e": {"value": cpu["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_reference(args) -> dict:
    """The reference's CPU solver (the oracle restatement of Cg/Bicg/Cgs) on
    all host cores: one independent single-threaded binary64 solve per core,
    the reference's sequential build being one process per system.

    A step is a bounded sample of that work.  When one full solve takes at
    most WHOLE_SOLVE_S seconds, every core runs one whole solve per step.
    Otherwise every core runs the solve from x0 = 0 and stops after k
    iterations (k sized for about SAMPLE_S seconds); the step then counts
    (P + k I) / (P + n_it I) solves per core, where n_it is the iteration
    count of a full solve and P (preconditioner form and initial residual)
    and I (one iteration) are measured on the same system outside the timed
    steps.  ms_per_step is the measured wall time of a step, so the timed
    region is exactly the steps run."""
    import multiprocessing as mp

    import numpy as np
    if args.workload not in WORKLOADS:
        return run_reference_other(args)
    WHOLE_SOLVE_S, SAMPLE_S = 5.0, 3.0
    kind, nside, method, prec, desc = WORKLOADS[args.workload]
    cores = os.cpu_count() or 1
    _ref_init(kind, nside, BASE_SEED)
    s = _REF["s"]
    tol = REL_TOL * float(np.linalg.norm(s.b))
    # Outside the timed steps: the prologue alone (niter = 0), a probe, and
    # the full solve (iteration count and time), stopped after FULL_S
    # seconds' worth of iterations: a solve that has not converged by then
    # is counted as running to the iteration limit.
    FULL_S = 150.0
    _ref_solve((method, prec, 0, tol))          # loads the oracle library
    p_s, _ = _ref_solve((method, prec, 0, tol))
    probe = 8
    t_probe, _ = _ref_solve((method, prec, probe, tol))
    it_s = max(1e-9, (t_probe - p_s) / probe)
    budget = max(probe, min(args.niter, int((FULL_S - p_s) / it_s)))
    run_s, run_it = _ref_solve((method, prec, budget, tol))
    if run_it <= budget or budget == args.niter:
        full_s, full_it, full_known = run_s, run_it, True
    else:
        full_it, full_known = args.niter + 1, False
        full_s = p_s + (run_s - p_s) / budget * full_it
    it_s = max(1e-9, (run_s - p_s) / max(1, min(run_it, budget)))
    if full_s <= WHOLE_SOLVE_S:
        k, frac = args.niter, 1.0
    else:
        k = max(1, min(full_it, int(round((SAMPLE_S - p_s) / it_s))))
        frac = (p_s + k * it_s) / (p_s + full_it * it_s)
    log(f"[bench-ref] full solve {full_it} it in {full_s:.2f}s (prologue {p_s:.3f}s); "
        f"step = {k if frac < 1 else 'all'} iterations x {cores} cores = {cores * frac:.4f} solves")
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores, initializer=_ref_init, initargs=(kind, nside, BASE_SEED)) as pool:
        for _ in range(args.warmup):
            pool.map(_ref_solve, [(method, prec, k, tol)] * cores)
        step_s = []
        for _ in range(args.steps):
            t = time.perf_counter()
            pool.map(_ref_solve, [(method, prec, k, tol)] * cores)
            step_s.append(time.perf_counter() - t)
    total_s = sum(step_s)
    value = cores * frac * args.steps / total_s
    if frac >= 1.0:
        sample = (f"each step: {cores} whole single-threaded binary64 solves, one per core "
                  f"({full_it} iterations each)")
    else:
        sample = (f"each step: {cores} single-threaded binary64 solves from x0 = 0, one per core, each "
                  f"stopped after {k} of the {full_it} iterations of a full solve"
                  f"{'' if full_known else f' (the iteration limit + 1: not converged after {budget} iterations)'}, "
                  f"counted as {frac:.5f} of a solve each (prologue {p_s:.3f} s and {it_s * 1e3:.2f} ms "
                  f"per iteration, measured outside the steps; a full solve took {full_s:.1f} s)")
    return {
        "impl": "reference", "metric": METRIC, "value": round(value, 6), "unit": UNIT,
        "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(total_s / args.steps * 1e3, 2), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (same seeded system as our arm)",
        "config": workload_config(args, s.n, s.nnz),
        "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
        "reference_solve": {"iterations": full_it, "seconds_one_core": round(full_s, 3),
                            "full_solve_run": full_known},
        "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


# ---------------------------------------------------------------- main

DEFAULT_WORKLOAD = "poisson128_dic_cg"


def legs(args, dist: Dist, line: dict | None) -> None:
    """The batched and served paths of the metric, bounded so the default run
    stays within a few minutes: the first --leg-batch-systems systems of the
    256-system specification and a --leg-serve-requests request prefix of the
    trace over a --leg-serve-pool system pool.  Added to the line as extra
    keys; the headline value stays the single-system solve."""
    b = batched_leg(args, dist, args.leg_batch_systems, min(args.steps, 10), 3)
    sv = serving_leg(args, dist, args.leg_serve_pool, args.leg_serve_requests)
    if line is None:
        return
    b["bounded"] = (f"the first {args.leg_batch_systems} of the 256 systems of {BATCH_WORKLOAD} "
                    f"(--workload {BATCH_WORKLOAD} runs all)")
    sv["bounded"] = (f"{args.leg_serve_requests} requests over a {args.leg_serve_pool}-system pool "
                     f"(--workload {SERVE_WORKLOAD} runs {args.serve_requests} over {args.serve_pool})")
    line["batched"] = b
    line["serving"] = sv
    line["target_mixed_over_fp64"] = {
        "target": "mixed, batched, served path >= 1.7x the plain binary64 GPU path's solves/s",
        "batched_mixed_over_plain_fp64": b["mixed_batched_over_plain_fp64"],
        "served_mixed_over_fp64": sv["mixed_over_fp64"],
        "served_mixed_over_fp64_e2e": sv["mixed_over_fp64_e2e"],
        "single_mixed_over_fp64": line.get("mixed_over_fp64"),
    }



def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + [BATCH_WORKLOAD, SERVE_WORKLOAD],
                    default=DEFAULT_WORKLOAD)
    ap.add_argument("--serve-pool", type=int, default=32)
    ap.add_argument("--serve-requests", type=int, default=1200)
    ap.add_argument("--serve-rate", type=float, default=400.0)
    ap.add_argument("--serve-slots", type=int, default=8)
    ap.add_argument("--serve-inflight", type=int, default=16)
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--batch-systems", type=int, default=256)
    ap.add_argument("--leg-batch-systems", type=int, default=64,
                    help="systems of the batched leg of the default run")
    ap.add_argument("--leg-serve-pool", type=int, default=16,
                    help="resident systems of the serving leg of the default run")
    ap.add_argument("--leg-serve-requests", type=int, default=400,
                    help="requests of the serving leg of the default run")
    ap.add_argument("--no-legs", action="store_true",
                    help="default run without the batched and serving legs")
    ap.add_argument("--niter", type=int, default=5000)
    ap.add_argument("--spmv-reps", type=int, default=50)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default launch shapes of the single-solve kernels")
    ap.add_argument("--no-next-rows", action="store_true",
                    help="skip the device topology / assembly measurements")
    ap.add_argument("--modes", default="fp64,mixed",
                    help="arithmetic legs to run (profiling runs may pick one)")
    ap.add_argument("--option", action="append", default=[], metavar="NAME=VALUE",
                    help="a TFS_OPT_* option of the single-system solver, e.g. PDL=0 (repeatable)")
    ap.add_argument("--eager", action="store_true",
                    help="launch the solve kernels from a host loop instead of a CUDA graph "
                         "(TFS_OPT_LAUNCH = 1), for kernel-level profiling")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        log("[bench] warm-up raised to 3 steps")
        args.warmup = 3
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return 0
        print(json.dumps(run_reference(args)), flush=True)
        return 0
    import __graft_entry__
    __graft_entry__.build()
    dist = Dist()
    try:
        if args.workload == BATCH_WORKLOAD:
            line = run_batched(args, dist)
        elif args.workload == SERVE_WORKLOAD:
            line = run_serving(args, dist)
        else:
            line = run_ours(args, dist)
            if args.workload == DEFAULT_WORKLOAD and not args.no_legs:
                legs(args, dist, line)
    finally:
        dist.close()
    if line is not None:
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
