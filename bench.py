#!/usr/bin/env python
"""Benchmark of the HeatFlow time-stepping hot path on GB300.

Metric: time-steps/s (and cell-iterations/s) at 256^3 with the mixed FP32-CG + FP64-refinement
path at a true relative residual ||S - H T||/||S|| <= 1e-10 per step, beside the plain FP64 GPU
path at the same residual.  Workload: two-material layered slab (z-layers alternating every 16
cells between silicon-like kappa 149 and polymer-like kappa 0.2), Cattaneo mode, Dirichlet 300 K
on all faces, Gaussian heating over the top face, dx = 1 nm, dt = 1e-13 s; synthetic, seeded.

One "step" is one implicit time step (RHS, initial guess, solve, state rotation) of the whole grid.
`value` is timed with CUDA events on the library's stream with the state resident in HBM;
`e2e` is the same metric through the C ABI with host buffers: every step uploads T^n, T^(n-1)
from pinned host memory and downloads the new T^n into pinned host memory, queued through
hf_step_host_async (T^(n-1)'s upload overlaps the previous step's solve, T^n moves in chunks
behind the previous step's download, and each chunk's RHS runs as it lands) and ended by
hf_host_sync; `e2e.sync_value` times the same steps through hf_set_state, hf_step, hf_get_state.

    python bench.py [--gpus N --steps K --warmup W] [--impl reference]

With N > 1 (torchrun, one process per GPU) every rank advances its own replica of the grid
(replicas only: the path has no data-path collective) and `value` sums the ranks.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "time-steps/s at 256^3, mixed FP32-CG + FP64 refinement, rel-res 1e-10"
UNIT = "time-steps/s"

# Algorithmic bytes per cell of each kernel (what the kernel must read + write from HBM),
# for the layered-slab workload (Cattaneo, per-cell heater power array present).
BYTES_PER_CELL = {
    # every cell: T^n, T^(n-1), the T^n coefficient of S, tau'*rho*c read, S and x0 written (8 B
    # each); B, heater case and power only where they exist (rhs_bytes)
    "rhs": 6 * 8,
    # mixed: x, diag, cx, cy, cz, S (8 B) + 1/sqrt|H_II| (4 B) read; g (4 B) + H x (8 B) written
    "residual_mixed": 6 * 8 + 4 + 4 + 8,
    # mixed step start from the stored products: S, H T^n, H T^(n-1) (8 B) + 1/sqrt|H_II| (4 B)
    # read; g (4 B) written (no +TINY under the true-residual criterion, so no H*1)
    "residual_init_hx_mixed": 3 * 8 + 4 + 4,
    # FP64: x, diag, cx, cy, cz, S, 1/sqrt|H_II| (8 B) read; g, H x (8 B) written
    "residual_fp64": 7 * 8 + 8 + 8,
    # direction update: r, p_old read, p written; SpMV: p, ax, ay, az read, q written
    "cg_p_fp32": 3 * 4, "cg_spmv_fp32": 5 * 4, "cg_update_fp32": 6 * 4,
    # fused direction update + SpMV: r, p_old, ax, ay, az read, p, q written
    "cg_pq_fp32": 7 * 4,
    # x read (8) + y (4) + sinv (4) read, x written (8)
    "xupdate_mixed": 8 + 4 + 4 + 8,
    # x, y, sinv read and x written (8 B each)
    "xupdate_fp64": 4 * 8,
    "cg_p_fp64": 3 * 8, "cg_spmv_fp64": 5 * 8, "cg_update_fp64": 6 * 8,
}
# FP64 floating-point operations per cell (an FMA counts 2) of the FP64-pipe kernels: the mixed
# residual does 7 FMA for S - Hx and 1 sub for H x = S - r (||r||^2 in FP32), the FP64 one also
# 1 FMA for ||r||^2 and a multiply and an FMA for g and ||g||^2; the mixed step-start residual
# from the stored products 1 FMA + 1 add (S - 2 H T^n + H T^(n-1), ||r||^2 in FP32); the RHS
# under the true-residual criterion 1 mul + 1 FMA (S = T^n c1 + ccat T^(n-1)) and 1 FMA
# (x0 = 2 T^n - T^(n-1)) per interior cell - its ||S||^2 runs on the integer/FP32 pipes.
FP64_FLOPS_PER_CELL = {"residual_mixed": 15, "residual_fp64": 20, "residual_init_hx_mixed": 3,
                       "rhs": 5}

# Algorithmic bytes per cell of each round of the persistent solve kernel (k_solve), by phase:
# (bytes, bytes of the first inner iteration / of an update without a correction).  Under the
# true-residual criterion the reference's +TINY on x0 is not applied (it moves only the starting
# point), so the first residual does not read H*1.  A CG update that also forms x ("cg_bx", the
# iteration predicted to end the inner solve) counts the CG update's bytes plus, if its x is the
# one the next residual sweep reads, the x update's (x, S^-1 in, x out: XB); when the solve went
# on after it, the x it formed was not used and is not counted.
PHASE_BYTES = {
    "mixed": {"res_init": (56, 56), "res_init_hx": (32, 32), "res": (64, 64), "cg_p": (12, 12),
              "cg_q": (20, 20), "cg_pq": (28, 24), "cg_b": (24, 20), "cg_bx": (24, 20),
              "xupd": (24, 16)},
    "fp64": {"res_init": (64, 64), "res_init_hx": (40, 40), "res": (72, 72), "cg_p": (24, 24),
             "cg_q": (40, 40), "cg_b": (48, 40), "cg_bx": (48, 40), "xupd": (32, 16)},
}
XB = {"mixed": 8 + 4 + 8, "fp64": 3 * 8}


def rhs_bytes(prob):
    """Algorithmic bytes of one RHS launch: 48 B per cell (BYTES_PER_CELL["rhs"]), the boundary
    vector B at the cells on non-periodic outer faces (boundary() leaves every other cell at 0),
    and the heater case (1 B) and power (8 B) of the heated cells."""
    import numpy as np
    dims = (prob.nx, prob.ny, prob.nz)
    per = tuple(getattr(prob, "periodic", (0, 0, 0)) or (0, 0, 0))
    inner = 1
    for n, p in zip(dims, per):
        inner *= n if p else max(n - 2, 0)
    N = prob.nx * prob.ny * prob.nz
    heated = int(np.count_nonzero(np.asarray(prob.iheater) > 0)) if prob.iheater is not None else 0
    return BYTES_PER_CELL["rhs"] * N + 8 * (N - inner) + 9 * heated


def round_bytes_per_cell(rounds, precision):
    """Algorithmic bytes per cell of each round of one persistent-solve launch (its round log)."""
    table = PHASE_BYTES[precision]
    out, first_cg, first_b, have_y, bx = [], True, True, False, None
    for ph, _ in rounds:
        full, alt = table.get(ph, (0, 0))
        b = 0
        if ph in ("res_init", "res_init_hx", "res"):
            if ph == "res" and bx is not None:      # this sweep reads the x that update formed
                out[bx] += XB[precision]
            b = full
            first_cg = first_b = True
            have_y = False
            bx = None
        elif ph == "cg_p":                        # iteration 0 has no direction round (p_0 = r)
            b = full
            first_cg = False
        elif ph == "cg_pq":
            b = alt if first_cg else full
            first_cg = False
        elif ph == "cg_q":
            b = full
        elif ph in ("cg_b", "cg_bx"):
            b = alt if first_b else full
            first_b = False
            have_y = True
            bx = len(out) if ph == "cg_bx" else None
        elif ph == "xupd":
            b = full if have_y else alt
            bx = None
        out.append(b)
    return out


def solve_bytes_per_cell(rounds, precision):
    """Algorithmic bytes per cell of one persistent-solve launch from its round phases."""
    return sum(round_bytes_per_cell(rounds, precision))


# FP64 instructions per cell of each round (the rest of the work is FP32/integer): the mixed
# path's residual sweep 7 FMA + 1 sub, its pointwise first residual 1 FMA + 1 add, the stencil
# first residual 7 FMA (||r||^2 in FP32 in all three), the x update 1 add (also when a CG update
# forms x).
PHASE_FP64_INSTR = {
    "mixed": {"res_init_hx": 2, "res_init": 7, "res": 8, "xupd": 1, "cg_bx": 1},
    "fp64": {"res_init_hx": 5, "res_init": 10, "res": 11, "xupd": 1, "cg_p": 1, "cg_q": 7,
             "cg_b": 3, "cg_bx": 4},
}


def solve_floor(rounds, precision, N, hbm_gbs, fp64_tflops):
    """Each round's floor is the larger of its algorithmic bytes at the measured HBM rate and its
    FP64 instructions at the measured FP64 issue rate (an FMA's 2 flops per instruction); the
    launch's floor is their sum, compared with the rounds' measured times (round log)."""
    instr_rate = fp64_tflops * 1e12 / 2.0
    table = PHASE_FP64_INSTR[precision]
    by = {}
    floor = actual = 0.0
    for (ph, us), b in zip(rounds, round_bytes_per_cell(rounds, precision)):
        t_mem = b * N / (hbm_gbs * 1e9) * 1e6
        t_fp64 = table.get(ph, 0) * N / instr_rate * 1e6
        f = max(t_mem, t_fp64)
        floor += f
        actual += us
        e = by.setdefault(ph, {"floor_us": 0.0, "us": 0.0, "bound": "fp64" if t_fp64 > t_mem else "hbm"})
        e["floor_us"] += f
        e["us"] += us
    for e in by.values():
        e["frac"] = e["floor_us"] / e["us"] if e["us"] else None
    return {"floor_us": floor, "us": actual, "frac": floor / actual if actual else None,
            "by_phase": by,
            "note": "per round max(algorithmic bytes / measured HBM, FP64 instructions / measured "
                    "FP64 rate), summed over the launch's rounds"}


def phase_table(rounds, precision, N):
    """Per phase of one persistent-solve launch: rounds, microseconds, upper GB/s (full bytes)."""
    out = {}
    for ph, us in rounds:
        e = out.setdefault(ph, {"rounds": 0, "us": 0.0})
        e["rounds"] += 1
        e["us"] += us
    for ph, e in out.items():
        full, _ = PHASE_BYTES[precision].get(ph, (0, 0))
        if ph == "cg_bx":
            full += XB[precision]
        e["us_per_round"] = e["us"] / e["rounds"]
        e["GB/s_upper"] = full * N / (e["us_per_round"] * 1e-6) / 1e9 if full else None
    return out


def kernel_table(kms, N, peak, fp_rates, total_bytes=None):
    """Standalone kernel times -> GB/s, fraction of HBM and, for the FP64-pipe kernels, TFLOP/s.
    total_bytes: {kernel: algorithmic bytes per launch} where it is not BYTES_PER_CELL x N."""
    out = {}
    for k, v in kms.items():
        b = (total_bytes or {}).get(k, BYTES_PER_CELL[k] * N)
        gbs = b / (v / 1000.0) / 1e9
        e = {"ms": v, "GB/s": gbs, "frac": gbs / peak}
        if fp_rates and k in FP64_FLOPS_PER_CELL:
            tf = FP64_FLOPS_PER_CELL[k] * N / (v / 1000.0) / 1e12
            e["fp64_tflops"] = tf
            e["fp64_frac"] = tf / fp_rates["fp64_tflops"]
        out[k] = e
    return out


def compact(obj, digits=5):
    """Floats rounded to `digits` significant digits (the line stays short enough to be kept whole)."""
    if isinstance(obj, float):
        if obj != obj or obj in (float("inf"), float("-inf")) or obj == 0.0:
            return obj
        return float(f"{obj:.{digits}g}")
    if isinstance(obj, dict):
        return {k: compact(v, digits) for k, v in obj.items()}
    if isinstance(obj, (list, tuple)):
        return [compact(v, digits) for v in obj]
    return obj


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--fourier", action="store_true", help="Fourier instead of Cattaneo")
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--workload", choices=["layered", "batched", "inclusions"], default="layered",
                    help="layered: the headline 256^3 slab; batched: 256 uneven grids (edges "
                         "16..96, 200-step sweep); inclusions: 512^3 with polymer spheres")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default task depth and inner tolerance")
    ap.add_argument("--per-step-graph", action="store_true",
                    help="one graph launch per step instead of one for the whole loop (profilers "
                         "see the kernels)")
    ap.add_argument("--host-loop", action="store_true",
                    help="drive the solve loop from the host instead of the captured graph")
    ap.add_argument("--detail", default=None,
                    help="also write per-phase and standalone-kernel timings to this JSON file")
    ap.add_argument("--cpu-seconds", type=float, default=90.0,
                    help="wall-clock bound of the reference arm's timed steps")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_max(v, dist=None, device="cuda"):
    """Max of a per-rank timing over all ranks (identity without a process group)."""
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(world, steps, ms_max):
    """Whole-job rate of `world` independent replicas, each advancing `steps` steps, timed by the
    slowest rank (weak scaling: the per-rank work is fixed)."""
    return world * steps / (ms_max / 1000.0)


def measured_peak():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_traffic():
    """Per-cell DRAM bytes of each kernel from the committed ncu summary, if present."""
    path = os.path.join(HERE, "profiles", "dram_bytes_per_cell.txt")
    out = {}
    if os.path.exists(path):
        for line in open(path):
            parts = line.split()
            if len(parts) == 2 and not line.startswith("#"):
                try:
                    out[parts[0]] = float(parts[1])
                except ValueError:
                    pass
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.gpu)], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sms)) if sms else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sms)}


def cpu_baseline(prob, steps_cap: int, seconds: float, tol: float, warm: int = 0):
    """The oracle port of the reference's step (COO H, Jacobi BiCG with the reference's itol=1
    criterion at `tol`, OpenMP-atomic SpMV as in the reference's Parallel build) on all host
    cores.  Runs `warm` untimed steps, then times whole steps until `steps_cap` steps or `seconds`
    elapse."""
    from oracle.oracle import Oracle, set_threads
    cores = os.cpu_count() or 1
    set_threads(cores)
    o = Oracle(prob)
    o.set_state(*prob.initial_state())
    for k in range(warm):
        o.simulate(k + 1, mode=0, tol=tol, itmax=50000)
    times, iters = [], []
    t_all = time.perf_counter()
    k = warm
    while k < warm + steps_cap:
        t0 = time.perf_counter()
        rc, it, _ = o.simulate(k + 1, mode=0, tol=tol, itmax=50000)
        times.append(time.perf_counter() - t0)
        iters.append(it)
        k += 1
        if rc != 0 or time.perf_counter() - t_all > seconds:
            break
    ms = 1000.0 * float(np.mean(times))
    return {"value": 1000.0 / ms, "unit": UNIT, "cores": cores, "kind": "port",
            "ms_per_step": ms, "steps_timed": len(times), "bicg_iters_per_step": iters,
            "sample": f"{len(times)} full step(s) of the same {prob.nx}^3 workload: COO H, "
                      f"Jacobi BiCG at itol=1 tol={tol:g}, OpenMP atomic SpMV, {cores} threads"}


def cpu_clean_pcg(prob, steps_cap: int, seconds: float, tol: float):
    """A clean CPU solver on all host cores (oracle/cpu_pcg.c: stencil Jacobi-PCG in FP64 to the
    same true relative residual, OpenMP, no atomics): the fairer CPU comparison beside the faithful
    restatement.  One untimed step, then whole steps until `steps_cap` or `seconds`."""
    from oracle.oracle import CleanPCG, Oracle
    cores = os.cpu_count() or 1
    o = Oracle(prob)
    o.set_state(*prob.initial_state())
    cp = CleanPCG(o, threads=cores)
    rc, _, _ = cp.step(1, tol=tol)
    times, iters = [], []
    t_all = time.perf_counter()
    k = 1
    while rc == 0 and k < steps_cap + 1:
        t0 = time.perf_counter()
        rc, it, rel = cp.step(k + 1, tol=tol)
        times.append(time.perf_counter() - t0)
        iters.append(it)
        k += 1
        if time.perf_counter() - t_all > seconds:
            break
    ms = 1000.0 * float(np.mean(times)) if times else float("nan")
    return {"value": 1000.0 / ms, "unit": UNIT, "cores": cores, "kind": "clean CPU solver",
            "ms_per_step": ms, "steps_timed": len(times), "cg_iters_per_step": iters,
            "sample": f"{len(times)} step(s) of the {prob.nx}^3 workload after one untimed: "
                      f"stencil Jacobi-PCG, FP64, true rel-res {tol:g}, {cores} threads "
                      f"(oracle/cpu_pcg.c, not the reference's algorithm)"}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    from heatflow_gb300.problem import layered_slab
    prob = layered_slab(args.n, icattaneo=0 if args.fourier else 1)
    warm = max(args.warmup, 0)
    cb = cpu_baseline(prob, max(args.steps, 1), args.cpu_seconds, args.tol, warm=warm)
    line = {
        "metric": METRIC, "value": cb["value"], "unit": UNIT, "impl": "reference",
        "n_gpus": world, "steps": cb["steps_timed"], "warmup": warm,
        "ms_per_step": cb["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(args, prob),
        "cpu_baseline": {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "notes": "reference Fortran not buildable on either machine (no Fortran compiler); "
                 "the oracle port restates it statement by statement",
    }
    print(json.dumps(compact(line), separators=(",", ":")), flush=True)
    return 0


def workload_config(args, prob):
    return {
        "workload": f"layered slab {prob.nx}x{prob.ny}x{prob.nz}, "
                    f"{'Fourier' if args.fourier else 'Cattaneo'}, top-face Gaussian heating",
        "cells": prob.ncells, "dx_m": 1e-9, "dt_s": 1e-13, "rel_res": args.tol,
        "layers": "z-alternating every 16 cells, kappa 149 / 0.2",
        "l2": f"inputs larger than L2: ~{prob.ncells * 230 / 1e9:.1f} GB resident per grid "
              f"(L2 129 MB), no flush needed",
        "parallelism": f"replicas x{args.gpus}",
        "step_loop": "host-polled kernels" if args.host_loop else
                     ("one CUDA graph launch per step" if args.per_step_graph else
                      "the whole loop as one CUDA graph (WHILE node)") +
                     ": RHS + one persistent cooperative solve kernel per step",
    }


def timed_run(hf, torch, stream, itime0, steps):
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed")
    e0.record(stream)
    st = hf.run(itime0, steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.nvtx.range_pop()
    return e0.elapsed_time(e1), st


def other_workload(args):
    """Time-steps/s of the batched sweep or the 512^3 inclusion grid, mixed and FP64 (one JSON
    line; the headline contract line is the layered slab's)."""
    import torch
    from heatflow_gb300.build import build_library
    from heatflow_gb300.problem import batched_sweep, inclusions
    from heatflow_gb300.solver import HeatFlow
    build_library()
    if args.workload == "batched":
        probs = batched_sweep(256, seed=0)
        name = "batched sweep: 256 grids, edges U{16..96}, lognormal kappa, 1-4 sources, Cattaneo"
    else:
        probs = [inclusions(512)]
        name = "512^3 inclusion grid (5 % polymer spheres), periodic x/y, Cattaneo"
    cells = sum(p.ncells for p in probs)
    stream = torch.cuda.Stream()
    W, K = max(args.warmup, 0), max(args.steps, 1)
    out = {"workload": name, "grids": len(probs), "cells": cells, "steps": K, "warmup": W,
           "data": "synthetic", "unit": "time-steps/s (every grid advances one step)"}
    for prec, tol in (("mixed", args.tol), ("fp64", args.tol)):
        hf = HeatFlow(probs, precision=prec, criterion="true", tol=tol, use_graph=1)
        hf.set_stream(stream.cuda_stream)
        hf.initial_evolve()
        if W:
            hf.run(1, W)
        tuned = None
        if not args.no_autotune:
            best = next(r for r in hf.autotune(itime0=W + 1, steps=4) if r["chosen"])
            tuned = {"task_depth": best["task_depth"], "inner_tol": best["inner_tol"]}
        ms, st = timed_run(hf, torch, stream, W + 1, K)
        out[prec] = {"steps_per_s": K / (ms / 1000.0), "ms_per_step": ms / K,
                     "cell_steps_per_s": cells * K / (ms / 1000.0),
                     "iterations_per_step": (st["iterations"] + st["inner_iterations"]) / K,
                     "unconverged": st["unconverged"], "last_true_relres": st["last_true_relres"],
                     "kernel_launches_per_step": st["kernel_launches"] / K, "autotuned": tuned}
        hf.close()
    out["mixed_over_fp64"] = out["mixed"]["steps_per_s"] / out["fp64"]["steps_per_s"]
    print(json.dumps(out), flush=True)
    return 0


def main():
    args = parse()
    rank, world, local = dist_info()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    if args.workload != "layered":
        return other_workload(args)

    import torch
    from heatflow_gb300 import abi
    from heatflow_gb300.build import build_library
    from heatflow_gb300.problem import layered_slab
    from heatflow_gb300.solver import HeatFlow

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    build_library()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(v):
        return reduce_max(v, dist, "cuda")

    prob = layered_slab(args.n, icattaneo=0 if args.fourier else 1)
    N = prob.ncells
    graph = 0 if args.host_loop else (3 if args.per_step_graph else 1)
    stream = torch.cuda.Stream()
    W, K = max(args.warmup, 0), max(args.steps, 1)

    # ---- headline: mixed path, state resident in HBM
    hf = HeatFlow(prob, precision="mixed", criterion="true", tol=args.tol, use_graph=graph)
    hf.set_stream(stream.cuda_stream)
    hf.initial_evolve()
    if W:
        hf.run(1, W)
    tuned = {}
    if not args.no_autotune:        # task depth and inner tolerance, timed on this problem
        t0 = time.perf_counter()
        cand = hf.autotune(itime0=W + 1, steps=6)
        best = next(r for r in cand if r["chosen"])
        tuned["mixed"] = {"task_depth": best["task_depth"], "inner_tol": best["inner_tol"],
                          "candidates": len(cand), "seconds": time.perf_counter() - t0}
    barrier()
    with ClockSampler(torch.cuda.current_device()) as clk:
        ms, st = timed_run(hf, torch, stream, W + 1, K)
    ms = max_over_ranks(ms)
    clocks = clk.summary()
    steps_per_s = aggregate_rate(world, K, ms)
    cell_iters = N * (st["inner_iterations"] + st["iterations"] + st["refinements"])
    cell_iters_per_s = world * cell_iters / (ms / 1000.0)

    # ---- kernel roofline.  The dominant kernel is the persistent solve (k_solve: the whole
    # refinement loop of a step in one cooperative launch); it is timed alone with CUDA events on
    # the library's stream.  Its algorithmic bytes come from the phase of every grid-wide round of
    # the timed launches (the kernel's own round log).
    peak, peak_kind = measured_peak()
    prec = "mixed"
    solve_ms = hf.time_kernel(abi.HF_KERNEL_SOLVE, reps=10)
    rounds, nrounds = hf.solve_profile()
    solve_bpc = solve_bytes_per_cell(rounds, prec)
    f64 = C.c_double()
    f32 = C.c_double()
    rc = abi.load_library().hf_measure_fp_rates(C.byref(f64), C.byref(f32))
    fp_rates = {"fp64_tflops": f64.value, "fp32_tflops": f32.value} if rc == 0 else None
    achieved = solve_bpc * N / (solve_ms / 1000.0) / 1e9
    ratio = ncu_traffic().get("solve_mixed_ratio")     # DRAM bytes per algorithmic byte (ncu)
    roofline = {"kernel": "k_solve<float> (persistent cooperative solve, one launch per step)",
                "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": f"of {peak_kind}",
                "traffic": ratio * solve_bpc * N if ratio else None,
                "traffic_source": "ncu DRAM read+write per algorithmic byte (profiles/solve_kernel_"
                                  "layered_slab_256cube_dram.md) x this launch's algorithmic bytes",
                "algorithmic_bytes_per_launch": solve_bpc * N, "ms_per_launch": solve_ms,
                "rounds_per_launch": nrounds, "share_of_step": solve_ms / (ms / K)}
    rhs_ms = hf.time_kernel(abi.HF_KERNEL_RHS, reps=10)
    rhs_gbs = rhs_bytes(prob) / (rhs_ms / 1000.0) / 1e9
    roofline["k_rhs"] = {"ms": rhs_ms, "GB/s": rhs_gbs, "frac": rhs_gbs / peak,
                         "share_of_step": rhs_ms / (ms / K)}
    detail = {"phases": phase_table(rounds, prec, N)}
    if fp_rates:
        comb = solve_floor(rounds, prec, N, peak, fp_rates["fp64_tflops"])
        roofline["combined"] = {"floor_us": comb["floor_us"], "us": comb["us"], "frac": comb["frac"],
                                "by_phase": {ph: [e["us"], e["frac"], e["bound"]]
                                             for ph, e in comb["by_phase"].items()},
                                "note": "per round max(bytes / measured HBM, FP64 instructions / "
                                        "measured FP64 rate); by_phase: [us, frac, bound]"}
    if args.detail:
        # standalone kernels (timed repeatedly on the same data, partly L2-resident)
        kernels = {"cg_p_fp32": abi.HF_KERNEL_CG_P, "cg_spmv_fp32": abi.HF_KERNEL_CG_SPMV,
                   "cg_pq_fp32": abi.HF_KERNEL_CG_PQ, "cg_update_fp32": abi.HF_KERNEL_CG_UPDATE,
                   "xupdate_mixed": abi.HF_KERNEL_XUPDATE,
                   "residual_init_hx_mixed": abi.HF_KERNEL_RESIDUAL_INIT,   # before the sweep
                   "residual_mixed": abi.HF_KERNEL_RESIDUAL}                # that rewrites H x
        kms = {name: hf.time_kernel(k, reps=10) for name, k in kernels.items()}
        kms["rhs"] = rhs_ms
        detail["kernels"] = kernel_table(kms, N, peak, fp_rates, {"rhs": rhs_bytes(prob)})
    hf.close()

    # ---- plain FP64 GPU path at the same residual
    fp64 = None
    if not args.no_fp64:
        h2 = HeatFlow(prob, precision="fp64", criterion="true", tol=args.tol, use_graph=graph)
        h2.set_stream(stream.cuda_stream)
        h2.initial_evolve()
        if W:
            h2.run(1, W)
        if not args.no_autotune:
            cand = h2.autotune(itime0=W + 1, steps=6)
            best = next(r for r in cand if r["chosen"])
            tuned["fp64"] = {"task_depth": best["task_depth"], "candidates": len(cand)}
        barrier()
        ms64, st64 = timed_run(h2, torch, stream, W + 1, K)
        ms64 = max_over_ranks(ms64)
        solve64 = h2.time_kernel(abi.HF_KERNEL_SOLVE, 10)
        r64, n64 = h2.solve_profile()
        fp64 = {"steps_per_s": aggregate_rate(world, K, ms64), "ms_per_step": ms64 / K,
                "iterations_per_step": st64["iterations"] / K,
                "refinements_per_step": st64["refinements"] / K,
                "last_true_relres": st64["last_true_relres"],
                "solve_ms": solve64, "solve_rounds": n64,
                "solve_GB/s": solve_bytes_per_cell(r64, "fp64") * N / (solve64 / 1000.0) / 1e9}
        if args.detail:
            k64 = {"residual_fp64": h2.time_kernel(abi.HF_KERNEL_RESIDUAL, 10),
                   "xupdate_fp64": h2.time_kernel(abi.HF_KERNEL_XUPDATE, 10),
                   "cg_spmv_fp64": h2.time_kernel(abi.HF_KERNEL_CG_SPMV, 10),
                   "cg_update_fp64": h2.time_kernel(abi.HF_KERNEL_CG_UPDATE, 10),
                   "cg_p_fp64": h2.time_kernel(abi.HF_KERNEL_CG_P, 10)}
            detail["fp64_kernels"] = kernel_table(k64, N, peak, fp_rates)
            detail["fp64_phases"] = phase_table(r64, "fp64", N)
        h2.close()

    # ---- end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        kw3 = {}
        if "mixed" in tuned:
            kw3 = dict(task_depth=tuned["mixed"]["task_depth"], inner_tol=tuned["mixed"]["inner_tol"])
        h3 = HeatFlow(prob, precision="mixed", criterion="true", tol=args.tol, use_graph=graph, **kw3)
        h3.set_stream(stream.cuda_stream)
        # three pinned host fields: the step's inputs (T^n, T^(n-1)) go in, its result (the new
        # T^n) comes back into the third; the new T^(n-1) is the input T^n, already on the host
        bufs = [torch.full((N,), prob.t_system, dtype=torch.float64).pin_memory().numpy()
                for _ in range(3)]
        cur, prev, free = 0, 1, 2
        for k in range(W):
            h3.step_host_async(k + 1, bufs[cur], bufs[prev], bufs[free])
            cur, prev, free = free, cur, prev
        h3.host_sync()
        barrier()
        t0 = time.perf_counter()
        for k in range(K):
            h3.step_host_async(W + 1 + k, bufs[cur], bufs[prev], bufs[free])
            cur, prev, free = free, cur, prev
        h3.host_sync()
        e2e_s = max_over_ranks(time.perf_counter() - t0)
        # the same steps through the host-synchronous calls (no transfer overlapped with another)
        barrier()
        t0 = time.perf_counter()
        for k in range(K):
            h3.set_state(bufs[cur], bufs[prev])
            h3.simulate(W + K + 1 + k)
            h3.get_state(out=(bufs[free], None))
            cur, prev, free = free, cur, prev
        torch.cuda.synchronize()
        sync_s = max_over_ranks(time.perf_counter() - t0)
        e2e = {"value": world * K / e2e_s, "unit": UNIT, "h2d_bytes_per_step": 2 * 8 * N,
               "d2h_bytes_per_step": 8 * N,
               "timing": "wall clock, K steps through hf_step_host_async from/to pinned host "
                         "memory (T^n, T^(n-1) up, new T^n down every step), then hf_host_sync",
               "sync_value": world * K / sync_s,
               "sync_timing": "hf_set_state + hf_step + hf_get_state per step"}
        h3.close()

    cb = clean = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(prob, 2, 60.0, args.tol)
        cb = {k: cb[k] for k in ("value", "unit", "cores", "kind", "sample")}
        clean = cpu_clean_pcg(prob, 20, 15.0, args.tol)
        clean = {k: clean[k] for k in ("value", "unit", "cores", "kind", "ms_per_step", "sample")}

    if rank == 0:
        mixed_over_fp64 = (steps_per_s / fp64["steps_per_s"]) if fp64 else None
        # the contract keys first, the large sub-objects next, and the spec comparison
        # (mixed vs FP64 GPU at the same true residual) last, so it closes the line
        line = {
            "metric": METRIC, "value": steps_per_s, "unit": UNIT, "n_gpus": world, "steps": K,
            "warmup": W, "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": dict(workload_config(args, prob), autotuned=tuned),
            "gpu_launches": st["kernel_launches"],
            "roofline": roofline, "fp_rates_measured": fp_rates,
            "cpu_baseline": cb, "cpu_clean_pcg": clean, "clocks": clocks, "e2e": e2e,
            "cell_iters_per_s": cell_iters_per_s,
            "iterations_per_step": {"fp32_cg": st["inner_iterations"] / K,
                                    "fp64_refinement_sweeps": st["refinements"] / K},
            "last_true_relres": st["last_true_relres"],
            "fp64_gpu": fp64,
            "mixed_over_fp64": mixed_over_fp64,
        }
        line = compact(line)
        if args.detail:
            with open(args.detail, "w") as f:
                json.dump(compact(dict(detail, line=line)), f, indent=1)
        print(json.dumps(line, separators=(",", ":")), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
