"""Parity cases for the configurations the benchmark line does not time: the 128^3 layered slab
over 1000 graph-captured steps (mixed vs FP64), the batched sweep of 256 uneven grids over 200
steps (per-instance convergence; the smallest instances against the oracle), and the 512^3
inclusion grid over 100 steps (mixed vs FP64).  Each states its tolerance; the measured errors
are printed (pytest -s)."""
import numpy as np
import pytest

from heatflow_gb300.problem import batched_sweep, inclusions, layered_slab
from heatflow_gb300.solver import HeatFlow

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _pair(prob, steps, fp64_tol=1e-12):
    out = {}
    for prec, tol in (("fp64", fp64_tol), ("mixed", 1e-10)):
        with HeatFlow(prob, precision=prec, criterion="true", tol=tol, use_graph=1) as hf:
            hf.initial_evolve()
            st = hf.run(1, steps)
            out[prec] = (hf.get_state()[0], st)
    return out


@pytest.mark.parametrize("icattaneo", [0, 1])
def test_config_layered_slab_128_1000_steps(cuda_lib, icattaneo):
    """Layered slab 128^3, Fourier and Cattaneo, 1000 steps as one CUDA-graph loop per step:
    every step meets ||S - H T|| / ||S|| <= 1e-10 (mixed) / 1e-12 (FP64); after 1000 steps the
    mixed field agrees with the FP64 one to 1e-8 relative L2 (per-step residual 1e-10,
    accumulated) and its temperature rise to 1e-6."""
    out = _pair(layered_slab(128, icattaneo=icattaneo), 1000)
    (T64, s64), (T32, s32) = out["fp64"], out["mixed"]
    assert s64["unconverged"] == 0 and s32["unconverged"] == 0
    assert s64["last_true_relres"] <= 1e-12 and s32["last_true_relres"] <= 1e-10
    err_T = _rel(T32, T64)
    err_rise = _rel(T32 - 300.0, T64 - 300.0)
    print(f"\nconfig 2 (icattaneo={icattaneo}): mixed vs FP64 rel L2: T {err_T:.3e}, "
          f"T-300 {err_rise:.3e}; max rise {np.max(T64) - 300.0:.4g} K")
    assert err_T <= 1e-8
    assert err_rise <= 1e-6


def test_config_batched_sweep_256(cuda_lib):
    """256 grids with edges U{16..96}, lognormal kappa, 1-4 point sources, 200 Cattaneo steps in
    one persistent launch per step (autotuned): no instance leaves a step above rel-res 1e-10.
    The three smallest grids are run again alone on the FP64 path (true rel-res 1e-13) and on the
    oracle (BiCG, tol 1e-12): FP64 GPU vs oracle within 1e-10 relative L2 of the field, and the
    batched mixed field vs FP64 within 1e-8 (a per-step residual of 1e-10 accumulated over 200
    steps on high-contrast kappa)."""
    from oracle.oracle import Oracle
    probs = batched_sweep(256, seed=0)
    with HeatFlow(probs, precision="mixed", criterion="true", tol=1e-10, use_graph=1) as hf:
        hf.initial_evolve()
        hf.run(1, 2)
        cand = hf.autotune(itime0=3, steps=2)
        assert sum(c["chosen"] for c in cand) == 1
        st = hf.run(3, 198)
        parts = hf.split(hf.get_state()[0])
    assert st["unconverged"] == 0 and st["last_true_relres"] <= 1e-10
    small = sorted(range(len(probs)), key=lambda i: probs[i].ncells)[:3]
    for i in small:
        with HeatFlow(probs[i], precision="fp64", criterion="true", tol=1e-13, use_graph=1) as h1:
            h1.initial_evolve()
            h1.run(1, 200)
            T64 = h1.get_state()[0]
        o = Oracle(probs[i])
        o.set_state(*probs[i].initial_state())
        for k in range(200):
            rc, _, _ = o.simulate(k + 1, mode=0, tol=1e-12, itmax=50000)
            assert rc == 0
        Tref = o.get_state()[0]
        e64 = _rel(T64, Tref)
        e32 = _rel(parts[i], T64)
        rise = _rel(parts[i] - 300.0, T64 - 300.0)
        print(f"\nconfig 3 instance {i} ({probs[i].nx}x{probs[i].ny}x{probs[i].nz}): FP64 GPU vs "
              f"oracle {e64:.3e}; batched mixed vs FP64 {e32:.3e} (rise {rise:.3e})")
        assert e64 <= 1e-10
        assert e32 <= 1e-8


def test_config_inclusions_512_100_steps(cuda_lib):
    """512^3 (134M cells) with 5 % polymer inclusions, periodic x/y, 100 Cattaneo steps: both
    paths converge every step; the mixed field agrees with FP64 to 1e-8 relative L2 and its
    temperature rise (a few K) to 1e-5."""
    out = _pair(inclusions(512), 100, fp64_tol=1e-12)
    (T64, s64), (T32, s32) = out["fp64"], out["mixed"]
    assert s64["unconverged"] == 0 and s32["unconverged"] == 0
    assert s32["last_true_relres"] <= 1e-10
    err_T = _rel(T32, T64)
    err_rise = _rel(T32 - 300.0, T64 - 300.0)
    print(f"\nconfig 5: mixed vs FP64 rel L2: T {err_T:.3e}, rise {err_rise:.3e}; "
          f"max rise {np.max(T64) - 300.0:.4g} K")
    assert err_T <= 1e-8
    assert err_rise <= 1e-5


# ---- oracle legs at size: the FP64 GPU field tied to the reference's arithmetic ------------------
def _cpu_pcg_run(prob, steps, tol=1e-13):
    """The clean CPU solver (oracle/cpu_pcg.c: the oracle's operator bit for bit, Jacobi-PCG in
    FP64 to the true relative residual `tol`, all host cores) over `steps` steps."""
    import os
    from oracle.oracle import CleanPCG, Oracle
    o = Oracle(prob)
    o.set_state(*prob.initial_state())
    cp = CleanPCG(o, threads=os.cpu_count() or 1)
    for k in range(steps):
        rc, _, rel = cp.step(k + 1, tol=tol)
        assert rc == 0 and rel <= tol, (k, rc, rel)
    return o.get_state()[0]


def _gpu_run(probs, steps, precision):
    tol = 1e-13 if precision == "fp64" else 1e-10
    with HeatFlow(probs, precision=precision, criterion="true", tol=tol, use_graph=1) as hf:
        hf.initial_evolve()
        st = hf.run(1, steps)
        T = hf.get_state()[0]
        parts = hf.split(T) if isinstance(probs, list) else [T]
    assert st["unconverged"] == 0
    return parts


def test_config_layered_slab_128_vs_oracle(cuda_lib):
    """128^3 layered slab (Cattaneo), 10 steps: the FP64 GPU field against the oracle's BiCG (the
    reference's COO Jacobi-BiCG, tol 1e-12) within 1e-10 relative L2; the mixed field within 1e-9."""
    from oracle.oracle import Oracle, set_threads
    import os
    prob = layered_slab(128, icattaneo=1)
    # all host threads for this run only: with more than one, the oracle's SpMV takes the
    # reference's OpenMP-atomic form, whose summation order varies, and later bit-exact
    # comparisons with the oracle expect the serial order
    set_threads(os.cpu_count() or 1)
    try:
        o = Oracle(prob)
        o.set_state(*prob.initial_state())
        for k in range(10):
            rc, _, _ = o.simulate(k + 1, mode=0, tol=1e-12, itmax=50000)
            assert rc == 0
        Tref = o.get_state()[0]
    finally:
        set_threads(1)
    (T64,) = _gpu_run(prob, 10, "fp64")
    (T32,) = _gpu_run(prob, 10, "mixed")
    e64, e32 = _rel(T64, Tref), _rel(T32, Tref)
    print(f"\nconfig 2 at 128^3, 10 steps vs oracle BiCG: FP64 {e64:.3e}, mixed {e32:.3e}")
    assert e64 <= 1e-10 and e32 <= 1e-9


def test_config_batched_sweep_all_instances_vs_cpu(cuda_lib):
    """All 256 grids of the batched sweep, 20 steps in one persistent launch per step: every
    instance's FP64 GPU field within 1e-10 relative L2 of the CPU FP64 solver (true rel-res
    1e-13) on the same grid, and every mixed field within 1e-9."""
    probs = batched_sweep(256, seed=0)
    g64 = _gpu_run(probs, 20, "fp64")
    g32 = _gpu_run(probs, 20, "mixed")
    worst64 = worst32 = 0.0
    for i, p in enumerate(probs):
        Tref = _cpu_pcg_run(p, 20)
        e64, e32 = _rel(g64[i], Tref), _rel(g32[i], Tref)
        worst64, worst32 = max(worst64, e64), max(worst32, e32)
        assert e64 <= 1e-10, (i, e64)
        assert e32 <= 1e-9, (i, e32)
    print(f"\nconfig 3, 256 instances x 20 steps vs CPU FP64 PCG: worst FP64 {worst64:.3e}, "
          f"worst mixed {worst32:.3e}")


def test_config_inclusions_512_vs_cpu(cuda_lib):
    """512^3 inclusion grid (periodic x/y), 3 steps: the FP64 GPU field within 1e-10 relative L2
    of the CPU FP64 solver on the same grid, the mixed field within 1e-9."""
    prob = inclusions(512)
    (T64,) = _gpu_run(prob, 3, "fp64")
    (T32,) = _gpu_run(prob, 3, "mixed")
    Tref = _cpu_pcg_run(prob, 3)
    e64, e32 = _rel(T64, Tref), _rel(T32, Tref)
    print(f"\nconfig 5 at 512^3, 3 steps vs CPU FP64 PCG: FP64 {e64:.3e}, mixed {e32:.3e}")
    assert e64 <= 1e-10 and e32 <= 1e-9
