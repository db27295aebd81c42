"""Non-convergence injected through the solver limits (no GPU fault): the reference's linbcg
simply leaves its loop after itmax iterations (`do iter=1,itmax`, mod_Sparse.f90:404) and simulate
goes on -- the NaN check, then Temp_pp = Temp_p, Temp_p = x (mod_evolve.f90:142-170).  With the
limits forced to 1 the library must do the same: count every such step in hf_stats.unconverged,
still rotate the state, and give the same bits on every step path (host-polled kernels, the
whole-loop graph around the persistent solve, the per-step conditional graph)."""
import numpy as np
import pytest

from heatflow_gb300.problem import point_source_cube
from heatflow_gb300.solver import HeatFlow

pytestmark = pytest.mark.gpu

STEPS = 6


def _run(prob, steps=STEPS, **kw):
    """Per-step fields of a run from the problem's initial state, and the run's statistics."""
    out, tot = [], {"unconverged": 0, "iterations": 0, "inner_iterations": 0, "refinements": 0}
    with HeatFlow(prob, **kw) as hf:
        hf.initial_evolve()
        for k in range(1, steps + 1):
            st = hf.run(k, 1)
            for key in tot:
                tot[key] += st[key]
            out.append(hf.get_state())
    return out, tot


@pytest.mark.parametrize("itmax", [1, 3])
def test_fp64_itmax_reached_every_step(cuda_lib, itmax):
    """FP64 with the reference's rule (tol 1e-32 is never met): every step stops at itmax, is
    counted unconverged, and rotates the state; the field follows the oracle's BiCG, which stops
    at the same iteration, and all three step paths agree bit for bit."""
    from oracle.oracle import Oracle
    prob = point_source_cube(10, icattaneo=1, power_in=1e-6)
    runs = {}
    for g in (0, 1, 2):
        runs[g] = _run(prob, precision="fp64", criterion="recursive", tol=1e-32, itmax=itmax,
                       use_graph=g)
    fields, st = runs[0]
    assert st["unconverged"] == STEPS
    assert st["iterations"] == STEPS * itmax
    for g in (1, 2):
        f2, s2 = runs[g]
        assert s2["unconverged"] == STEPS and s2["iterations"] == STEPS * itmax, g
        for (a, b), (c, d) in zip(fields, f2):
            assert np.array_equal(a, c) and np.array_equal(b, d), g
    # the state rotates although no step converged: T^(n-1) after step k is T^n after step k-1
    for k in range(1, STEPS):
        assert np.array_equal(fields[k][1], fields[k - 1][0])
    o = Oracle(prob)
    o.set_state(*prob.initial_state())
    for k in range(1, STEPS + 1):
        rc, it, _ = o.simulate(k, mode=0, tol=1e-32, itmax=itmax)
        assert rc == 0 and it == itmax + 1          # Fortran's DO leaves iter at itmax + 1
        T, _ = o.get_state()
        rel = np.linalg.norm(fields[k - 1][0] - T) / np.linalg.norm(T)
        assert rel <= 1e-12, (k, rel)
    # the field moved: a truncated solve is still a solve
    assert not np.array_equal(fields[-1][0], prob.initial_state()[0])


@pytest.mark.parametrize("inner_itmax,max_refine", [(1, 1), (1, 3), (2, 1)])
def test_mixed_limits_reached_every_step(cuda_lib, inner_itmax, max_refine):
    """Mixed precision with one FP32 CG iteration per inner solve and few refinement sweeps cannot
    reach the true residual 1e-10: every step is counted unconverged after max_refine + 1 sweeps,
    the state rotates, and the step paths agree bit for bit."""
    prob = point_source_cube(12, icattaneo=1, power_in=1e-5)
    runs = {g: _run(prob, precision="mixed", criterion="true", tol=1e-10,
                    inner_itmax=inner_itmax, max_refine=max_refine, use_graph=g) for g in (0, 1, 2)}
    fields, st = runs[0]
    assert st["unconverged"] == STEPS
    assert st["refinements"] == STEPS * (max_refine + 1)
    assert st["inner_iterations"] <= STEPS * max_refine * inner_itmax
    for g in (1, 2):
        f2, s2 = runs[g]
        assert s2 == st, g
        for (a, b), (c, d) in zip(fields, f2):
            assert np.array_equal(a, c) and np.array_equal(b, d), g
    for k in range(1, STEPS):
        assert np.array_equal(fields[k][1], fields[k - 1][0])
    assert all(np.isfinite(f[0]).all() for f in fields)
