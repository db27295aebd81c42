"""The first residual of a step from the stored products H T^n and H T^(n-1): used once two
consecutive steps of the context stored them, dropped whenever the state or the operator changes
outside the step sequence, and in agreement with the stencil sweep it replaces."""
import numpy as np
import pytest

from heatflow_gb300.problem import layered_slab
from heatflow_gb300.solver import HeatFlow
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def _prob():
    return layered_slab(16, nz=20, layer=5)


def _phases(hf):
    rounds, _ = hf.solve_profile()
    return [p for p, _ in rounds]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_products_used_from_the_third_step(cuda_lib, precision):
    with HeatFlow(_prob(), precision=precision, criterion="true", tol=1e-10, use_graph=3) as hf:
        hf.initial_evolve()
        first = []
        for k in range(1, 6):
            hf.run(k, 1)
            first.append(_phases(hf)[0])
    assert first[:2] == ["res_init", "res_init"], first
    assert all(p == "res_init_hx" for p in first[2:]), first


def test_continuation_keeps_products_and_bits(cuda_lib):
    """One run of 10 steps and 4 + 6 steps over two calls give the same bits."""
    out = []
    for split in (None, 4):
        with HeatFlow(_prob(), precision="mixed", criterion="true", tol=1e-10, use_graph=1) as hf:
            hf.initial_evolve()
            if split is None:
                hf.run(1, 10)
            else:
                hf.run(1, split)
                hf.run(split + 1, 10 - split)
            out.append(hf.get_state())
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])


@pytest.mark.parametrize("use_graph", [0, 1, 2])
def test_set_state_drops_products(cuda_lib, use_graph):
    """A state written from the host is stepped exactly like the same state in a fresh context
    (both form their first two residuals with the stencil sweep), on every step path."""
    prob = _prob()
    with HeatFlow(prob, precision="mixed", criterion="true", tol=1e-10, use_graph=use_graph) as a:
        a.initial_evolve()
        a.run(1, 6)
        Tp, Tpp = a.get_state()
        a.set_state(Tp, Tpp)
        a.run(7, 4)
        ra = a.get_state()
    with HeatFlow(prob, precision="mixed", criterion="true", tol=1e-10, use_graph=use_graph) as b:
        b.set_state(Tp, Tpp)
        b.run(7, 4)
        rb = b.get_state()
    assert np.array_equal(ra[0], rb[0]) and np.array_equal(ra[1], rb[1])


def test_products_agree_with_stencil_start(cuda_lib):
    """Twenty steps with the stored products and twenty steps that each restart from a host-written
    state (stencil first residual every step) agree to the solver tolerance, and both stay within
    1e-9 of the oracle."""
    prob = _prob()
    o = Oracle(prob)
    o.set_state(*prob.initial_state())
    rc, _ = o.run(20, itime0=1, mode=0, tol=1e-32, itmax=50000)
    assert rc == 0
    Tref = o.get_state()[0]
    with HeatFlow(prob, precision="mixed", criterion="true", tol=1e-10, use_graph=1) as hf:
        hf.initial_evolve()
        hf.run(1, 20)
        T_hx = hf.get_state()[0]
    with HeatFlow(prob, precision="mixed", criterion="true", tol=1e-10, use_graph=1) as hf:
        hf.initial_evolve()
        for k in range(1, 21):
            hf.set_state(*hf.get_state())
            hf.run(k, 1)
        T_st = hf.get_state()[0]
    scale = np.linalg.norm(Tref)
    assert np.linalg.norm(T_hx - T_st) / scale <= 1e-10
    assert np.linalg.norm(T_hx - Tref) / scale <= 1e-9
    assert np.linalg.norm(T_st - Tref) / scale <= 1e-9


def test_timing_restores_products(cuda_lib):
    """Timing the persistent solve repeats a step's solve and restores H T^(n-1) for every
    repetition: the following steps give the bits of an untimed run."""
    from heatflow_gb300 import abi
    out = []
    for timed in (False, True):
        with HeatFlow(_prob(), precision="mixed", criterion="true", tol=1e-10, use_graph=1) as hf:
            hf.initial_evolve()
            hf.run(1, 5)
            if timed:
                hf.time_kernel(abi.HF_KERNEL_SOLVE, reps=3)
                hf.time_kernel(abi.HF_KERNEL_RESIDUAL_INIT, reps=2)
            hf.run(6, 4)
            out.append(hf.get_state()[0])
    assert np.array_equal(out[0], out[1])


def test_property_tables_never_use_products(cuda_lib):
    """With temperature-dependent properties H changes after every step: no step starts from the
    stored products."""
    prob = _prob()
    T = np.array([250.0, 300.0, 400.0])
    tab = np.c_[T, 150.0 - 0.3 * (T - 250.0), 2300.0 + 0.0 * T, 700.0 + 0.5 * (T - 250.0)]
    with HeatFlow(prob, precision="mixed", criterion="true", tol=1e-10, use_graph=3) as hf:
        hf.set_property_tables([tab], np.zeros(prob.ncells, np.int32))
        hf.initial_evolve()
        first = []
        for k in range(1, 5):
            hf.run(k, 1)
            first.append(_phases(hf)[0])
    assert first == ["res_init"] * 4, first
