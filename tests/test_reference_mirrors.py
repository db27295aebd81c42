"""The reference's own unit-test fixtures run through this implementation.

test/test_mod_evolve.f90:48-101 builds a 10x10x1 grid (L = 1 per cell, kappa = kappa_B = 1,
rho*c = 1, dt = 1, every cell a case-1 heater with power_in = 1, 300 K baths, steady state,
TempDepProp = 1) and checks that one simulate step yields no NaN and no negative temperature
(:28-37).  TempDepProp = 1 makes the reference rebuild H from unchanged properties after the step
(mod_tempdep.f90: the table lookup is commented out), which changes no result, so it needs no
counterpart here.  The oracle runs the fixture on the CPU; the GPU path must match it."""
import numpy as np
import pytest

from heatflow_gb300.problem import Problem


def evolve_fixture():
    n = 100
    return Problem(nx=10, ny=10, nz=1, lx=10.0, ly=10.0, lz=1.0, kappa=1.0, rho=1.0,
                   heat_capacity=1.0, tau=0.0, em=0.0, iheater=np.ones(n, np.int64),
                   power_in=1.0, time_step=1.0, icattaneo=1, isteady=1,
                   kappa_bound=(1.0,) * 6, t_bath_face=(300.0,) * 6, t_bath=300.0, t_bath_cg=0.0)


def test_evolve_fixture_oracle():
    from oracle.oracle import Oracle
    prob = evolve_fixture()
    o = Oracle(prob)
    o.set_state(*prob.initial_state())
    rc, _, _ = o.simulate(1, mode=0, tol=1e-32, itmax=50000)
    assert rc == 0
    T, _ = o.get_state()
    assert not np.isnan(T).any() and (T >= 0.0).all()
    assert T.max() > 300.0                      # every cell is heated


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [0, 1])
def test_evolve_fixture_gpu(cuda_lib, use_graph):
    from oracle.oracle import Oracle
    from heatflow_gb300.solver import HeatFlow
    prob = evolve_fixture()
    o = Oracle(prob)
    o.set_state(*prob.initial_state())
    o.simulate(1, mode=0, tol=1e-32, itmax=50000)
    Tref, _ = o.get_state()
    with HeatFlow(prob, precision="fp64", criterion="recursive", tol=1e-32,
                  use_graph=use_graph) as hf:
        hf.initial_evolve()
        hf.simulate(1)
        T, _ = hf.get_state()
    assert not np.isnan(T).any() and (T >= 0.0).all()
    assert np.linalg.norm(T - Tref) / np.linalg.norm(Tref) <= 1e-12
