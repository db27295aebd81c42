"""The clean CPU solver (oracle/cpu_pcg.c, the second CPU baseline): its geometric operator is
the oracle's H bit for bit, and its steps match the faithful restatement's (Jacobi-BiCG to the
reference's 1e-32) to the solver tolerance, with the true relative residual at or below it."""
import numpy as np
import pytest

from heatflow_gb300.problem import Problem, layered_slab
from heatflow_gb300.solver import geometric_to_dense
from oracle.oracle import CleanPCG, Oracle, lib


def _periodic_problem():
    rng = np.random.default_rng(5)
    nx, ny, nz = 6, 5, 4
    N = nx * ny * nz
    ih = np.zeros(N, np.int64)
    ih[rng.choice(N, 3, replace=False)] = 1
    return Problem(nx=nx, ny=ny, nz=nz, lx=nx * 1e-9, ly=ny * 1e-9, lz=nz * 1e-9,
                   kappa=rng.choice([149.0, 0.2, 50.0], N), rho=rng.uniform(1000, 3000, N),
                   heat_capacity=rng.uniform(500, 1500, N), tau=1e-12, em=0.0, iheater=ih,
                   power_in=3e-6, time_step=1e-13, icattaneo=1, periodic=(1, 0, 1),
                   kappa_bound=(149.0,) * 6, t_bath_face=(300.0,) * 6, t_bath=300.0, br=0.8)


CASES = [layered_slab(8, nz=12, layer=3), _periodic_problem(),
         Problem(nx=2, ny=3, nz=2, lx=2e-9, ly=3e-9, lz=2e-9, kappa=149.0, rho=2329.0,
                 heat_capacity=710.0, tau=1e-12, time_step=1e-13, periodic=(1, 1, 1),
                 iheater=np.r_[1, np.zeros(11, np.int64)], power_in=1e-6,
                 kappa_bound=(149.0,) * 6, t_bath_face=(300.0,) * 6, t_bath=300.0)]


@pytest.mark.parametrize("k", range(len(CASES)))
def test_geometric_operator_is_the_oracle_H(k):
    prob = CASES[k]
    o = Oracle(prob)
    arrs = {name: np.empty(prob.ncells) for name in ("diag", "cx", "cy", "cz")}
    lib().or_geometric(o.h, *[a.ctypes.data_as(lib().or_geometric.argtypes[1]) for a in arrs.values()])
    assert np.array_equal(geometric_to_dense(prob, arrs), o.dense())


@pytest.mark.parametrize("k", range(len(CASES)))
def test_clean_pcg_steps_match_the_faithful_solver(k):
    prob = CASES[k]
    ref = Oracle(prob)
    ref.set_state(*prob.initial_state())
    rc, _ = ref.run(6, itime0=1, mode=0, tol=1e-32, itmax=50000)
    assert rc == 0
    o = Oracle(prob)
    o.set_state(*prob.initial_state())
    cp = CleanPCG(o, threads=2)
    for itime in range(1, 7):
        rc, it, rel = cp.step(itime, tol=1e-12)
        assert rc == 0 and rel <= 1e-12, (itime, rel)
    T, Tref = o.get_state()[0], ref.get_state()[0]
    assert np.linalg.norm(T - Tref) / np.linalg.norm(Tref) <= 1e-11
