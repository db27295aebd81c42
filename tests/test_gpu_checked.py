"""The index-checked build (-DHF_CHECKED, heatflow_gb300/_build/checked/): every global load and
store of the step kernels checks its index against its array's extent and records a failure
instead of touching memory outside the array.  It stands in for a memory checker: on the tiny
grids where edge, wrap and padding rules matter most (one cell, periodic axes of length 2, FP32
rows padded to 4 cells, one-layer and one-line grids, Neumann faces, heaters, uneven batches) every
step path runs with no failed check, and gives the bits of the normal build."""
import numpy as np
import pytest

from heatflow_gb300 import abi
from heatflow_gb300.problem import Problem, point_source_cube
from heatflow_gb300.solver import HeatFlow

pytestmark = pytest.mark.gpu


def _rng_problem(nx, ny, nz, seed=3, **kw):
    rng = np.random.default_rng(seed + nx * 100 + ny * 10 + nz)
    N = nx * ny * nz
    ih = np.zeros(N, np.int64)
    ih[rng.integers(0, N)] = 1
    base = dict(nx=nx, ny=ny, nz=nz, lx=nx * 1e-9, ly=ny * 1.3e-9, lz=nz * 0.8e-9,
                kappa=rng.choice([149.0, 0.2, 50.0], size=N), rho=rng.uniform(1000, 3000, N),
                heat_capacity=rng.uniform(500, 1500, N), tau=1e-12, em=0.0, iheater=ih,
                power_in=1e-6, time_step=1e-13, icattaneo=1,
                kappa_bound=(149.0, 20.0, 149.0, 0.2, 60.0, 149.0),
                t_bath_face=(300.0, 310.0, 295.0, 300.0, 305.0, 290.0), t_bath=300.0, br=0.7)
    base.update(kw)
    return Problem(**base)


CASES = {
    "single_cell": [_rng_problem(1, 1, 1)],
    "periodic_n2": [_rng_problem(2, 2, 2, periodic=(1, 1, 1))],
    "padded_rows_periodic_x": [_rng_problem(5, 3, 4, periodic=(1, 0, 0))],
    "padded_rows_n6": [_rng_problem(6, 7, 3, periodic=(0, 1, 1))],
    "vector_rows": [_rng_problem(8, 4, 5)],
    "one_layer": [_rng_problem(9, 5, 1)],
    "one_line": [_rng_problem(7, 1, 1)],
    "neumann": [_rng_problem(4, 5, 3, cg_face=(1, 0, 0, 0, 0, 1), t_bath_cg=2.0)],
    "emissivity": [_rng_problem(4, 4, 4, em=0.3)],
    "batch": [_rng_problem(1, 1, 1), _rng_problem(2, 2, 2, periodic=(1, 1, 1)),
              _rng_problem(5, 3, 4), point_source_cube(8), _rng_problem(35, 9, 33)],
}


@pytest.fixture(scope="module")
def checked_lib(cuda_lib):
    from heatflow_gb300.build import build_library
    build_library(checked=True)
    return abi.load_library(checked=True)


def _run(probs, lib, steps=4, **kw):
    with HeatFlow(probs, library=lib, **kw) as hf:
        hf.initial_evolve()
        st = hf.run(1, steps)
        T = hf.get_state()
        en, rec = hf.index_checks()
    return T, st, en, rec


@pytest.mark.parametrize("use_graph", [0, 1, 2])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("name", sorted(CASES))
def test_no_index_fails_on_tiny_grids(checked_lib, name, precision, use_graph):
    probs = CASES[name]
    kw = dict(precision=precision, criterion="true", tol=1e-10 if precision == "mixed" else 1e-13,
              use_graph=use_graph)
    (T, Tp), st, en, rec = _run(probs, checked_lib, **kw)
    assert en is True
    assert rec[0] == 0, rec
    assert st["unconverged"] == 0
    (T0, Tp0), st0, en0, _ = _run(probs, abi.load_library(), **kw)
    assert en0 is False
    assert np.array_equal(T, T0) and np.array_equal(Tp, Tp0)


def test_failed_check_is_recorded(checked_lib):
    """The probe runs one check on an index outside its range (no memory access): the record
    names it (a site in the solver's file, 3), and reading the record clears it."""
    with HeatFlow(point_source_cube(4), library=checked_lib) as hf:
        en, rec = hf.index_checks(probe=True)
        assert en is True and rec[0] == 1 and rec[1] // 100000 == 3 and rec[2] == -1 and rec[3] == 1
        assert hf.index_checks()[1][0] == 0
        hf.initial_evolve()
        hf.run(1, 2)                                     # the context stays usable
        assert hf.index_checks()[1][0] == 0
