"""The bounded-wait failure path of the persistent solve, exercised without any GPU fault: one
block leaves without arriving at the grid barrier, the others give up after a short time limit,
the host reads HF_EDEVICE, and the context keeps working (its next steps equal an untouched run)."""
import ctypes as C

import numpy as np
import pytest

from heatflow_gb300 import abi
from heatflow_gb300.problem import point_source_cube
from heatflow_gb300.solver import HeatFlow

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_barrier_timeout_is_reported_and_context_survives(cuda_lib, precision):
    prob = point_source_cube(40)
    kw = dict(precision=precision, criterion="true", tol=1e-10, use_graph=1)
    lib = abi.load_library()
    with HeatFlow(prob, **kw) as hf:
        hf.initial_evolve()
        hf.run(1, 2)
        status, seconds = C.c_int32(), C.c_double()
        rc = lib.hf_check_barrier_timeout(hf.h, 200, C.byref(status), C.byref(seconds))
        assert rc == abi.HF_OK, lib.hf_last_error()
        assert status.value == abi.HF_EDEVICE
        assert 0.2 <= seconds.value < 3.0, seconds.value
        hf.run(3, 3)
        T = hf.get_state()
    with HeatFlow(prob, **kw) as h2:
        h2.initial_evolve()
        h2.run(1, 2)
        h2.run(3, 3)
        T2 = h2.get_state()
    assert np.array_equal(T[0], T2[0]) and np.array_equal(T[1], T2[1])
