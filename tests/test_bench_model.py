"""bench.py's algorithmic-byte and FP64-instruction model of the persistent solve's rounds and of
the RHS kernel, which the roofline fractions rest on (no GPU): the bytes of each round follow its
phase, a CG update that formed x counts the x update's bytes only when the next residual sweep
reads that x, iteration 0 has no direction round, and the RHS is charged B only on the outer faces
and the heater arrays only on heated cells."""
import numpy as np
import pytest

import bench
from heatflow_gb300.problem import layered_slab, point_source_cube

MIX = bench.PHASE_BYTES["mixed"]


def _rounds(*phases):
    return [(p, 1.0) for p in phases]


def test_one_inner_solve_with_fused_x_update():
    r = _rounds("res_init_hx", "cg_q", "cg_b", "cg_p", "cg_q", "cg_bx", "res")
    b = bench.round_bytes_per_cell(r, "mixed")
    assert b == [MIX["res_init_hx"][0], MIX["cg_q"][0], MIX["cg_b"][1], MIX["cg_p"][0],
                 MIX["cg_q"][0], MIX["cg_bx"][0] + bench.XB["mixed"], MIX["res"][0]]
    # the same solve with the separate x update: the x update's bytes move to their own round
    r2 = _rounds("res_init_hx", "cg_q", "cg_b", "cg_p", "cg_q", "cg_b", "xupd", "res")
    b2 = bench.round_bytes_per_cell(r2, "mixed")
    assert sum(b2) - sum(b) == MIX["xupd"][0] - bench.XB["mixed"]


def test_fused_x_update_that_was_not_the_last():
    """The prediction fired one iteration early: that round's x is overwritten, so only the CG
    update's bytes count there, and the x formed by the final update counts once."""
    r = _rounds("res_init_hx", "cg_q", "cg_bx", "cg_p", "cg_q", "cg_bx", "res")
    b = bench.round_bytes_per_cell(r, "mixed")
    assert b[2] == MIX["cg_bx"][1]
    assert b[5] == MIX["cg_bx"][0] + bench.XB["mixed"]


def test_direction_rounds_always_full():
    for prec in ("mixed", "fp64"):
        r = _rounds("res_init_hx", "cg_q", "cg_b", "cg_p", "cg_q", "cg_b", "cg_p", "cg_q",
                    "cg_b", "xupd", "res")
        b = bench.round_bytes_per_cell(r, prec)
        full = bench.PHASE_BYTES[prec]["cg_p"][0]
        assert b[3] == full and b[6] == full


def test_second_inner_solve_restarts_first_iteration_forms():
    r = _rounds("res_init_hx", "cg_q", "cg_b", "xupd", "res", "cg_q", "cg_b", "xupd", "res")
    b = bench.round_bytes_per_cell(r, "mixed")
    assert b[2] == MIX["cg_b"][1] and b[6] == MIX["cg_b"][1]
    assert b[3] == MIX["xupd"][0] and b[7] == MIX["xupd"][0]


def test_solve_floor_marks_the_residual_fp64_bound():
    N = 256 ** 3
    r = [("res_init_hx", 124.0), ("cg_q", 70.0), ("cg_b", 63.0), ("cg_p", 34.0), ("cg_q", 70.0),
         ("cg_bx", 124.0), ("res", 317.0)]
    f = bench.solve_floor(r, "mixed", N, 6794.0, 1.056)
    assert f["by_phase"]["res"]["bound"] == "fp64"
    assert f["by_phase"]["cg_q"]["bound"] == "hbm"
    assert f["by_phase"]["res_init_hx"]["bound"] == "hbm"    # 2 FP64 instructions per cell
    # the residual's floor is its 8 FP64 instructions per cell at the FP64 issue rate
    floor_res = 8 * N / (1.056e12 / 2) * 1e6
    assert f["by_phase"]["res"]["floor_us"] == pytest.approx(floor_res)
    assert 0.0 < f["frac"] < 1.0


@pytest.mark.parametrize("n", [8, 12, 20])
def test_rhs_bytes_counts_faces_and_heated_cells(n):
    prob = layered_slab(n, layer=4)
    N = n ** 3
    faces = N - (n - 2) ** 3
    heated = int(np.count_nonzero(np.asarray(prob.iheater) > 0))
    assert heated == n * n                                  # the heated top face
    assert bench.rhs_bytes(prob) == 48 * N + 8 * faces + 9 * heated


def test_rhs_bytes_periodic_axes_have_no_faces():
    prob = point_source_cube(10)
    prob.periodic = (1, 1, 0)
    N = 1000
    faces = N - 10 * 10 * 8                                 # only the z faces
    assert bench.rhs_bytes(prob) == 48 * N + 8 * faces + 9 * 1
