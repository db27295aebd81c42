"""The oracle (CPU restatement of the reference) against the reference's own known answers.

Pins: test/data/TempDis.dat (golden run), the manual's Chapter 6 steady 1-D cases 1-4,
test/test_mod_cattaneo.f90:64-73, test/test_mod_boundary.f90:64-72,
test/test_mod_hmatrix.f90:56-64 and test/test_mod_material.f90:21-32.
"""
import numpy as np
import pytest

from heatflow_gb300 import inputs
from heatflow_gb300.problem import Problem, point_source_cube
from oracle.oracle import Oracle


def test_golden_tempdis(golden):
    """10 Fourier steps of the reference's test deck reproduce its TempDis.dat to the ES16.8
    print precision (8 significant decimals after the point)."""
    param, prob = inputs.read_all_files(golden["param_in"], golden["mat_in"], golden["system_in"])
    o = Oracle(prob)
    tp, tpp = prob.initial_state()
    o.set_state(tp, tpp)
    rc, iters = o.run(param["ntime"], mode=0, tol=1e-32, itmax=50000)
    assert rc == 0
    T, _ = o.get_state()
    gold = np.asarray(golden["tempdis"])
    assert np.linalg.norm(T - gold) / np.linalg.norm(gold) < 1.1e-9
    assert np.max(np.abs(T - gold)) <= 5.0e-7 + 1e-12      # half an ES16.8 unit at ~280 K
    assert all(100 < it < 200 for it in iters)              # BiCG at tol=1e-32 (observed 130-161)


def _manual_case(kappa_mid: float, heat: float):
    """Manual Chapter 6: three cells along x, kappaBound(x)=1, kappaBound(y,z)=0, boundary 200,
    steady state, heater density `heat` in the middle cell."""
    ih = np.array([0, 1 if heat else 0, 0], np.int64)
    return Problem(nx=3, ny=1, nz=1, lx=3.0, ly=1.0, lz=1.0, kappa=np.array([1.0, kappa_mid, 1.0]),
                   rho=1.0, heat_capacity=1.0, tau=0.0, em=0.0, iheater=ih, power_in=heat,
                   time_step=1.0, icattaneo=0, isteady=1, kappa_bound=(1, 1, 0, 0, 0, 0),
                   t_bath_face=(200.0,) * 6, t_bath=200.0, br=1.0, t_system=200.0)


@pytest.mark.parametrize("kappa_mid,heat,expect", [
    (1.0, 0.0, [200.0, 200.0, 200.0]),
    (1.0, 10.0, [205.0, 210.0, 205.0]),
    (2.0, 0.0, [200.0, 200.0, 200.0]),
    (2.0, 10.0, [205.0, 208.75, 205.0]),
])
def test_manual_cases(kappa_mid, heat, expect):
    prob = _manual_case(kappa_mid, heat)
    o = Oracle(prob)
    tp, tpp = prob.initial_state()
    o.set_state(tp, tpp)
    rc, _ = o.run(1)
    assert rc == 0
    T, _ = o.get_state()
    np.testing.assert_allclose(T, expect, rtol=0, atol=1e-9)


def test_manual_case3_matrix():
    """Manual case 3 prints H = [[-7/3, 4/3, 0], [4/3, -8/3, 4/3], [0, 4/3, -7/3]]."""
    H = Oracle(_manual_case(2.0, 0.0)).dense()
    np.testing.assert_allclose(H, [[-7 / 3, 4 / 3, 0], [4 / 3, -8 / 3, 4 / 3], [0, 4 / 3, -7 / 3]],
                               rtol=1e-15, atol=0)


def test_cattaneo_formula():
    """test_mod_cattaneo.f90:64-73: S_cat = (T_pp - 2 T_p) tau rhoc with tau already scaled."""
    n = 3
    # tau given unscaled: the oracle scales by 1/dt^2 (dt = 0.5 -> factor 4); pick tau so that
    # the scaled value is the test's 0.5
    prob = Problem(nx=n, ny=n, nz=n, lx=3, ly=3, lz=3, kappa=1.0, rho=1.0, heat_capacity=1.0,
                   tau=0.5 * 0.25, time_step=0.5, kappa_bound=(1,) * 6)
    o = Oracle(prob)
    tp = np.full(27, 100.0)
    s = o.cattaneo(tp, tp)
    np.testing.assert_allclose(s, (100.0 - 200.0) * 0.5 * 1.0, rtol=0, atol=1e-12)


def test_boundary_corner():
    """test_mod_boundary.f90:64-72: 3x3x3, kappa = kappaBound = 1, L = 1, baths 300 -> B(1) = 900."""
    prob = Problem(nx=3, ny=3, nz=3, lx=3, ly=3, lz=3, kappa=1.0, rho=1.0, heat_capacity=1.0,
                   tau=0.0, kappa_bound=(1,) * 6, t_bath_face=(300.0,) * 6, br=0.0)
    B = Oracle(prob).boundary()
    assert abs(B[0] - 900.0) <= 1e-10
    assert B[13] == 0.0                # the centre cell has no outside face


def test_alpha_fourier():
    """test_mod_hmatrix.f90:56-64: calculate_alpha = rhoc/dt in Fourier mode; visible as the
    diagonal of a 1-cell steady-free grid minus its six boundary faces."""
    prob = Problem(nx=1, ny=1, nz=1, lx=1, ly=1, lz=1, kappa=1.0, rho=1.0, heat_capacity=1.0,
                   tau=0.0, icattaneo=0, time_step=1.0, kappa_bound=(0,) * 6, br=1.0)
    H = Oracle(prob).dense()
    assert H[0, 0] == -1.0             # -(0 faces) - rhoc * (1/dt)


def test_silicon_material():
    """test_mod_material.f90:21-32: built-in material 140."""
    m = inputs.material(140, [])
    assert (m.kappa, m.kappa3D, m.heat_capacity, m.rho, m.sound_speed) == (130.0, 130.0, 4200.0, 2328.0, 8433.0)


def test_config1_iterations():
    """20^3 Cattaneo point source: BiCG at tol=1e-32 takes tens of iterations per step and the
    source cell warms monotonically."""
    prob = point_source_cube(20)
    o = Oracle(prob)
    tp, tpp = prob.initial_state()
    o.set_state(tp, tpp)
    rc, iters = o.run(3)
    assert rc == 0
    assert all(40 <= it <= 200 for it in iters), iters
    T, _ = o.get_state()
    assert T.max() > 300.0 and np.argmax(T) == 9 + 20 * (9 + 20 * 9)
