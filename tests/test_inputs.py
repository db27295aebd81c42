"""Readers of the reference's input decks and restart files (host set-up, CPU only)."""
import numpy as np
import pytest

from heatflow_gb300 import inputs


def test_read_test_deck(golden):
    param, prob = inputs.read_all_files(golden["param_in"], golden["mat_in"], golden["system_in"])
    assert (prob.nx, prob.ny, prob.nz) == (25, 25, 1)
    assert param["ntime"] == 10 and param["icattaneo"] == 0 and param["isteady"] == 0
    assert prob.t_bath_face == (283.0, 278.0, 278.0, 278.0, 278.0, 278.0)
    assert prob.kappa_bound == (0.541,) * 6
    assert np.all(prob.kappa == 0.541) and np.all(prob.rho == 997.0)
    assert np.all(prob.heat_capacity == 4200.0) and np.all(prob.iheater == 0)
    assert prob.t_system == 278.0 and prob.time_step == 1.0
    assert prob.periodic == (0, 0, 0)


def test_duplicate_keyword():
    with pytest.raises(inputs.InputError):
        inputs.read_param("ntime = 1\nntime = 2\nkappaBound = 1\n")


def test_missing_kappa_bound():
    with pytest.raises(inputs.InputError):
        inputs.read_param("ntime = 1\n")


def test_kappa_bound_fallback_and_periodic():
    p = inputs.read_param("kappaBound = 3.5\nPeriodic = xz\nT_Bath = 290\nCG_dir = -x+z\n")
    assert p["kappaBoundx1"] == 3.5 and p["kappaBoundNz"] == 3.5
    assert p["Periodicx"] and not p["Periodicy"] and p["Periodicz"]
    assert p["T_Bathx1"] == 290.0 and p["T_Bathz2"] == 290.0
    assert p["CG_x_m"] and p["CG_z_p"] and not p["CG_x_p"]
    # list-directed read of a string stops at the first blank (assignS, mod_inputs.f90:800)
    p = inputs.read_param("kappaBound = 1\nCG_dir = -x +z\n")
    assert p["CG_x_m"] and not p["CG_z_p"]


def test_mat_errors():
    with pytest.raises(inputs.InputError):
        inputs.read_mat("1\nkappa = 1\n0\n")          # missing parameters before the 0 line
    text = "1\n" + "".join(f"{k} = 1\n" for k in inputs.MAT_KEYS) + "0\n"
    with pytest.raises(inputs.InputError):
        inputs.read_mat(text + text)                  # duplicate index


def test_unknown_material():
    with pytest.raises(inputs.InputError):
        inputs.material(55, [])
    with pytest.raises(inputs.InputError):
        inputs.material(0, [])


def test_temp_file_round_trip():
    vals = np.linspace(270.0, 310.0, 13)
    text = inputs.format_temp_file(vals)
    lines = text.splitlines()
    assert len(lines[0]) == 6 * 17 and lines[-1] == "" and lines[-2] == ""
    back = inputs.parse_temp_file(text, 13)
    np.testing.assert_allclose(back, vals, rtol=1e-8)
    with pytest.raises(inputs.InputError):
        inputs.parse_temp_file(text, 14)
    with pytest.raises(inputs.InputError):
        inputs.parse_temp_file(text, 12)


def test_golden_file_parses(golden):
    txt = "\n".join(" ".join(f"{v:.8E}" for v in golden["tempdis"][k:k + 6])
                    for k in range(0, 625, 6))
    assert inputs.parse_temp_file(txt, 625).shape == (625,)
