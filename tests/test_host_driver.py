"""The C++ host program (heatflow_gb300/host): its deck readers give the problem the Python readers
give (both restate mod_inputs.f90 / mod_material.f90), value for value, and it stops with the
reference's messages on the reference's input errors.  No GPU: --dump-problem stops before the
first CUDA call."""
import json
import os
import re
import subprocess

import numpy as np
import pytest

from heatflow_gb300 import inputs
from heatflow_gb300.build import build_driver, build_library


@pytest.fixture(scope="module")
def driver():
    build_library()
    return build_driver()


def _write_deck(d, param, mat, system):
    os.makedirs(d, exist_ok=True)
    for name, text in (("param.in", param), ("mat.in", mat), ("system.in", system)):
        with open(os.path.join(d, name), "w") as f:
            f.write(text)


def _dump(driver, d):
    r = subprocess.run([driver, "--inputs", d, "--dump-problem"], capture_output=True, text=True)
    return r.returncode, r.stdout


def _compare(js, param, prob):
    assert (js["nx"], js["ny"], js["nz"]) == (prob.nx, prob.ny, prob.nz)
    assert (js["lx"], js["ly"], js["lz"]) == (prob.lx, prob.ly, prob.lz)
    for k in ("kappa", "rho", "heat_capacity", "tau"):
        assert np.array_equal(np.asarray(js[k]), getattr(prob, k)), k
    em = prob.em if prob.em is not None else np.zeros(prob.ncells)
    assert np.array_equal(np.asarray(js["em"]), em)
    assert np.array_equal(np.asarray(js["iheater"]), prob.iheater)
    for k in ("power_in", "freq", "time_step", "heated_steps", "icattaneo", "isteady", "t_bath",
              "t_bath_cg", "br", "t_system"):
        assert js[k] == getattr(prob, k), k
    assert tuple(js["periodic"]) == tuple(prob.periodic)
    assert tuple(js["cg_face"]) == tuple(prob.cg_face)
    assert tuple(js["kappa_bound"]) == tuple(prob.kappa_bound)
    assert tuple(js["t_bath_face"]) == tuple(prob.t_bath_face)
    assert js["ntime"] == param["ntime"] and js["write_every"] == param["write_every"]
    assert js["run_name"] == param["_RunName"]
    assert js["box"] == [param[k] for k in ("start_ix", "end_ix", "start_iy", "end_iy",
                                            "start_iz", "end_iz")]
    assert js["input_temp_dis"] == int(param["_InputTempDis"])
    assert js["write_to_txt"] == int(param["_WriteToTxt"])


def _json_line(out):
    return json.loads(next(l for l in out.splitlines() if l.startswith("{")))


def test_golden_deck_parses_alike(driver, golden, tmp_path):
    d = str(tmp_path / "inputs")
    _write_deck(d, golden["param_in"], golden["mat_in"], golden["system_in"])
    rc, out = _dump(driver, d)
    assert rc == 0, out
    param, prob = inputs.read_all_files(golden["param_in"], golden["mat_in"], golden["system_in"])
    _compare(_json_line(out), param, prob)


PARAM_B = """  IVERB = 1 ! a comment = with an equals sign
  ntime = 7
  time_step = 1.0d-13   ! Fortran exponent
  freq = 2.5D3
  icattaneo = 1
  isteady = 0
  power_in = 3e-6
  T_System = 290.5
  T_Bath = 300
  kappaBound = 149
  Periodic = xy
  CG_dir = +z
  T_BathCG = 12.5
  BR = 0.75
  heattime = 4
  _RunName = deckB
  _WriteToTxt = .True.
  write_every = 3
  start_ix = 2
  end_ix = 3
"""
MAT_B = """1
heat_capacity = 710
h_conv = 0
kappa = 149
kappa3D = 149
rho = 2329
sound_speed = 8433
tau = 1d-12
em = 0.1
0
2
heat_capacity = 1500.
h_conv = 0
kappa = .2
kappa3D = 0.2
rho = 1153
sound_speed = 100
tau = 0
em = 0
0
"""


def _system(nx, ny, nz, cells):
    lines = [f"{nx} {ny} {nz}", f"{nx * 1e-9} {ny * 1e-9} {nz * 1e-9}"]
    it = iter(cells)
    for _ in range(nz):
        lines.append("")
        for _ in range(ny):
            lines.append(" ".join(next(it) for _ in range(nx)))
    return "\n".join(lines) + "\n"


def _cells(n, seed):
    rng = np.random.default_rng(seed)
    mats = rng.choice(["1", "2", "310", "340"], n)
    heat = rng.choice(["0", "0", "0", "1", "5"], n)
    return [f"{m}:{h}" for m, h in zip(mats, heat)]


@pytest.mark.parametrize("dims", [(4, 3, 2), (5, 2, 3)])
def test_synthetic_deck_parses_alike(driver, tmp_path, dims):
    """Periodic axes, a Neumann face with T_BathCG, kappaBound filling the six faces, BR, Fortran
    d exponents, comments, built-in materials 310 and 340, heaters."""
    system = _system(*dims, _cells(int(np.prod(dims)), sum(dims)))
    d = str(tmp_path / "inputs")
    _write_deck(d, PARAM_B, MAT_B, system)
    rc, out = _dump(driver, d)
    assert rc == 0, out
    param, prob = inputs.read_all_files(PARAM_B, MAT_B, system)
    js = _json_line(out)
    _compare(js, param, prob)
    assert js["periodic"] == [1, 1, 0] and js["cg_face"] == [0, 0, 0, 0, 0, 1]
    assert js["kappa_bound"] == [149.0] * 6 and js["t_bath_cg"] == 12.5


@pytest.mark.parametrize("edit,message", [
    (lambda p: p + "ntime = 9\n", "ERROR: same KEYWORD apears more than once"),
    (lambda p: p.replace("  kappaBound = 149\n", "").replace("Periodic = xy", "Periodic = x"),
     "ERROR: KappaBoundx,y,z and KappaBound are not set"),
])
def test_input_errors_stop_like_the_reference(driver, tmp_path, edit, message):
    system = _system(2, 2, 2, ["1:0"] * 8)
    param = edit(PARAM_B)
    d = str(tmp_path / "inputs")
    _write_deck(d, param, MAT_B, system)
    rc, out = _dump(driver, d)
    assert rc == 1 and message in out
    with pytest.raises(inputs.InputError, match=re.escape(message)):
        inputs.read_all_files(param, MAT_B, system)


def test_missing_deck_file(driver, tmp_path):
    rc, out = _dump(driver, str(tmp_path / "nowhere"))
    assert rc == 1 and "Error cannot find file: param.in" in out


def test_unknown_material_stops(driver, tmp_path):
    system = _system(2, 1, 1, ["1:0", "77:0"])
    d = str(tmp_path / "inputs")
    _write_deck(d, PARAM_B, MAT_B, system)
    rc, out = _dump(driver, d)
    assert rc == 1 and "Error: imaterial_type not recognized: 77" in out
