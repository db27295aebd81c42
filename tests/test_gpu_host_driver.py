"""The C++ host program runs the reference's test deck end to end on the GPU: ./inputs read,
10 steps, ./outputs/TempDis.dat and TempDisTPD.dat in final_print's layout, and the sub-box log
output_<RunName>_00 with data_write's records: one when the log opens after step 1 and, with
_WriteToTxt, one every write_every steps (mod_output.f90:79-113), so step 1 twice at write_every 1."""
import os
import subprocess

import numpy as np
import pytest

from heatflow_gb300 import inputs
from heatflow_gb300.build import build_driver, build_library
from heatflow_gb300.output import parse_records
from heatflow_gb300.solver import HeatFlow

pytestmark = pytest.mark.gpu


def test_driver_runs_the_golden_deck(cuda_lib, golden, tmp_path):
    build_library()
    drv = build_driver()
    work = tmp_path / "run"
    (work / "inputs").mkdir(parents=True)
    for key, name in (("param_in", "param.in"), ("mat_in", "mat.in"), ("system_in", "system.in")):
        (work / "inputs" / name).write_text(golden[key])
    r = subprocess.run([drv], cwd=work, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all done" in r.stdout
    param, prob = inputs.read_all_files(golden["param_in"], golden["mat_in"], golden["system_in"])
    n = prob.ncells
    T = inputs.parse_temp_file((work / "outputs" / "TempDis.dat").read_text(), n)
    gold = np.asarray(golden["tempdis"])
    assert np.linalg.norm(T - gold) / np.linalg.norm(gold) < 1.1e-9
    # the same library through Python: identical fields, identical file text
    with HeatFlow(prob, precision="fp64", criterion="recursive", tol=1e-32) as hf:
        hf.initial_evolve()
        states = []
        for k in range(1, param["ntime"] + 1):
            hf.run(k, 1)
            states.append(hf.get_state())
    Tp, Tpp = states[-1]
    assert (work / "outputs" / "TempDis.dat").read_text() == inputs.format_temp_file(Tp)
    assert (work / "outputs" / "TempDisTPD.dat").read_text() == inputs.format_temp_file(Tpp)
    # the log: T^(n-1) after each logged step over the 25 x 25 x 1 box, at time (itime-1) dt;
    # write_every = 1 with _WriteToTxt: step 1 is logged twice, then every step
    recs = parse_records((work / "outputs" / "output_IntRun_00").read_text())
    marks = [1] + list(range(1, param["ntime"] + 1))
    assert len(recs) == param["ntime"] + 1 == 11
    assert r.stdout.count("Writing Temperature difference to file") == param["ntime"]
    for k, (t, vals) in zip(marks, recs):
        assert t == float(np.float32((k - 1) * param["time_step"]))
        assert np.allclose(vals, states[k - 1][1], rtol=1e-15, atol=0)


def test_driver_chunks_steps_between_records(cuda_lib, golden, tmp_path):
    """IVERB 1 and write_every 3: the program runs the steps between records as whole-loop graph
    launches and copies the records while the next steps run; the records (after steps 1, 3, 6,
    9) and the final fields are those of the per-step path."""
    build_library()
    drv = build_driver()
    param_in = golden["param_in"].replace("IVERB = 6", "IVERB = 1").replace(
        "write_every = 1", "write_every = 3")
    work = tmp_path / "run"
    (work / "inputs").mkdir(parents=True)
    (work / "inputs" / "param.in").write_text(param_in)
    (work / "inputs" / "mat.in").write_text(golden["mat_in"])
    (work / "inputs" / "system.in").write_text(golden["system_in"])
    r = subprocess.run([drv], cwd=work, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    param, prob = inputs.read_all_files(param_in, golden["mat_in"], golden["system_in"])
    assert param["write_every"] == 3 and param["IVERB"] == 1
    with HeatFlow(prob, precision="fp64", criterion="recursive", tol=1e-32) as hf:
        hf.initial_evolve()
        states = []
        for k in range(1, param["ntime"] + 1):
            hf.run(k, 1)
            states.append(hf.get_state())
    recs = parse_records((work / "outputs" / "output_IntRun_00").read_text())
    marks = [1, 3, 6, 9]
    assert len(recs) == len(marks)
    for (t, vals), k in zip(recs, marks):
        assert t == float(np.float32((k - 1) * param["time_step"]))
        assert np.array_equal(vals, states[k - 1][1])
    assert (work / "outputs" / "TempDis.dat").read_text() == inputs.format_temp_file(states[-1][0])
