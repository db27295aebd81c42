"""Sub-box log: file naming (last_log, mod_output.f90:199-213), record format round trip, and
data_write's record cadence (mod_output.f90:79-113) in the Python mirror and in the C++ host
program (its --dump-log-schedule stops before any GPU call)."""
import json
import subprocess

import numpy as np
import pytest

from heatflow_gb300.output import format_record, next_log_name, parse_records, records_after


def test_next_log_name(tmp_path):
    assert next_log_name(str(tmp_path), "run") == str(tmp_path / "output_run_00")
    (tmp_path / "output_run_00").write_text("")
    (tmp_path / "output_run_01").write_text("")
    assert next_log_name(str(tmp_path), "run") == str(tmp_path / "output_run_02")


def test_record_round_trip():
    rng = np.random.default_rng(0)
    vals = 300.0 + rng.standard_normal(17)
    line = format_record(3 * 1e-13, vals)
    (t, back), = parse_records(line)
    assert np.float32(t) == np.float32(3e-13)    # single precision, as real() gives
    assert np.array_equal(back, vals)          # 17 significant digits round-trip FP64


def _schedule(ntime, write_every, write_to_txt=True, test_run=False):
    return [(k, records_after(k, write_every, write_to_txt, test_run)) for k in range(1, ntime + 1)
            if records_after(k, write_every, write_to_txt, test_run)]


def test_record_cadence_rule():
    # write_every = 1 (the reference's test deck): the opening record of step 1 plus the
    # _WriteToTxt record of every step -> 11 records over 10 steps
    assert sum(n for _, n in _schedule(10, 1)) == 11
    assert _schedule(10, 1)[0] == (1, 2)
    # write_every = 3: step 1 (opening), then 3, 6, 9
    assert _schedule(10, 3) == [(1, 1), (3, 1), (6, 1), (9, 1)]
    # without _WriteToTxt only the opening record; test runs write no log
    assert _schedule(10, 1, write_to_txt=False) == [(1, 1)]
    assert _schedule(10, 1, test_run=True) == []


@pytest.fixture(scope="module")
def driver():
    from heatflow_gb300.build import build_driver, build_library
    build_library()
    return build_driver()


@pytest.mark.parametrize("write_every,write_to_txt,test_run", [
    (1, True, False), (3, True, False), (4, False, False), (1, True, True), (2, True, False)])
def test_host_program_record_cadence(driver, golden, tmp_path, write_every, write_to_txt, test_run):
    param = golden["param_in"].replace("write_every = 1", f"write_every = {write_every}")
    param = param.replace("_WriteToTxt = .True.", f"_WriteToTxt = .{write_to_txt}.")
    param = param.replace("_Test_Run = .False.", f"_Test_Run = .{test_run}.")
    d = tmp_path / "inputs"
    d.mkdir()
    (d / "param.in").write_text(param)
    (d / "mat.in").write_text(golden["mat_in"])
    (d / "system.in").write_text(golden["system_in"])
    r = subprocess.run([driver, "--inputs", str(d), "--dump-log-schedule"], capture_output=True,
                       text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    got = [tuple(x) for x in json.loads(r.stdout.strip().splitlines()[-1])]
    assert got == _schedule(golden["ntime"], write_every, write_to_txt, test_run)
