"""Sub-box log: file naming (last_log, mod_output.f90:199-213) and record format round trip."""
import numpy as np

from heatflow_gb300.output import format_record, next_log_name, parse_records


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
