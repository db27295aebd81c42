"""bench.py's output lines keep their contract: the keys and types the benchmark lines are read by,
on small grids (our line on the GPU: 64^3, 3 warm-up + 3 timed steps; the reference arm on the
host cores)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _line(args):
    r = subprocess.run([sys.executable, "bench.py", *args], cwd=ROOT, capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


@pytest.mark.gpu
def test_bench_line_contract(cuda_lib):
    d = _line(["--n", "64", "--steps", "3", "--warmup", "3", "--no-cpu-baseline"])
    for k, t in (("metric", str), ("value", float), ("unit", str), ("n_gpus", int),
                 ("steps", int), ("warmup", int), ("ms_per_step", float),
                 ("higher_is_better", bool), ("scaling", str), ("dtype", str), ("data", str),
                 ("config", dict), ("roofline", dict), ("clocks", dict), ("e2e", dict),
                 ("gpu_launches", int)):
        assert isinstance(d[k], t), (k, d.get(k))
    assert "vs_baseline" in d
    assert d["n_gpus"] == 1 and d["steps"] == 3 and d["warmup"] == 3 and d["value"] > 0
    assert d["higher_is_better"] is True and d["scaling"] == "weak"
    r = d["roofline"]
    for k in ("bound", "achieved", "peak", "unit", "frac", "traffic"):
        assert k in r, k
    assert r["bound"] in ("hbm", "tensor") and 0 < r["frac"] < 1.5
    e = d["e2e"]
    for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step"):
        assert k in e, k
    assert e["h2d_bytes_per_step"] == 2 * 8 * 64 ** 3 and e["d2h_bytes_per_step"] == 8 * 64 ** 3
    assert e["value"] > 0
    assert d["gpu_launches"] >= 5 * d["steps"]
    assert {"sm_mhz", "sm_max_mhz", "reasons"} <= set(d["clocks"])
    assert "workload" in d["config"]


@pytest.mark.parametrize("steps,warmup", [(2, 1), (3, 3)])
def test_reference_arm_contract(steps, warmup):
    """The reference arm (the oracle port on the host cores) needs no GPU."""
    d = _line(["--impl", "reference", "--n", "24", "--steps", str(steps), "--warmup", str(warmup)])
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["steps"] == steps and d["warmup"] == warmup
    assert {"value", "unit", "cores", "kind", "sample"} <= set(d["cpu_baseline"])
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
