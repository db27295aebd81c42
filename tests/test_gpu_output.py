"""Sub-box snapshots copied on a second stream while the steps continue: the logged records equal
the fields read synchronously from an identical run."""
import numpy as np
import pytest

from heatflow_gb300.output import SubboxLog, parse_records
from heatflow_gb300.problem import layered_slab
from heatflow_gb300.solver import HeatFlow

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("use_graph,write_every,marks", [
    (0, 4, (1, 4, 8, 12)), (1, 4, (1, 4, 8, 12)),
    # write_every 1: the opening record and the _WriteToTxt record both at step 1
    (1, 1, (1,) + tuple(range(1, 15)))])
def test_subbox_log_matches_synchronous_reads(cuda_lib, tmp_path, use_graph, write_every, marks):
    prob = layered_slab(40, nz=36, layer=6)
    lo, hi = (3, 5, 30), (20, 9, 35)
    kw = dict(precision="mixed", criterion="true", tol=1e-10, use_graph=use_graph)
    path = tmp_path / "output_run_00"
    with HeatFlow(prob, **kw) as hf:
        hf.initial_evolve()
        st = SubboxLog(hf, lo, hi, write_every=write_every, path=str(path),
                       time_step=prob.time_step).run(1, 14)
    assert st == {"steps": 14, "records": len(marks)}
    recs = parse_records(path.read_text())
    want = {}
    with HeatFlow(prob, **kw) as h2:
        h2.initial_evolve()
        for k in range(1, 15):
            h2.simulate(k)
            if k in marks:
                _, tpp = h2.get_state()
                box = tpp.reshape(prob.nz, prob.ny, prob.nx)[lo[2]:hi[2] + 1, lo[1]:hi[1] + 1,
                                                              lo[0]:hi[0] + 1]
                want[k] = box.ravel()
    assert [np.float32(r[0]) for r in recs] == [np.float32((k - 1) * prob.time_step)
                                                for k in marks]
    for (t, vals), k in zip(recs, marks):
        assert np.array_equal(vals, want[k]), k
