"""The N > 1 host logic of bench.py on CPU: two gloo ranks (world_size 2, 127.0.0.1).

The path does not shard (one grid per GPU, replicas only): every rank advances its own replica with
no collective on the data path; the ranks meet only in a barrier and a MAX of their timings, and the
whole-job rate sums the replicas.  The replicas here run the oracle on a small grid, so the test
needs no GPU; the reference arm's rule (rank 0 alone runs and prints) is checked too."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    from heatflow_gb300.problem import point_source_cube
    from oracle.oracle import Oracle
    dist.init_process_group("gloo", rank=rank, world_size=world)
    r, w, local = bench.dist_info()
    # the replica: every rank advances the same small grid on its own (no data-path collective)
    prob = point_source_cube(6)
    o = Oracle(prob)
    o.set_state(*prob.initial_state())
    for k in range(3):
        rc, _, _ = o.simulate(k + 1, mode=0, tol=1e-12, itmax=5000)
        assert rc == 0
    T, _ = o.get_state()
    dist.barrier()
    ms_local = 10.0 * (rank + 1)                       # per-rank timings differ
    ms_max = bench.reduce_max(ms_local, dist, "cpu")
    rate = bench.aggregate_rate(w, 4, ms_max)
    # reference arm under torchrun: ranks other than 0 exit 0 without work
    class A:  # the fields run_reference reads before it returns on rank != 0
        n, fourier, steps, warmup, cpu_seconds, tol, gpus = 6, False, 1, 0, 1.0, 1e-10, w
    ref_rc = bench.run_reference(A, r, w) if r != 0 else None
    out.put((r, w, local, ms_max, rate, float(np.abs(T).sum()), float(T.max()), ref_rc))
    dist.destroy_process_group()


def test_two_gloo_ranks_replicas_and_max_timing():
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(out.get(timeout=240) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, w0, l0, m0, rate0, s0, t0, ref0), (r1, w1, l1, m1, rate1, s1, t1, ref1) = res
    assert (r0, r1, w0, w1, l0, l1) == (0, 1, 2, 2, 0, 1)
    assert m0 == m1 == 20.0                             # MAX over ranks, seen by every rank
    assert rate0 == rate1 == pytest.approx(2 * 4 / 0.020)
    assert s0 == s1 and t0 == t1 and t0 > 300.0         # independent replicas, same result
    assert ref1 == 0                                    # reference arm: rank 1 does no work
