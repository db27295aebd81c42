"""Host-buffer steps queued without host round trips (hf_step_host_async / hf_host_sync): a caller
that feeds back the results it downloads gets the bits of an uninterrupted hf_run (the stored
products H T^n, H T^(n-1) survive an input equal to the device's state; such calls start early,
from the device's copy, while their uploads travel), on one grid and on a batch, with torch-pinned
and with registered host arrays; a changed input drops the products as hf_set_state does; an
input changed while queued under an early start is caught by the check of the uploaded bits and
the queue runs again from there; pageable arrays and calls while steps are queued are refused."""
import ctypes as C

import numpy as np
import pytest

from heatflow_gb300 import abi
from heatflow_gb300.problem import layered_slab, point_source_cube, random_instance
from heatflow_gb300.solver import HeatFlow

pytestmark = pytest.mark.gpu

KW = dict(precision="mixed", criterion="true", tol=1e-10, use_graph=1)


def _pinned(n, fill):
    torch = pytest.importorskip("torch")
    return torch.full((n,), fill, dtype=torch.float64).pin_memory().numpy()


def _run_ref(probs, tp, tpp, itime0, K):
    """An uninterrupted run from a host-written state."""
    with HeatFlow(probs, **KW) as hf:
        hf.set_state(tp, tpp)
        st = hf.run(itime0, K)
        T, Tp = hf.get_state()
        return T, Tp, st["inner_iterations"]


def _run_async(hf, bufs, itime0, K, rot=(0, 1, 2)):
    cur, prev, free = rot
    for k in range(K):
        hf.step_host_async(itime0 + k, bufs[cur], bufs[prev], bufs[free])
        cur, prev, free = free, cur, prev
    return hf.host_sync(), (cur, prev, free)


def _initial(probs):
    with HeatFlow(probs, **KW) as hf:
        hf.initial_evolve()
        hf.run(1, 2)
        return hf.get_state()


def test_async_equals_uninterrupted_run(cuda_lib):
    prob = layered_slab(16, nz=20, layer=5)
    tp, tpp = _initial(prob)
    T_ref, Tp_ref, iters = _run_ref(prob, tp, tpp, 3, 7)
    bufs = [_pinned(prob.ncells, 0.0) for _ in range(3)]
    bufs[0][:] = tp
    bufs[1][:] = tpp
    with HeatFlow(prob, **KW) as hf:
        st, (cur, prev, _) = _run_async(hf, bufs, 3, 7)
    assert np.array_equal(bufs[cur], T_ref) and np.array_equal(bufs[prev], Tp_ref)
    assert st["steps"] == 7 and st["inner_iterations"] == iters and st["unconverged"] == 0


def test_async_step_accepted_at_first_residual(cuda_lib):
    """The result of a host-buffer step is stored by the step's last residual sweep; a step
    accepted at its first residual (x = x0, no sweep of an updated x) gets it from the fallback
    copy after the solve: the bits of an uninterrupted run either way."""
    prob = layered_slab(16, nz=20, layer=5)
    kw = dict(KW, tol=1e-1)
    tp, tpp = _initial(prob)
    with HeatFlow(prob, **kw) as hf:
        hf.set_state(tp, tpp)
        st = hf.run(3, 5)
        T_ref, Tp_ref = hf.get_state()
    assert st["inner_iterations"] == 0 and st["refinements"] == 5
    bufs = [_pinned(prob.ncells, 0.0) for _ in range(3)]
    bufs[0][:] = tp
    bufs[1][:] = tpp
    with HeatFlow(prob, **kw) as hf:
        st2, (cur, prev, _) = _run_async(hf, bufs, 3, 5)
    assert st2["inner_iterations"] == 0 and st2["refinements"] == 5
    assert np.array_equal(bufs[cur], T_ref) and np.array_equal(bufs[prev], Tp_ref)


def test_async_products_used_and_dropped(cuda_lib):
    """Fed-back inputs keep the products (the first residual is pointwise from the third step on);
    a changed input makes the next two steps use the stencil, like a fresh context."""
    prob = layered_slab(16, nz=20, layer=5)
    tp, tpp = _initial(prob)
    bufs = [_pinned(prob.ncells, 0.0) for _ in range(3)]
    bufs[0][:] = tp
    bufs[1][:] = tpp
    kw = dict(KW, use_graph=3)
    with HeatFlow(prob, **kw) as hf:
        rot = (0, 1, 2)
        first = []
        for k in range(4):
            _, rot = _run_async(hf, bufs, 3 + k, 1, rot)
            first.append(hf.solve_profile()[0][0][0])
        assert first == ["res_init", "res_init", "res_init_hx", "res_init_hx"], first
        cur, prev, free = rot
        bufs[cur][123] += 1e-3                      # the caller changes the state
        T0, Tp0 = bufs[cur].copy(), bufs[prev].copy()
        _, rot = _run_async(hf, bufs, 7, 3, rot)
        assert hf.solve_profile()[0][0][0] == "res_init_hx"
        T = bufs[rot[0]].copy()
    T_ref, _, _ = _run_ref(prob, T0, Tp0, 7, 3)
    assert np.array_equal(T, T_ref)


def test_async_batch_registered(cuda_lib):
    probs = [point_source_cube(12), layered_slab(8, nz=10, layer=3)]
    tp, tpp = _initial(probs)
    T_ref, Tp_ref, _ = _run_ref(probs, tp, tpp, 3, 5)
    bufs = [np.zeros(tp.size) for _ in range(3)]
    lib = abi.load_library()
    for b in bufs:
        assert lib.hf_host_register(b.ctypes.data_as(C.c_void_p), b.nbytes) == abi.HF_OK
    try:
        bufs[0][:] = tp
        bufs[1][:] = tpp
        with HeatFlow(probs, **KW) as hf:
            _, (cur, prev, _) = _run_async(hf, bufs, 3, 5)
        assert np.array_equal(bufs[cur], T_ref) and np.array_equal(bufs[prev], Tp_ref)
    finally:
        for b in bufs:
            lib.hf_host_unregister(b.ctypes.data_as(C.c_void_p))


@pytest.mark.parametrize("use_graph", [1, 3])
def test_async_batch_many_chunks(cuda_lib, use_graph):
    """Uneven grids whose z-slabs of tasks fill the 8 upload chunks unevenly: chunks that hold
    several grids and a tall grid spread over several chunks.  Each chunk's RHS runs as it lands;
    the result is the uninterrupted run's, bit for bit."""
    rng = np.random.default_rng(11)
    probs = [random_instance(rng, lo=6, hi=40) for _ in range(12)]
    probs.append(layered_slab(40, nz=70, layer=7))
    kw = dict(KW, use_graph=use_graph)
    with HeatFlow(probs, **kw) as hf:
        hf.initial_evolve()
        hf.run(1, 2)
        tp, tpp = hf.get_state()
    with HeatFlow(probs, **kw) as hf:
        hf.set_state(tp, tpp)
        hf.run(3, 4)
        T_ref, Tp_ref = hf.get_state()
    bufs = [_pinned(tp.size, 0.0) for _ in range(3)]
    bufs[0][:] = tp
    bufs[1][:] = tpp
    with HeatFlow(probs, **kw) as hf:
        st, (cur, prev, _) = _run_async(hf, bufs, 3, 4)
    assert st["unconverged"] == 0
    assert np.array_equal(bufs[cur], T_ref) and np.array_equal(bufs[prev], Tp_ref)


def test_async_nan_input_reported(cuda_lib):
    """A NaN in the T^n handed to the second queued step: hf_host_sync reports the reference's
    Cattaneo NaN error (mod_evolve.f90 stops there) and the state is left unrotated, as a
    synchronous step leaves it."""
    prob = point_source_cube(6, icattaneo=1)
    tp, tpp = _initial(prob)
    bufs = [_pinned(prob.ncells, 0.0) for _ in range(4)]
    bufs[0][:] = tp
    bufs[1][:] = tpp
    bad = bufs[3]
    bad[:] = tp
    bad[7] = np.nan
    with HeatFlow(prob, **KW) as hf:
        hf.step_host_async(3, bufs[0], bufs[1], bufs[2])
        hf.step_host_async(4, bad, bufs[2], bufs[1])
        with pytest.raises(abi.HeatFlowError) as e:
            hf.host_sync()
        assert e.value.code == abi.HF_ENAN_SCAT
        after, _ = hf.get_state()
    assert np.isnan(after[7]) and np.isfinite(np.delete(after, 7)).all()


def test_pageable_arrays_refused(cuda_lib):
    prob = point_source_cube(8)
    with HeatFlow(prob, **KW) as hf:
        a = np.full(prob.ncells, 300.0)
        with pytest.raises(abi.HeatFlowError) as e:
            hf.step_host_async(1, a, a.copy(), a.copy())
        assert e.value.code == abi.HF_EARG


def test_calls_refused_while_queued(cuda_lib):
    prob = point_source_cube(10)
    bufs = [_pinned(prob.ncells, 300.0) for _ in range(3)]
    with HeatFlow(prob, **KW) as hf:
        hf.step_host_async(1, bufs[0], bufs[1], bufs[2])
        table = np.array([[250.0, 100.0, 2000.0, 700.0], [350.0, 120.0, 2000.0, 700.0]])
        for call in (hf.get_state, hf.operator, hf.step_timeline, hf.solve_profile,
                     lambda: hf.set_property_tables([table], np.zeros(prob.ncells, np.int32))):
            with pytest.raises(abi.HeatFlowError) as e:
                call()
            assert e.value.code == abi.HF_ESTATE
        st = hf.host_sync()
        assert st["steps"] == 1
        T, Tp = hf.get_state()
        assert np.array_equal(T, bufs[2]) and np.array_equal(Tp, bufs[0])


def test_async_inputs_in_any_order(cuda_lib):
    """Inputs need not rotate: T^(n-1) may be the download of two calls back after a step whose
    T^n came from another array (here a fresh copy with the same bits).  Every upload from an
    array that a queued step downloads into waits for that download; the download targets start
    as NaN, so an upload that ran early would surface as a NaN error or a changed field."""
    prob = layered_slab(48, nz=40, layer=8)
    tp, tpp = _initial(prob)
    K = 8
    with HeatFlow(prob, **KW) as hf:
        hf.set_state(tp, tpp)
        ref = []
        for k in range(K):
            hf.run(3 + k, 1)
            ref.append(hf.get_state()[0])
    n = prob.ncells
    outs = [_pinned(n, np.nan) for _ in range(K)]
    fresh = [_pinned(n, 0.0) for _ in range(K)]
    a, b = _pinned(n, 0.0), _pinned(n, 0.0)
    a[:] = tp
    b[:] = tpp
    with HeatFlow(prob, **KW) as hf:
        for k in range(K):
            if k == 0:
                tn = a
            elif k % 2:                       # T^n from an array no step downloads into
                fresh[k][:] = ref[k - 1]
                tn = fresh[k]
            else:                             # T^n: the previous download
                tn = outs[k - 1]
            # T^(n-1): the download of two calls back (from k = 2 on)
            tnm1 = b if k == 0 else (a if k == 1 else outs[k - 2])
            hf.step_host_async(3 + k, tn, tnm1, outs[k])
        st = hf.host_sync()
    assert st["steps"] == K and st["unconverged"] == 0
    for k in range(K):
        assert np.array_equal(outs[k], ref[k]), k


@pytest.mark.parametrize("n,cell", [(16, 5), (16, 16 * 16 * 19 + 40), (15, 7)])
def test_early_start_checked_against_uploads(cuda_lib, n, cell):
    """The second call's T^(n-1) is the first call's T^n array, which the caller changes after the
    first call (breaking the rule that queued arrays stay untouched): the second and third calls
    start early from the device's copy, the check of the uploaded bits finds the difference, and
    hf_host_sync runs both again from their uploaded inputs.  The results equal steps run from
    those inputs with hf_set_state.  The changed cell lies in the bottom slab, in the heated top
    slab, and on a grid whose rows are not 4k cells."""
    torch = pytest.importorskip("torch")
    prob = layered_slab(n, nz=20, layer=5)
    tp, tpp = _initial(prob)
    a, b, c, d, e = (_pinned(prob.ncells, 0.0) for _ in range(5))
    a[:] = tp
    b[:] = tpp
    with HeatFlow(prob, **KW) as hf:
        hf.step_host_async(3, a, b, c)          # T^n = a, T^(n-1) = b -> c
        torch.cuda.synchronize()                # every copy of the first call has landed
        a[cell] += 0.25                         # the caller changes a queued array
        hf.step_host_async(4, c, a, d)          # the rotation: starts early from the device copy
        hf.step_host_async(5, d, c, e)
        st = hf.host_sync()
    assert st["steps"] == 3
    with HeatFlow(prob, **KW) as ref:
        ref.set_state(c, a)                     # the second call's uploaded inputs
        ref.run(4, 1)
        d_ref, _ = ref.get_state()
        ref.set_state(d_ref, c)
        ref.run(5, 1)
        e_ref, _ = ref.get_state()
    assert np.array_equal(d, d_ref) and np.array_equal(e, e_ref)
