"""Python host mirror of the reference's hot-path interface, over the C ABI.

``HeatFlow`` owns one device context (one grid, or a batch of independent grids) and exposes
the reference's routines under their reference names:

==========================  ===========================================================
reference                   here
==========================  ===========================================================
set_global_variables +      ``HeatFlow(problem)`` (mod_setup.f90:34-83, 89-152)
sparse_Hmatrix
initial_evolve              ``initial_evolve()`` / ``set_state`` (mod_init_evolve.f90:34-51)
simulate(itime)             ``simulate(itime)`` (mod_evolve.f90:45-177)
the time loop               ``run(itime0, nsteps)`` (heatflow.f90:67-90)
linbcg                      ``linbcg(b, x)`` (mod_Sparse.f90:372-434)
atimes / SRSax              ``atimes(x)`` (mod_Sparse.f90:436-450, 293-315)
boundary / heater / S_catS  ``rhs(itime)`` (mod_boundary.f90:24, mod_heating.f90:27,
                            mod_cattaneo.f90:23)
sparse_Hmatrix COO          ``sparse_hmatrix()``
==========================  ===========================================================

Errors raise :class:`heatflow_gb300.abi.HeatFlowError` carrying the reference's message (the
reference writes it and executes ``stop 1``).
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence, Union

import numpy as np

from . import abi
from .problem import Problem

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int64)


def _d(a):
    return a.ctypes.data_as(_dp)


def make_opts(precision="fp64", criterion="recursive", tol=None, itmax=50000, inner_tol=1e-4,
              inner_itmax=200, max_refine=20, check_every=2, use_graph=0,
              task_depth=0) -> abi.HfSolverOpts:
    lib = abi.load_library()
    o = abi.HfSolverOpts()
    lib.hf_default_opts(C.byref(o))
    o.precision = {"fp64": abi.HF_PREC_FP64, "mixed": abi.HF_PREC_MIXED}[precision]
    o.criterion = {"recursive": abi.HF_STOP_RECURSIVE, "true": abi.HF_STOP_TRUE}[criterion]
    if tol is None:
        tol = 1e-32 if criterion == "recursive" else 1e-10
    o.tol = tol
    o.itmax = itmax
    o.inner_tol = inner_tol
    o.inner_itmax = inner_itmax
    o.max_refine = max_refine
    o.check_every = check_every
    o.use_graph = use_graph
    o.task_depth = task_depth
    return o


class HeatFlow:
    def __init__(self, problems: Union[Problem, Sequence[Problem]], library=None, **opts):
        """library: the loaded CUDA library to run on (default: abi.load_library(); the tests
        pass the index-checked build, abi.load_library(checked=True))."""
        self.lib = library or abi.load_library()
        self.problems = [problems] if isinstance(problems, Problem) else list(problems)
        self.opts = make_opts(**opts)
        arr = (abi.HfProblem * len(self.problems))(*[p.to_c() for p in self.problems])
        self._arr = arr
        h = C.c_void_p()
        self._check(self.lib.hf_create_batch(arr, len(self.problems), C.byref(self.opts), C.byref(h)),
                  "hf_create")
        self.h = h
        self.sizes = [p.ncells for p in self.problems]
        self.n = sum(self.sizes)

    def _check(self, code: int, where: str):
        abi.check(code, where, self.lib)

    def index_checks(self, probe: bool = False):
        """(enabled, record) of the index checks: enabled is True in the checked build; record =
        [failed checks, site of the first, its index, the extent]; the record is cleared."""
        en = C.c_int32()
        rec = (C.c_int64 * 4)()
        self._check(self.lib.hf_index_checks(self.h, int(probe), C.byref(en), rec), "hf_index_checks")
        return bool(en.value), list(rec)

    def close(self):
        if getattr(self, "h", None):
            self.lib.hf_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream_handle: int):
        """Run on an existing CUDA stream (cudaStream_t as an integer, e.g. torch's
        ``stream.cuda_stream``); 0 returns to the context's own stream."""
        self._check(self.lib.hf_set_stream(self.h, C.c_void_p(stream_handle or None)), "hf_set_stream")

    def time_kernel(self, kernel: int, reps: int = 20) -> float:
        """Mean duration (ms) of one launch of a step kernel, CUDA-event timed."""
        ms = C.c_double()
        self._check(self.lib.hf_time_kernel(self.h, int(kernel), int(reps), C.byref(ms)), "hf_time_kernel")
        return ms.value

    def solve_profile(self, cap: int = 512):
        """Rounds of the last persistent solve: [(phase name, microseconds), ...] and the total
        number of rounds (the per-round list stops at 512)."""
        rounds = C.c_int64()
        ph = (C.c_int32 * cap)()
        us = (C.c_double * cap)()
        self._check(self.lib.hf_solve_profile(self.h, cap, C.byref(rounds), ph, us), "hf_solve_profile")
        n = min(rounds.value, cap, 512)
        return [(abi.PHASE_NAMES.get(ph[i], str(ph[i])), us[i]) for i in range(n)], rounds.value

    def step_timeline(self):
        """Microseconds of the latest step: step begin -> RHS, RHS -> its finalize, finalize ->
        persistent solve, solve (to the end of its last round), -> step end (None where absent)."""
        us = (C.c_double * 5)()
        self._check(self.lib.hf_step_timeline(self.h, us), "hf_step_timeline")
        keys = ("begin_to_rhs", "rhs", "finalize", "solve", "solve_to_end")
        return {k: (us[i] if us[i] >= 0 else None) for i, k in enumerate(keys)}

    def set_property_tables(self, tables, cell_table):
        """Temperature-dependent properties: `tables` = list of (m, 4) arrays of rows
        (T ascending, kappa, rho, c); `cell_table` = a table index or -1 per cell (all grids, cell
        order).  After every step each such cell takes its properties at its new T^n and the
        operator is rebuilt on the device.  An empty list returns to fixed properties."""
        if not tables:
            self._check(self.lib.hf_set_property_tables(self.h, 0, None, None, None),
                      "hf_set_property_tables")
            return
        offsets = np.cumsum([0] + [len(t) for t in tables]).astype(np.int32)
        rows = np.ascontiguousarray(np.concatenate([np.asarray(t, np.float64) for t in tables]))
        ct = np.ascontiguousarray(cell_table, np.int32)
        assert ct.size == self.n
        self._tables = (offsets, rows, ct)      # the library copies them; keep until the call ends
        self._check(self.lib.hf_set_property_tables(
            self.h, len(tables), offsets.ctypes.data_as(C.POINTER(C.c_int32)), _d(rows),
            ct.ctypes.data_as(C.POINTER(C.c_int32))), "hf_set_property_tables")

    def subbox_async(self, lo, hi, which: int = 1, out=None, instance: int = 0):
        """Start copying the box lo..hi (0-based, inclusive, (x, y, z)) of T^(n-1) (which=1, the
        field the reference logs) or T^n (which=0) into `out` (float64, x fastest; pinned for
        overlap) behind the queued steps.  Returns (ticket, out); `subbox_wait(ticket)` waits."""
        lo = (C.c_int64 * 3)(*[int(v) for v in lo])
        hi = (C.c_int64 * 3)(*[int(v) for v in hi])
        n = int(np.prod([hi[k] - lo[k] + 1 for k in range(3)]))
        if out is None:
            out = np.empty(n)
        assert out.dtype == np.float64 and out.flags.c_contiguous and out.size == n
        t = C.c_int64()
        self._check(self.lib.hf_subbox_async(self.h, int(instance), lo, hi, int(which), _d(out),
                                           C.byref(t)), "hf_subbox_async")
        return t.value, out

    def subbox_wait(self, ticket: int):
        self._check(self.lib.hf_subbox_wait(self.h, int(ticket)), "hf_subbox_wait")

    def autotune(self, itime0: int = 1, steps: int = 3):
        """Choose the task depth (and, mixed, the inner tolerance) by timing `steps` steps of this
        problem per candidate; state and statistics are unchanged.  Returns the candidates."""
        res = (abi.HfTuneResult * 16)()
        n = C.c_int32()
        self._check(self.lib.hf_autotune(self.h, int(itime0), int(steps), res, 16, C.byref(n)),
                  "hf_autotune")
        out = [dict(task_depth=r.task_depth, inner_tol=r.inner_tol, ms_per_step=r.ms_per_step,
                    chosen=bool(r.chosen)) for r in res[:n.value]]
        best = next(r for r in out if r["chosen"])
        self.opts.task_depth = best["task_depth"]
        self.opts.inner_tol = best["inner_tol"]
        return out

    # ---- options
    def set_opts(self, **opts):
        self.opts = make_opts(**opts)
        self._check(self.lib.hf_set_opts(self.h, C.byref(self.opts)), "hf_set_opts")

    # ---- state
    def set_state(self, tp, tpp):
        tp = np.ascontiguousarray(tp, np.float64)
        tpp = np.ascontiguousarray(tpp, np.float64)
        assert tp.size == self.n and tpp.size == self.n
        self._check(self.lib.hf_set_state(self.h, _d(tp), _d(tpp)), "hf_set_state")

    def initial_evolve(self):
        """Temp_p = Temp_pp = T_System (mod_init_evolve.f90:47-48)."""
        t = np.concatenate([np.full(p.ncells, p.t_system) for p in self.problems])
        self.set_state(t, t)

    def get_state(self, out=None):
        """(T^n, T^(n-1)) in cell order; `out` = two contiguous float64 arrays to fill (e.g.
        pinned host buffers, which the copies then reach without staging); an entry of `out` that
        is None is not read back."""
        if out is None:
            out = (np.empty(self.n), np.empty(self.n))
        for a in out:
            if a is not None:
                assert a.dtype == np.float64 and a.flags.c_contiguous and a.size == self.n
        tp, tpp = out
        self._check(self.lib.hf_get_state(self.h, _d(tp) if tp is not None else None,
                                        _d(tpp) if tpp is not None else None), "hf_get_state")
        return tp, tpp

    def split(self, a):
        out, pos = [], 0
        for s in self.sizes:
            out.append(a[pos:pos + s])
            pos += s
        return out

    # ---- stepping
    def simulate(self, itime: int) -> dict:
        st = abi.HfStats()
        self._check(self.lib.hf_step(self.h, int(itime), C.byref(st)), "simulate")
        return st.as_dict()

    def run(self, itime0: int, nsteps: int) -> dict:
        st = abi.HfStats()
        self._check(self.lib.hf_run(self.h, int(itime0), int(nsteps), C.byref(st)), "run")
        return st.as_dict()

    def step_host_async(self, itime: int, tp, tpp, out):
        """Queue one step from pinned host arrays (tp = T^n, tpp = T^(n-1)) into pinned `out`
        (all float64, total_cells long, kept alive and untouched until host_sync)."""
        for a in (tp, tpp, out):
            assert a.dtype == np.float64 and a.flags.c_contiguous and a.size == self.n
        self._queued = getattr(self, "_queued", []) + [(tp, tpp, out)]
        self._check(self.lib.hf_step_host_async(self.h, int(itime), _d(tp), _d(tpp), _d(out)),
                  "hf_step_host_async")

    def host_sync(self) -> dict:
        st = abi.HfStats()
        self._queued = []
        self._check(self.lib.hf_host_sync(self.h, C.byref(st)), "hf_host_sync")
        return st.as_dict()

    # ---- parity probes
    def operator(self):
        out = [np.empty(self.n) for _ in range(4)]
        self._check(self.lib.hf_get_operator(self.h, *[_d(a) for a in out]), "hf_get_operator")
        return dict(zip(("diag", "cx", "cy", "cz"), out))

    def rhs(self, itime: int):
        out = [np.empty(self.n) for _ in range(6)]
        self._check(self.lib.hf_get_rhs(self.h, int(itime), *[_d(a) for a in out]), "hf_get_rhs")
        return dict(zip(("B", "Q", "Qdens", "S_cat", "S", "x0"), out))

    def atimes(self, x):
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty(self.n)
        self._check(self.lib.hf_apply_operator(self.h, _d(x), _d(y)), "atimes")
        return y

    def linbcg(self, b, x):
        b = np.ascontiguousarray(b, np.float64)
        x = np.array(x, np.float64, copy=True)
        st = abi.HfStats()
        self._check(self.lib.hf_solve(self.h, _d(b), _d(x), C.byref(st)), "linbcg")
        return x, st.as_dict()

    def sparse_hmatrix(self, instance: int = 0):
        ln = C.c_int64()
        self._check(self.lib.hf_assemble_coo(self.h, instance, 0, None, None, None, C.byref(ln), None),
                  "hf_assemble_coo")
        cap = ln.value
        irow = np.empty(cap, np.int64)
        jcol = np.empty(cap, np.int64)
        val = np.empty(cap, np.float64)
        cnt = C.c_int64()
        self._check(self.lib.hf_assemble_coo(self.h, instance, cap, irow.ctypes.data_as(_ip),
                                           jcol.ctypes.data_as(_ip), _d(val), C.byref(ln),
                                           C.byref(cnt)), "hf_assemble_coo")
        return irow, jcol, val, cnt.value


def geometric_to_dense(problem: Problem, op: dict) -> np.ndarray:
    """Expand the geometric SoA operator into a dense matrix (small grids; tests)."""
    nx, ny, nz = problem.nx, problem.ny, problem.nz
    N = problem.ncells
    H = np.diag(op["diag"].copy())
    per = problem.periodic
    for I in range(N):
        x, y, z = I % nx, (I // nx) % ny, I // (nx * ny)
        for a, (c, n, stride, key) in enumerate(((x, nx, 1, "cx"), (y, ny, nx, "cy"),
                                                 (z, nz, nx * ny, "cz"))):
            v = op[key][I]
            if v == 0.0 or n == 1:
                continue
            if c + 1 < n:
                J = I + stride
            elif per[a]:
                J = I - (n - 1) * stride
            else:
                continue
            H[I, J] += v
            H[J, I] += v
    return H
