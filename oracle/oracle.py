"""ORACLE — test infrastructure only.  ctypes wrapper of oracle/hf_oracle.c, the plain-C
restatement of the HeatFlow reference's hot path (see the header of hf_oracle.c for the
citations and the fixtures it is pinned against).  Used by tests/, __graft_entry__.smoke() and
bench.py's CPU baseline legs; never by the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int64)
_lib = None


def build(force: bool = False) -> str:
    srcs = [os.path.join(HERE, f) for f in ("hf_oracle.c", "cpu_pcg.c", "Makefile")]
    if force or not os.path.exists(LIB) or any(os.path.getmtime(LIB) < os.path.getmtime(p) for p in srcs):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        from heatflow_gb300.abi import HfProblem
        L = C.CDLL(LIB)
        L.or_create.restype = C.c_void_p
        L.or_create.argtypes = [C.POINTER(HfProblem)]
        L.or_destroy.argtypes = [C.c_void_p]
        L.or_num_cells.restype = C.c_int64
        L.or_num_cells.argtypes = [C.c_void_p]
        L.or_coo.restype = C.c_int64
        L.or_coo.argtypes = [C.c_void_p, _ip, _ip, _dp, _ip]
        L.or_set_state.argtypes = [C.c_void_p, _dp, _dp]
        L.or_get_state.argtypes = [C.c_void_p, _dp, _dp]
        L.or_boundary.argtypes = [C.c_void_p, _dp]
        L.or_heater.argtypes = [C.c_void_p, C.c_int64, _dp, _dp, _dp]
        L.or_cattaneo.argtypes = [C.c_void_p, _dp, _dp, _dp]
        L.or_rhs.restype = C.c_int
        L.or_rhs.argtypes = [C.c_void_p, C.c_int64, _dp, _dp, _dp, _dp, _dp, _dp]
        L.or_atimes.argtypes = [C.c_void_p, _dp, _dp, C.c_int]
        L.or_linbcg.restype = C.c_int
        L.or_linbcg.argtypes = [C.c_void_p, _dp, _dp, C.c_int, C.c_double, C.c_int64, _ip, _dp]
        L.or_pcg.restype = C.c_int
        L.or_pcg.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_int64, _ip, _dp]
        L.or_true_relres.restype = C.c_double
        L.or_true_relres.argtypes = [C.c_void_p, _dp, _dp]
        L.or_simulate.restype = C.c_int
        L.or_simulate.argtypes = [C.c_void_p, C.c_int64, C.c_int, C.c_double, C.c_int64, _ip, _dp]
        L.or_set_property_tables.restype = C.c_int
        L.or_set_property_tables.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), _dp,
                                             C.POINTER(C.c_int32)]
        L.or_set_threads.restype = C.c_int
        L.or_set_threads.argtypes = [C.c_int]
        L.or_geometric.argtypes = [C.c_void_p, _dp, _dp, _dp, _dp]
        L.cp_create.restype = C.c_void_p
        L.cp_create.argtypes = [C.c_void_p, C.c_int64, C.c_int64, C.c_int64,
                                C.POINTER(C.c_int32), C.c_int]
        L.cp_destroy.argtypes = [C.c_void_p]
        L.cp_step.restype = C.c_int
        L.cp_step.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_double, C.c_int64, _ip, _dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


class Oracle:
    """One reference grid: module state after set_global_variables + sparse_Hmatrix."""

    def __init__(self, problem):
        self.problem = problem
        self._cp = problem.to_c()
        self.h = lib().or_create(C.byref(self._cp))
        if not self.h:
            raise ValueError("grid not representable by the reference (COO capacity overflow)")
        self.n = problem.ncells

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().or_destroy(h)
            self.h = None

    # --- state
    def set_property_tables(self, tables, cell_table):
        """tables: list of (m, 4) arrays of rows (T, kappa, rho, c); cell_table: per cell."""
        offsets = np.cumsum([0] + [len(t) for t in tables]).astype(np.int32)
        rows = np.ascontiguousarray(np.concatenate([np.asarray(t, np.float64) for t in tables]))
        ct = np.ascontiguousarray(cell_table, np.int32)
        lib().or_set_property_tables(self.h, len(tables), offsets.ctypes.data_as(C.POINTER(C.c_int32)),
                                     _d(rows), ct.ctypes.data_as(C.POINTER(C.c_int32)))

    def set_state(self, tp, tpp):
        tp = np.ascontiguousarray(tp, np.float64)
        tpp = np.ascontiguousarray(tpp, np.float64)
        lib().or_set_state(self.h, _d(tp), _d(tpp))

    def get_state(self):
        tp = np.empty(self.n)
        tpp = np.empty(self.n)
        lib().or_get_state(self.h, _d(tp), _d(tpp))
        return tp, tpp

    # --- operator
    def coo(self):
        cap = C.c_int64()
        lib().or_coo(self.h, None, None, None, C.byref(cap))
        irow = np.empty(cap.value, np.int64)
        jcol = np.empty(cap.value, np.int64)
        val = np.empty(cap.value, np.float64)
        count = lib().or_coo(self.h, irow.ctypes.data_as(_ip), jcol.ctypes.data_as(_ip), _d(val),
                             C.byref(cap))
        return irow, jcol, val, int(count)

    def dense(self):
        irow, jcol, val, _ = self.coo()
        H = np.zeros((self.n, self.n))
        for i, j, v in zip(irow, jcol, val):
            if 0 < i <= self.n:
                H[i - 1, j - 1] += v
        return H

    def atimes(self, x, transpose=False):
        x = np.ascontiguousarray(x, np.float64)
        y = np.empty(self.n)
        lib().or_atimes(self.h, _d(x), _d(y), int(transpose))
        return y

    # --- RHS
    def boundary(self):
        B = np.zeros(self.n)
        lib().or_boundary(self.h, _d(B))
        return B

    def heater(self, itime, tp):
        tp = np.ascontiguousarray(tp, np.float64)
        Q = np.zeros(self.n)
        Qd = np.zeros(self.n)
        lib().or_heater(self.h, int(itime), _d(tp), _d(Q), _d(Qd))
        return Q, Qd

    def cattaneo(self, tp, tpp):
        tp = np.ascontiguousarray(tp, np.float64)
        tpp = np.ascontiguousarray(tpp, np.float64)
        s = np.zeros(self.n)
        lib().or_cattaneo(self.h, _d(tp), _d(tpp), _d(s))
        return s

    def rhs(self, itime):
        out = [np.zeros(self.n) for _ in range(6)]
        rc = lib().or_rhs(self.h, int(itime), *[_d(a) for a in out])
        return rc, dict(zip(("B", "Q", "Qdens", "S_cat", "S", "x0"), out))

    # --- solve / step
    def linbcg(self, b, x, tol=1e-32, itmax=50000, itol=1):
        b = np.ascontiguousarray(b, np.float64)
        x = np.array(x, np.float64, copy=True)
        it = C.c_int64()
        err = C.c_double()
        lib().or_linbcg(self.h, _d(b), _d(x), itol, tol, itmax, C.byref(it), C.byref(err))
        return x, it.value, err.value

    def pcg(self, b, x, tol=1e-13, itmax=100000):
        b = np.ascontiguousarray(b, np.float64)
        x = np.array(x, np.float64, copy=True)
        it = C.c_int64()
        rel = C.c_double()
        lib().or_pcg(self.h, _d(b), _d(x), tol, itmax, C.byref(it), C.byref(rel))
        return x, it.value, rel.value

    def true_relres(self, b, x):
        b = np.ascontiguousarray(b, np.float64)
        x = np.ascontiguousarray(x, np.float64)
        return lib().or_true_relres(self.h, _d(b), _d(x))

    def simulate(self, itime, mode=0, tol=1e-32, itmax=50000):
        it = C.c_int64()
        err = C.c_double()
        rc = lib().or_simulate(self.h, int(itime), int(mode), float(tol), int(itmax),
                               C.byref(it), C.byref(err))
        return rc, it.value, err.value

    def run(self, nsteps, itime0=1, **kw):
        iters = []
        for k in range(nsteps):
            rc, it, _ = self.simulate(itime0 + k, **kw)
            if rc:
                return rc, iters
            iters.append(it)
        return 0, iters


def set_threads(n: int) -> int:
    return lib().or_set_threads(int(n))


class CleanPCG:
    """The clean CPU solver of oracle/cpu_pcg.c (a second CPU baseline, not the reference's
    algorithm): stencil Jacobi-PCG in FP64 to a true relative residual, OpenMP, on the state of an
    Oracle, whose RHS it uses."""

    def __init__(self, oracle: "Oracle", threads: int = 0):
        p = oracle.problem
        self.o = oracle
        per = (C.c_int32 * 3)(*[int(v) for v in p.periodic])
        self.h = lib().cp_create(oracle.h, p.nx, p.ny, p.nz, per, int(threads or os.cpu_count() or 1))
        if not self.h:
            raise MemoryError("cp_create failed")

    def __del__(self):
        if getattr(self, "h", None):
            lib().cp_destroy(self.h)
            self.h = None

    def step(self, itime: int, tol: float = 1e-10, itmax: int = 100000):
        it = C.c_int64()
        rel = C.c_double()
        rc = lib().cp_step(self.h, self.o.h, int(itime), float(tol), int(itmax), C.byref(it), C.byref(rel))
        return rc, it.value, rel.value
