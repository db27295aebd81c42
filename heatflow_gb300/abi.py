"""ctypes mirror of include/heatflow_gb300.h and the loader of the CUDA library.

The library is built in-tree (``heatflow_gb300/_build/libheatflow_gb300.so``) by
``heatflow_gb300.build.build_library()``.  Loading fails loudly when it is missing: there is no
CPU fallback for the hot path.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
HEADER = os.path.join(REPO, "include", "heatflow_gb300.h")
LIB_PATH = os.path.join(HERE, "_build", "libheatflow_gb300.so")

# status codes (heatflow_gb300.h)
HF_OK, HF_EARG, HF_ECUDA, HF_ENOMEM, HF_ESTATE, HF_EDEVICE = 0, 1, 2, 3, 4, 5
HF_ENAN_B, HF_ENAN_Q, HF_ENAN_QDENS, HF_ENAN_SCAT, HF_ENAN_S, HF_ENAN_X = 10, 11, 12, 13, 14, 15
HF_PREC_FP64, HF_PREC_MIXED = 0, 1
HF_STOP_RECURSIVE, HF_STOP_TRUE = 0, 1
HF_QDENS_HEATED_VOLUME, HF_QDENS_CELL_VOLUME = 0, 1

# The reference's fatal messages (src/heatflow/mod_evolve.f90:70-158), keyed by status code.
REFERENCE_MESSAGES = {
    HF_ENAN_B: "fatal error: NAN in B vector",
    HF_ENAN_Q: "fatal error: NAN in Q vector",
    HF_ENAN_QDENS: "fatal error: NAN in Qdens vector",
    HF_ENAN_SCAT: "fatal error: NAN in S_CAT vector",
    HF_ENAN_S: "fatal error: NAN in S vector",
    HF_ENAN_X: "fatal error: NAN in x tempurature vector",
}

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int64)


class HfProblem(C.Structure):
    _fields_ = [
        ("nx", C.c_int64), ("ny", C.c_int64), ("nz", C.c_int64),
        ("lx", C.c_double), ("ly", C.c_double), ("lz", C.c_double),
        ("kappa", _dp), ("rho", _dp), ("heat_capacity", _dp), ("tau", _dp), ("em", _dp),
        ("iheater", _ip), ("power", _dp),
        ("power_in", C.c_double), ("freq", C.c_double), ("time_step", C.c_double),
        ("heated_steps", C.c_int64),
        ("icattaneo", C.c_int32), ("isteady", C.c_int32),
        ("periodic", C.c_int32 * 3), ("cg_face", C.c_int32 * 6),
        ("kappa_bound", C.c_double * 6), ("t_bath_face", C.c_double * 6),
        ("t_bath", C.c_double), ("t_bath_cg", C.c_double), ("br", C.c_double),
        ("qdens_mode", C.c_int32), ("reserved", C.c_int32),
    ]


class HfSolverOpts(C.Structure):
    _fields_ = [
        ("precision", C.c_int32), ("criterion", C.c_int32), ("tol", C.c_double),
        ("itmax", C.c_int64), ("inner_tol", C.c_double), ("inner_itmax", C.c_int32),
        ("max_refine", C.c_int32), ("check_every", C.c_int32), ("use_graph", C.c_int32),
        ("task_depth", C.c_int32),
    ]


class HfTuneResult(C.Structure):
    _fields_ = [("task_depth", C.c_int32), ("chosen", C.c_int32), ("inner_tol", C.c_double),
                ("ms_per_step", C.c_double)]


class HfStats(C.Structure):
    _fields_ = [
        ("steps", C.c_int64), ("iterations", C.c_int64), ("inner_iterations", C.c_int64),
        ("refinements", C.c_int64), ("last_iter", C.c_int64), ("last_err", C.c_double),
        ("last_true_relres", C.c_double), ("unconverged", C.c_int64),
        ("failed_step", C.c_int64), ("status", C.c_int32), ("failed_instance", C.c_int32),
        ("kernel_launches", C.c_int64),
    ]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


def header_functions(path: str = HEADER) -> list[str]:
    """Names of the functions declared in the public header."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(hf_[a-z0-9_]+)\s*\(",
                       text, flags=re.M)
    return sorted(set(names))


_SIGNATURES = {
    "hf_abi_version": (C.c_int, []),
    "hf_strerror": (C.c_char_p, [C.c_int]),
    "hf_last_error": (C.c_char_p, []),
    "hf_default_opts": (None, [C.POINTER(HfSolverOpts)]),
    "hf_create": (C.c_int, [C.POINTER(HfProblem), C.POINTER(HfSolverOpts), C.POINTER(C.c_void_p)]),
    "hf_create_batch": (C.c_int, [C.POINTER(HfProblem), C.c_int64, C.POINTER(HfSolverOpts),
                                  C.POINTER(C.c_void_p)]),
    "hf_destroy": (C.c_int, [C.c_void_p]),
    "hf_set_opts": (C.c_int, [C.c_void_p, C.POINTER(HfSolverOpts)]),
    "hf_get_sizes": (C.c_int, [C.c_void_p, _ip, _ip]),
    "hf_instance_cells": (C.c_int64, [C.c_void_p, C.c_int64]),
    "hf_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hf_set_state": (C.c_int, [C.c_void_p, _dp, _dp]),
    "hf_get_state": (C.c_int, [C.c_void_p, _dp, _dp]),
    "hf_state_device": (C.c_int, [C.c_void_p, C.POINTER(_dp), C.POINTER(_dp)]),
    "hf_state_device_ready": (C.c_int, [C.c_void_p]),
    "hf_step": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(HfStats)]),
    "hf_run": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, C.POINTER(HfStats)]),
    "hf_get_operator": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp]),
    "hf_get_rhs": (C.c_int, [C.c_void_p, C.c_int64, _dp, _dp, _dp, _dp, _dp, _dp]),
    "hf_apply_operator": (C.c_int, [C.c_void_p, _dp, _dp]),
    "hf_solve": (C.c_int, [C.c_void_p, _dp, _dp, C.POINTER(HfStats)]),
    "hf_assemble_coo": (C.c_int, [C.c_void_p, C.c_int64, C.c_int64, _ip, _ip, _dp, _ip, _ip]),
    "hf_time_kernel": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _dp]),
    "hf_measure_fp_rates": (C.c_int, [_dp, _dp]),
    "hf_step_host_async": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "hf_host_sync": (C.c_int, [C.c_void_p, C.c_void_p]),
    "hf_host_register": (C.c_int, [C.c_void_p, C.c_size_t]),
    "hf_host_unregister": (C.c_int, [C.c_void_p]),
    "hf_step_timeline": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "hf_solve_profile": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_int64),
                                   C.POINTER(C.c_int32), _dp]),
    "hf_subbox_async": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                  C.c_int, _dp, C.POINTER(C.c_int64)]),
    "hf_subbox_wait": (C.c_int, [C.c_void_p, C.c_int64]),
    "hf_set_property_tables": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), _dp,
                                         C.POINTER(C.c_int32)]),
    "hf_check_barrier_timeout": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), _dp]),
    "hf_autotune": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.POINTER(HfTuneResult), C.c_int32,
                              C.POINTER(C.c_int32)]),
    "hf_set_state_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hf_residual_noalloc": (C.c_int, [C.c_int64, C.c_int64, C.c_int64, C.POINTER(C.c_int32),
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "hf_get_state_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "hf_solve_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(HfStats)]),
    "hf_adjoint_rhs": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "hf_adjoint_accumulate": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                        C.c_void_p]),
    "hf_index_checks": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.POINTER(C.c_int64)]),
}
HF_KERNEL_RHS, HF_KERNEL_RESIDUAL, HF_KERNEL_CG_P, HF_KERNEL_CG_SPMV, HF_KERNEL_CG_UPDATE = 0, 1, 2, 3, 4
HF_KERNEL_XUPDATE, HF_KERNEL_SOLVE, HF_KERNEL_CG_PQ, HF_KERNEL_RESIDUAL_INIT = 5, 6, 7, 8
(HF_PHASE_IDLE, HF_PHASE_START, HF_PHASE_RES_INIT, HF_PHASE_CG_P, HF_PHASE_CG_Q, HF_PHASE_CG_PQ,
 HF_PHASE_CG_B, HF_PHASE_XUPD, HF_PHASE_RES, HF_PHASE_RES_INIT_HX, HF_PHASE_CG_BX) = range(11)
PHASE_NAMES = {HF_PHASE_IDLE: "idle", HF_PHASE_START: "start", HF_PHASE_RES_INIT: "res_init",
               HF_PHASE_CG_P: "cg_p", HF_PHASE_CG_Q: "cg_q", HF_PHASE_CG_PQ: "cg_pq",
               HF_PHASE_CG_B: "cg_b", HF_PHASE_XUPD: "xupd", HF_PHASE_RES: "res",
               HF_PHASE_RES_INIT_HX: "res_init_hx", HF_PHASE_CG_BX: "cg_bx"}

# the index-checked build of the same library (tests only; built by build_library(checked=True))
CHECKED_LIB_PATH = os.path.join(HERE, "_build", "checked", "libheatflow_gb300_checked.so")
_libs: dict = {}


def load_library(path: str = LIB_PATH, checked: bool = False):
    """Load libheatflow_gb300.so (or, with checked=True, its index-checked build) and declare its
    signatures.  Raises if it is missing."""
    if checked:
        path = CHECKED_LIB_PATH
    if path in _libs:
        return _libs[path]
    if not os.path.exists(path):
        raise RuntimeError(
            f"heatflow_gb300: CUDA library not built ({path}); run "
            "`python -c 'import __graft_entry__ as g; g.build()'` first")
    lib = C.CDLL(path)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    _libs[path] = lib
    return lib


class HeatFlowError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str = ""):
        self.code = code
        msg = REFERENCE_MESSAGES.get(code)
        if msg is None:
            lib = load_library()
            msg = lib.hf_strerror(code).decode()
        super().__init__(f"{where}: {msg}" + (f" ({detail})" if detail else ""))


def check(code: int, where: str, lib=None):
    """Raise HeatFlowError for a failed call; `lib` is the library that made it (its last error)."""
    if code != HF_OK:
        lib = lib or load_library()
        detail = lib.hf_last_error()
        raise HeatFlowError(code, where, detail.decode() if detail else "")
