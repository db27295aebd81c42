"""The C-ABI library builds for sm_103a, loads, and exports every function of include/*.h."""
import ctypes

from heatflow_gb300 import abi
from heatflow_gb300.build import build_library


def test_exports_every_declared_symbol():
    path = build_library()
    lib = ctypes.CDLL(path)
    names = abi.header_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_host_only_entry_points():
    lib = abi.load_library()
    assert lib.hf_abi_version() == 1
    assert lib.hf_strerror(abi.HF_ENAN_S) == b"fatal error: NAN in S vector"
    o = abi.HfSolverOpts()
    lib.hf_default_opts(ctypes.byref(o))
    assert o.tol == 1e-32 and o.itmax == 50000 and o.precision == abi.HF_PREC_FP64
