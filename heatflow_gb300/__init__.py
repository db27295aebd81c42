"""heatflow_gb300 — GB300 (sm_103a) implementation of HeatFlow's time-stepping hot path.

The product is the CUDA library ``_build/libheatflow_gb300.so`` behind the C ABI declared in
``include/heatflow_gb300.h``; this package holds its Python host mirror (``solver``), the
problem description and synthetic workloads (``problem``), the readers of the reference's input
decks (``inputs``) and the build script (``build``).
"""
from .abi import HeatFlowError, load_library  # noqa: F401
from .problem import Problem  # noqa: F401

__all__ = ["HeatFlow", "Problem", "HeatFlowError", "load_library"]


def __getattr__(name):
    if name == "HeatFlow":
        from .solver import HeatFlow
        return HeatFlow
    raise AttributeError(name)
