import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(ROOT, "tests", "golden", "tempdis_25x25.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library on a machine with a GPU (GPU tests only)."""
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from heatflow_gb300.build import build_library
    build_library()
    from heatflow_gb300 import abi
    return abi.load_library()
