import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libmic_gb300.so")


def _has_gpu():
    try:
        import ctypes
        from fvmic2d_gb300 import gpu
        return gpu.load() is not None and ctypes.CDLL("libcuda.so.1") is not None
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    # GPU tests are selected with -m gpu; without a GPU they would fail loudly, which is intended
    pass


@pytest.fixture(scope="session")
def golden_dir():
    return os.path.join(ROOT, "tests", "golden")
