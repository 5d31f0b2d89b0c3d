import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libmontegpu.so")


@pytest.fixture(scope="session")
def oracle():
    from tests import oracle_lib

    return oracle_lib.load()


@pytest.fixture(scope="session")
def gpu_lib():
    """libmontegpu loaded with a usable device (GPU tests only)."""
    import ctypes as C

    from casmcode_monte_gb300 import _lib

    L = _lib.lib()
    n = C.c_int()
    if L.mg_device_count(C.byref(n)) != 0 or n.value < 1:
        pytest.fail("GPU test run without a usable CUDA device")
    return L
