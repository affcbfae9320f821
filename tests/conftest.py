import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built backend")


def gpu_available():
    try:
        from quest_gb300 import _lib
        import ctypes
        n = ctypes.c_int(0)
        _lib.lib().qg_get_num_devices(ctypes.byref(n))
        return n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def built_lib():
    """The backend library, built in-tree if it is missing (nvcc cross-compiles without a GPU)."""
    from quest_gb300 import build
    return build.build()


@pytest.fixture(scope="session")
def env(built_lib):
    """An initialised QuEST environment on cuda:0 (GPU tests only)."""
    from quest_gb300 import api
    api.init_env()
    return api
