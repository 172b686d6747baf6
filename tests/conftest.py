import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through the engine's C-ABI)")


@pytest.fixture(scope="session", autouse=True)
def built():
    import __graft_entry__
    __graft_entry__.build()
    yield


def gpu_available() -> bool:
    import ctypes
    try:
        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        try:
            import glob
            cands = glob.glob("/usr/local/cuda/lib64/libcudart.so*")
            rt = ctypes.CDLL(cands[0])
        except Exception:
            return False
    n = ctypes.c_int(0)
    return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
