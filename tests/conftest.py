import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU (runs the CUDA path through the C ABI)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


def has_gpu() -> bool:
    try:
        import ctypes

        rt = None
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                rt = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if rt is None:
            return False
        n = ctypes.c_int(0)
        return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def port_lib():
    from oracle.oracle import Port

    return Port.lib()


@pytest.fixture(scope="session")
def gpu_lib():
    from tissuefolding_paperversion_gb300 import api

    return api.load()
