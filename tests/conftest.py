import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _has_gpu():
    try:
        import ctypes
        cudart = None
        for name in ("libcudart.so", "libcudart.so.13", "libcuda.so.1"):
            try:
                cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if cudart is None:
            return False
        if hasattr(cudart, "cuInit"):
            return cudart.cuInit(0) == 0
        n = ctypes.c_int(0)
        return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def lib():
    """The product library (built on demand)."""
    from fmd_gb300 import load
    from fmd_gb300.build import build_libfmd
    build_libfmd()
    return load()


@pytest.fixture(scope="session")
def gpu_lib(lib):
    if not _has_gpu():
        pytest.fail("GPU tests need a CUDA device; none is visible")
    return lib
