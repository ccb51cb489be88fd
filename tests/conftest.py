"""Shared fixtures.  GPU tests carry @pytest.mark.gpu; everything else runs on
a CPU-only host."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as entry  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    entry.build()
    return True


@pytest.fixture(scope="session")
def pp(built):
    return entry.load()


@pytest.fixture(scope="session")
def orc(built):
    return entry.load_oracle()


def has_gpu() -> bool:
    try:
        import ctypes
        rt = None
        for name in ("libcudart.so", "libcuda.so.1"):
            try:
                rt = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if rt is None:
            return False
        if hasattr(rt, "cuDeviceGetCount"):
            if rt.cuInit(0) != 0:
                return False
            n = ctypes.c_int(0)
            return rt.cuDeviceGetCount(ctypes.byref(n)) == 0 and n.value > 0
        n = ctypes.c_int(0)
        return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_ctx(pp):
    if not has_gpu():
        pytest.fail("GPU test run without a CUDA device")
    return pp.get_context(0)


# Configurations live in the package (pp.workloads): c0_setup, c1_setup,
# c2_setup, detector_400.
