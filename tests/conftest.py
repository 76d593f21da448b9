import ctypes
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); parity tests through the C ABI")


def _cuda_device_count() -> int:
    for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
        try:
            rt = ctypes.CDLL(name)
        except OSError:
            continue
        n = ctypes.c_int(0)
        if rt.cudaGetDeviceCount(ctypes.byref(n)) == 0:
            return n.value
        return 0
    return 0


HAVE_GPU = _cuda_device_count() > 0


def pytest_collection_modifyitems(config, items):
    if HAVE_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA device in this machine")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def built():
    """Build libcfgpu.so and the oracle in-tree (no-op when up to date)."""
    from cajitafluids_gb300.build import build_library
    from oracle.build import build_oracle
    build_oracle()
    build_library()
    return True
