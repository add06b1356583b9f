"""Shared test setup: marker registration, import paths, in-tree build."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "meso-lts_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); run with -m gpu")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds the library and the oracle in-tree if needed (incremental)."""
    import build

    build.build_library()
    build.build_oracle()
    build.build_apps()
    yield


def has_gpu() -> bool:
    """Asks the CUDA runtime directly (no framework in between)."""
    import ctypes

    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            continue
    else:
        return False
    n = ctypes.c_int(0)
    return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0


@pytest.fixture
def gpu():
    if not has_gpu():
        pytest.fail("a gpu-marked test ran on a machine without a CUDA device")
    return True
