"""Test configuration: the `gpu` marker, import paths and the build step.

CPU tests (-m "not gpu") check the oracle against the golden vectors, the
host logic and that libtfs_gb300.so loads and exports its C ABI; GPU tests
(-m gpu) compare the CUDA path with the oracle on the same seeded systems.
"""
import os
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
for p in (REPO, REPO / "t-flows_gb300"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from tflows import build
    build.build_library()
    build.build_synth()
    build.build_oracle()
    yield


def gpu_available() -> bool:
    import ctypes
    try:
        cudart = ctypes.CDLL("libcudart.so.13")
    except OSError:
        try:
            cudart = ctypes.CDLL("libcudart.so")
        except OSError:
            return False
    n = ctypes.c_int(0)
    return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0


@pytest.fixture(scope="session")
def gpu():
    if not gpu_available():
        pytest.fail("no CUDA device: GPU tests need a GB300")
    return True
