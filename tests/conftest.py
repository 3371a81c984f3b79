import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); runs the kernels through the C ABI")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    return oracle.load()


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if stale) and loads libsdem_gpu.so; the GPU tests run only through it."""
    from sdem_gb300 import build, capi
    build.build()
    return capi.load()
