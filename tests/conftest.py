import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs through the C ABI on the GPU)")
    config.addinivalue_line("markers", "reference: needs the reference library built in oracle/_ref")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def native_lib():
    from bayesiangrouptesting_gb300.build import build
    from bayesiangrouptesting_gb300 import _native
    build()
    return _native.load()


@pytest.fixture(scope="session")
def gpu(native_lib):
    if not native_lib.bgt_cuda_provider_available():
        pytest.fail("GPU test selected but no CUDA device is available")
    return native_lib
