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


def assert_posterior_close(got, want, updates):
    """Posterior parity with the oracle.

    The shape must agree to 1e-13: got / want is one constant up to the
    per-value rounding of the updates (a few ulp per update).  The constant
    itself is the oracle's own normalisation error: the reference normalises
    by a sequential FP64 sum of N terms (src/core/model/lattice_base.cpp:
    230-244), which drops terms below half an ulp of the running sum and so
    runs low by up to ~1e-11 at 2^26 states, while the device normalises by
    an exact fixed-point total.  So the constant must equal 1 / sum(want),
    with sum(want) taken pairwise (error ~log2(N) ulp), to 2e-13, and the
    device posterior itself must sum to 1 within 1e-13.  The reference's own
    tests use 1e-12 absolute (tests/cpp/support/assertions.hpp:14-19).
    """
    import numpy as np

    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    assert got.shape == want.shape
    nz = want > 1e-250
    ratio = got[nz] / want[nz]
    mid = float(np.median(ratio))
    shape_err = float(np.max(np.abs(ratio - mid))) if ratio.size else 0.0
    assert shape_err <= 1e-13 * max(1, updates), f"posterior shape differs: {shape_err:.3e}"
    want_sum = float(np.sum(want))
    assert abs(mid * want_sum - 1.0) <= 2e-13, (
        f"normalisation {mid!r} differs from the oracle's exact-sum constant {1.0 / want_sum!r}")
    assert abs(float(np.sum(got)) - 1.0) <= 1e-13, f"device posterior sums to {float(np.sum(got))!r}"
    # Values too small to compare by ratio agree absolutely.
    assert float(np.max(np.abs(got[~nz] - want[~nz]), initial=0.0)) <= 1e-250
