"""The K2 block-width autotuner (csrc/tune.cu) never changes results: the
zeta sums are exact integers whatever the blocking, so sessions are identical
with the tuned widths and with the fixed heuristic (BGT_GB300_TUNE=0)."""
import os

import numpy as np
import pytest

import bayesiangrouptesting_gb300 as bgt
from bayesiangrouptesting_gb300.serve import SessionRequest, serve_all

pytestmark = pytest.mark.gpu


def _session(n, seed):
    rng = np.random.default_rng(seed)
    pi0 = rng.uniform(0.01, 0.15, n)
    truth = int(rng.integers(0, 1 << n))
    lat = bgt.Lattice(bgt.LatticeType.replicated_dilution, n, pi0)
    out = lat.run_session(10, truth, seed=seed, selector=bgt.SelectorType.op_bbpa, alpha=0.01)
    return out, lat.posterior()


@pytest.mark.parametrize("n", [9, 15, 19])
def test_tuned_widths_do_not_change_sessions(gpu, n, monkeypatch):
    monkeypatch.setenv("BGT_GB300_TUNE", "0")
    fixed, post_fixed = _session(n, 100 + n)
    monkeypatch.setenv("BGT_GB300_TUNE", "1")
    tuned, post_tuned = _session(n, 100 + n)
    for key in ("experiments", "responses", "pos", "neg"):
        np.testing.assert_array_equal(fixed[key], tuned[key])
    np.testing.assert_array_equal(post_fixed, post_tuned)


def test_tuned_widths_do_not_change_served_sessions(gpu, monkeypatch):
    rng = np.random.default_rng(7)
    reqs = []
    for i in range(12):
        n = int(rng.integers(8, 19))
        reqs.append(SessionRequest(n, rng.uniform(0.01, 0.15, n), int(rng.integers(0, 1 << n)), 7, i,
                                   dilution=bool(i % 2), alpha=0.01 if i % 2 else 0.99))
    monkeypatch.setenv("BGT_GB300_TUNE", "0")
    a = serve_all(reqs, memory_budget=1 << 30)
    monkeypatch.setenv("BGT_GB300_TUNE", "1")
    b = serve_all(reqs, memory_budget=1 << 30)
    for x, y in zip(a, b):
        assert x.stages == y.stages
        np.testing.assert_array_equal(x.experiments, y.experiments)
        np.testing.assert_array_equal(x.neg_masks, y.neg_masks)
