"""Lattice.select_experiments (the greedy k-lookahead of
src/core/lattice_api.cpp:116-168) on the device against the oracle's
restatement of the reference's brute force, its unit-test pin, its argument
errors, and at n = 20 against host-side scores of sampled candidates."""
import numpy as np
import pytest

import bayesiangrouptesting_gb300 as bgt

pytestmark = pytest.mark.gpu


def _rev(v, n):
    return int(sum(1 << (n - 1 - i) for i in range(n) if v >> i & 1))


def _public_posterior(post_internal, n):
    idx = np.arange(1 << n, dtype=np.int64)
    rev = np.zeros_like(idx)
    for i in range(n):
        rev |= ((idx >> i) & 1) << (n - 1 - i)
    return post_internal[rev]


def _score(post_pub, n, exps):
    """The reference's score (lattice_api.cpp:145-158), vectorised over public states."""
    states = np.arange(1 << n, dtype=np.int64)
    g = np.zeros(1 << n, dtype=np.int64)
    for i, e in enumerate(exps):
        g |= (((states & e) == states).astype(np.int64)) << i
    mass = np.bincount(g, weights=post_pub, minlength=1 << len(exps))
    return float(np.sum(np.abs(mass - 1.0 / (1 << len(exps)))))


def _assert_lookahead(oracle, post, n, got, want):
    """Equal, or equal up to the first step where the oracle's own scores of
    both candidates differ by <= 1e-12 (a near-tie the reference's rounding
    decides)."""
    assert got[0] == want[0]
    for step in range(1, len(want)):
        if got[step] == want[step]:
            continue
        a = oracle.lookahead_score(post, n, got[:step + 1])
        b = oracle.lookahead_score(post, n, want[:step + 1])
        assert abs(a - b) <= 1e-12 * max(1.0, b), (step, got, want, a, b)
        return


def test_reference_pin(gpu):
    # tests/cpp/unit/lattice_api_test.cpp:75-79.
    lat = bgt.Lattice(bgt.LatticeType.replicated_non_dilution, 2, [0.2, 0.4])
    assert lat.select_experiments(2, bgt.SelectorType.op_bha) == [3, 2]
    assert lat.select_experiments(1, bgt.SelectorType.op_bbpa) == [3]
    assert lat.select_experiments(0) == []
    assert lat.select_experiments(2) == [3, 2]  # default selector: Op-BHA


def test_argument_errors(gpu):
    lat = bgt.Lattice(bgt.LatticeType.replicated_non_dilution, 4, [0.1, 0.2, 0.3, 0.4])
    with pytest.raises(ValueError):
        lat.select_experiments(-1)
    with pytest.raises(ValueError):
        lat.select_experiments(2, bgt.SelectorType.op_bbpa)
    multi = bgt.Lattice(bgt.LatticeType.replicated_non_dilution, 2, [0.1, 0.2, 0.3, 0.4], 2)
    with pytest.raises(ValueError):
        multi.select_experiments(2, bgt.SelectorType.op_bha)
    assert multi.select_experiments(1, bgt.SelectorType.auto_select) == [multi.select_experiment()]
    with pytest.raises(bgt.Error):
        lat.select_experiments(11)


@pytest.mark.parametrize("n,count,dilution", [(3, 3, False), (6, 4, False), (9, 3, True), (11, 3, False),
                                              (12, 2, True),
                                              # 6..10 experiments: 2..32 response groups per lane
                                              (6, 10, False), (8, 8, True), (10, 7, False)])
def test_matches_oracle(gpu, oracle, n, count, dilution):
    rng = np.random.default_rng(900 + n)
    pi0 = rng.uniform(0.02, 0.3, n)
    t = bgt.LatticeType.replicated_dilution if dilution else bgt.LatticeType.replicated_non_dilution
    lat = bgt.Lattice(t, n, pi0)
    table = bgt.api.DilutionTable(n, 0.99, 0.005) if dilution else None
    post = oracle.prior(pi0)
    for _ in range(3):
        e = int(rng.integers(1, 1 << n))
        r = int(rng.integers(0, 2))
        lat.update(e, r, table)
        post = oracle.update(1 if dilution else 0, n, 1, post, _rev(e, n), r, in_place=True)
    got = lat.select_experiments(count)
    want = oracle.select_experiments(post, n, count)
    _assert_lookahead(oracle, post, n, got, want)
    # the lattice is unchanged: selection and a later update still agree
    assert lat.select_experiments(count) == got
    e = int(rng.integers(1, 1 << n))
    lat.update(e, 1, table)
    post = oracle.update(1 if dilution else 0, n, 1, post, _rev(e, n), 1, in_place=True)
    np.testing.assert_allclose(lat.posterior(), post, rtol=1e-12, atol=0)


def test_fp32_lattice(gpu, oracle):
    n = 10
    rng = np.random.default_rng(950)
    pi0 = rng.uniform(0.02, 0.3, n)
    lat = bgt.Lattice(bgt.LatticeType.replicated_non_dilution, n, pi0, precision=bgt.Precision.float32)
    for _ in range(2):
        lat.update(int(rng.integers(1, 1 << n)), int(rng.integers(0, 2)))
    post = lat.posterior()  # the FP32 values the device scores
    _assert_lookahead(oracle, post, n, lat.select_experiments(3), oracle.select_experiments(post, n, 3))


def test_n20_against_sampled_candidates(gpu):
    n = 20
    rng = np.random.default_rng(960)
    pi0 = rng.uniform(0.01, 0.15, n)
    lat = bgt.Lattice(bgt.LatticeType.replicated_non_dilution, n, pi0)
    for _ in range(4):
        lat.update(int(rng.integers(1, 1 << n)), int(rng.integers(0, 2)))
    got = lat.select_experiments(3)
    post_pub = _public_posterior(lat.posterior(), n)
    for step in (1, 2):
        best = _score(post_pub, n, got[:step + 1])
        for cand in rng.integers(1, 1 << n, 64):
            other = _score(post_pub, n, got[:step] + [int(cand)])
            assert best <= other + 1e-12, (step, got, int(cand), best, other)


def _golden():
    import json
    import os
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_vectors.json")
    return json.load(open(path)).get("lookahead", [])


@pytest.mark.parametrize("case", range(len(_golden())))
def test_golden_reference_outputs(gpu, oracle, case):
    # The reference library's own select_experiments outputs (public order).
    c = _golden()[case]
    n = c["n"]
    lat = bgt.Lattice(bgt.LatticeType.replicated_non_dilution, n, c["pi0"])
    post = oracle.prior(c["pi0"])
    for e, r in c["updates"]:
        lat.update(e, r)
        post = oracle.update(0, n, 1, post, _rev(e, n), r, in_place=True)
    _assert_lookahead(oracle, post, n, lat.select_experiments(c["count"]), c["experiments"])
