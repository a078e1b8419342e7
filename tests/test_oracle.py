"""The CPU oracle (oracle/bgt_oracle.c) pinned against the reference:
its own known-answer tests, golden vectors generated by the reference library
(tests/golden/make_golden.py) and, where the reference library is built in
oracle/_ref, randomized bit-exact cross-checks."""
import json
import os

import numpy as np
import pytest

from oracle.oracle import Reference, reference_available

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = json.load(open(os.path.join(HERE, "golden", "reference_vectors.json")))


def test_known_answers_model(oracle):
    # tests/cpp/unit/model_math_test.cpp:41-62 (internal order).
    np.testing.assert_allclose(oracle.prior([0.2, 0.4]), [0.08, 0.32, 0.12, 0.48], atol=1e-12)
    post = oracle.update(0, 2, 1, oracle.prior([0.2, 0.4]), 1, 1, in_place=False)
    den = 0.08 * 0.01 + 0.32 * 0.99 + 0.12 * 0.01 + 0.48 * 0.99
    np.testing.assert_allclose(post, np.array([0.08 * 0.01, 0.32 * 0.99, 0.12 * 0.01, 0.48 * 0.99]) / den, atol=1e-12)
    dil = oracle.dilution_table(2, 0.99, 0.005)
    assert abs(dil[0, 0] - 0.99) < 1e-12 and abs(dil[0, 1] - 0.01) < 1e-12
    assert abs(dil[1, 0] - 0.99) < 1e-12 and abs(dil[1, 1] - (1.0 - 0.99 / 1.005)) < 1e-12
    assert abs(dil[1, 2] - 0.01) < 1e-12
    # tests/cpp/unit/dilution_test.cpp:11-13 (public order == internal for a full pool).
    assert abs(oracle.response_prob(1, 2, 1, 3, 1, 3) - 0.99) < 1e-12
    assert abs(oracle.response_prob(1, 2, 1, 3, 1, 2) - (1.0 - 0.99 / 1.005)) < 1e-12
    assert abs(oracle.response_prob(1, 2, 1, 3, 0, 2) - 0.99 / 1.005) < 1e-12


def test_known_answers_selection(oracle):
    # tests/cpp/unit/lattice_api_test.cpp:63-91; public state p is internal reverse(p).
    post = oracle.prior([0.2, 0.4])
    rev = {0: 0, 1: 2, 2: 1, 3: 3}
    for e_pub, m in ((1, 0.60), (2, 0.80), (3, 0.48)):
        assert abs(oracle.upset_mass(post, 2, rev[e_pub]) - m) < 1e-12
    for sel in (0, 1, 2):
        assert oracle.select(post, 2, 1, sel) == 3
    post = oracle.update(0, 2, 1, post, rev[1], 1)
    pos, neg = oracle.classify(post, 2, 0.01, 0.01)
    assert pos == 0 and neg == rev[1]


def test_known_answer_single_subject_tree(oracle):
    # tests/cpp/support/assertions.hpp:80-92.
    got = oracle.run_simulation(0, 1, 1, [0.2], 1)
    np.testing.assert_allclose(got, [2, 0.792, 0.002, 0.0, 0.002, 0.206, 1.0, 1.0], atol=1e-12)


@pytest.mark.parametrize("case", range(len(GOLDEN["model"])))
def test_golden_model(oracle, case):
    c = GOLDEN["model"][case]
    n, k, dil = c["n"], c["k"], c["dilution"]
    prior = oracle.prior(c["pi0"])
    np.testing.assert_array_equal(prior, c["prior"])
    np.testing.assert_array_equal(oracle.update(dil, n, k, prior, c["e"], c["r"], in_place=True), c["update_divide"])
    np.testing.assert_array_equal(oracle.update(dil, n, k, prior, c["e"], c["r"], in_place=False),
                                  c["update_multiply"])
    post = np.array(c["update_divide"])
    for sel, want in c["select"].items():
        assert oracle.select(post, n, k, int(sel)) == want
    np.testing.assert_array_equal(oracle.atom_masses(post, n * k), c["atom_masses"])
    assert oracle.classify(post, n * k, c["classify_up"], c["classify_lo"]) == (c["pos"], c["neg"])


@pytest.mark.parametrize("case", range(len(GOLDEN["tree"])))
def test_golden_tree(oracle, case):
    c = GOLDEN["tree"][case]
    got = oracle.run_simulation(c["dilution"], c["n"], c["k"], c["pi0"], c["depth"], c["up"], c["lo"], c["branch"],
                                c["selector"])
    np.testing.assert_array_equal(got, c["stats"])
    # The reference's default build (-ffast-math) agrees within the reference's own tolerance.
    np.testing.assert_allclose(got, c["stats_default_build"], rtol=0, atol=1e-12)


@pytest.mark.parametrize("case", range(len(GOLDEN["session"])))
def test_golden_session(oracle, case):
    c = GOLDEN["session"][case]
    got = oracle.session(c["dilution"], c["n"], 1, c["pi0"], c["stages"], c["seed"], c["session"], c["truth"],
                         selector=c["selector"], alpha=c["alpha"], h=c["h"])
    for key in ("experiments", "responses", "pos", "neg"):
        np.testing.assert_array_equal(got[key], c[key])
    np.testing.assert_array_equal(got["posterior"][:16], c["posterior_head"])
    assert float(np.sum(got["posterior"])) == c["posterior_sum"]


def test_workload_streams_match_host_copies(oracle):
    import bench

    for session in (0, 1, 7, (3 << 32) + 5):
        pi0 = oracle.sample_prior(24, bench.PRIOR_LO, bench.PRIOR_HI, bench.SEED, session)
        np.testing.assert_array_equal(pi0, bench.session_prior(bench.SEED, session))
        assert oracle.sample_truth(pi0, bench.SEED, session) == bench.session_truth(bench.SEED, session, pi0)


@pytest.mark.reference
@pytest.mark.skipif(not reference_available(), reason="reference library not built here (oracle/_ref)")
def test_randomized_bit_exact_against_reference(oracle):
    ref = Reference(strict=True)
    rng = np.random.default_rng(99)
    for trial in range(30):
        k = [1, 1, 2, 3][trial % 4]
        n = {1: int(rng.integers(1, 12)), 2: int(rng.integers(1, 6)), 3: int(rng.integers(1, 4))}[k]
        pi0 = rng.uniform(0.005, 0.3, n * k)
        dil = trial % 2
        post = oracle.prior(pi0)
        np.testing.assert_array_equal(post, ref.prior(pi0, k))
        for _ in range(3):
            e = int(rng.integers(1, 1 << n))
            r = int(rng.integers(0, 1 << k))
            nxt = oracle.update(dil, n, k, post, e, r)
            np.testing.assert_array_equal(nxt, ref.update(dil, n, k, post, e, r))
            post = nxt
        for sel in ((0, 1, 2) if k == 1 else (0, 2)):
            assert oracle.select(post, n, k, sel) == ref.select(post, n, k, sel)
    for (dil, n, depth) in ((0, 7, 5), (1, 8, 4), (0, 9, 3)):
        pi0 = rng.uniform(0.01, 0.2, n)
        np.testing.assert_array_equal(oracle.run_simulation(dil, n, 1, pi0, depth),
                                      ref.run_simulation(dil, n, 1, pi0, depth))


def test_closed_form_upset_masses_match_oracle(oracle):
    # The closed form used for the 27-30 atom device checks, pinned against
    # the oracle's own zeta on small lattices.
    from test_gpu_large import _closed_form_scores

    rng = np.random.default_rng(5)
    for n in (9, 12):
        pi0 = rng.uniform(0.01, 0.15, n)
        e0 = int(rng.integers(1, 1 << n))
        post = oracle.update(0, n, 1, oracle.prior(pi0), e0, 1)
        e, upset = oracle.op_bha(post, n)
        l_in = oracle.response_prob(0, n, 1, e0, 1, (1 << n) - 1)
        l_out = oracle.response_prob(0, n, 1, e0, 1, 0)
        best, mass = _closed_form_scores(n, pi0, e0, l_in, l_out)
        np.testing.assert_allclose([mass(x) for x in range(1 << n)], upset, rtol=0, atol=1e-14)
        assert abs(best - abs(2.0 * upset[e] - 1.0)) <= 1e-14


def test_host_response_stream_matches_oracle(oracle):
    # The benchmark's host copy of the response stream (its per-call Lattice
    # API loop) draws what the device sessions and the oracle draw.
    import bench

    rng = np.random.default_rng(3)
    for t in range(500):
        n = int(rng.integers(2, 20))
        e, s = int(rng.integers(0, 1 << n)), int(rng.integers(0, 1 << n))
        dil = bool(rng.integers(0, 2))
        alpha = 0.01 if dil else 0.99
        want = oracle.lib.orc_sample_response(1 if dil else 0, n, 1, e, s, alpha, 0.005, 7, t, t % 40)
        assert bench.session_response(dil, n, e, s, alpha, 0.005, 7, t, t % 40) == want


def test_test_accuracy_extension(oracle):
    # Non-dilution accuracy other than the reference's 0.99 / 0.99: the same
    # formula with specificity (contained pool) and sensitivity (a pooled
    # positive); the context restores the reference model.
    e, full, partial = 3, 3, 2  # internal order, n = 2: pool {0, 1}
    base = [oracle.response_prob(0, 2, 1, e, r, s) for r in (0, 1) for s in (full, partial)]
    with oracle.test_accuracy(0.95, 0.98):
        assert abs(oracle.response_prob(0, 2, 1, e, 1, full) - 0.98) < 1e-15
        assert abs(oracle.response_prob(0, 2, 1, e, 0, full) - (1 - 0.98)) < 1e-15
        assert abs(oracle.response_prob(0, 2, 1, e, 0, partial) - 0.95) < 1e-15
        assert abs(oracle.response_prob(0, 2, 1, e, 1, partial) - (1 - 0.95)) < 1e-15
        # two variants multiply their factors
        s = full | (partial << 2)
        assert abs(oracle.response_prob(0, 2, 2, e, 0b01, s) - 0.98 * 0.95) < 1e-15
        # dilution lattices keep their table
        assert abs(oracle.response_prob(1, 2, 1, 3, 1, 3) - 0.99) < 1e-12
    assert [oracle.response_prob(0, 2, 1, e, r, s) for r in (0, 1) for s in (full, partial)] == base
    # 0.99 / 0.99 set explicitly is the reference model bit for bit
    pi0 = [0.1, 0.2, 0.3, 0.05]
    want = oracle.run_simulation(0, 4, 1, pi0, 3, branch=1e-4)
    with oracle.test_accuracy(0.99, 0.99):
        np.testing.assert_array_equal(oracle.run_simulation(0, 4, 1, pi0, 3, branch=1e-4), want)
    with oracle.test_accuracy(0.95, 0.98):
        assert np.max(np.abs(oracle.run_simulation(0, 4, 1, pi0, 3, branch=1e-4) - want)) > 1e-6


def _rev(v, n):
    return int(sum(1 << (n - 1 - i) for i in range(n) if v >> i & 1))


def test_lookahead_pin(oracle):
    # tests/cpp/unit/lattice_api_test.cpp:75-79: select_experiments(2, op_bha) on
    # the prior {0.2, 0.4} is [3, 2] (public order).
    assert oracle.select_experiments(oracle.prior([0.2, 0.4]), 2, 2) == [3, 2]
    assert oracle.select_experiments(oracle.prior([0.2, 0.4]), 2, 1) == [3]
    assert oracle.select_experiments(oracle.prior([0.2, 0.4]), 2, 0) == []


@pytest.mark.skipif(not reference_available(), reason="reference library not built here (oracle/_ref)")
def test_lookahead_bit_exact_against_reference(oracle):
    ref = Reference(strict=True)
    assert ref.select_experiments([0.2, 0.4], [], 2) == [3, 2]
    rng = np.random.default_rng(31)
    for n, count in ((3, 3), (5, 3), (7, 3), (8, 4)):
        pi0 = rng.uniform(0.02, 0.3, n)
        updates = [(int(rng.integers(1, 1 << n)), int(rng.integers(0, 2))) for _ in range(3)]
        post = oracle.prior(pi0)
        for e, r in updates:
            post = oracle.update(0, n, 1, post, _rev(e, n), r, in_place=True)
        assert oracle.select_experiments(post, n, count) == ref.select_experiments(pi0, updates, count), (n, updates)


@pytest.mark.parametrize("case", range(len(GOLDEN.get("lookahead", []))))
def test_golden_lookahead(oracle, case):
    # select_experiments outputs of the reference library (tests/golden/make_golden.py).
    c = GOLDEN["lookahead"][case]
    n = c["n"]
    post = oracle.prior(c["pi0"])
    for e, r in c["updates"]:
        post = oracle.update(0, n, 1, post, _rev(e, n), r, in_place=True)
    assert oracle.select_experiments(post, n, c["count"]) == c["experiments"]


def test_session_sampler_test_accuracy(oracle):
    # bgt_session_sample_response (include/bgt_session_rng.h) under a
    # non-dilution accuracy: bit v set (negative) when the stream's uniform
    # is below specificity for a contained pool, below 1 - sensitivity else.
    rng = np.random.default_rng(12)
    for sens, spec in ((0.95, 0.98), (0.99, 0.99), (0.7, 0.6)):
        with oracle.test_accuracy(sens, spec):
            for t in range(200):
                n, k = int(rng.integers(1, 8)), int(rng.integers(1, 4))
                e = int(rng.integers(1, 1 << n))
                s = int(rng.integers(0, 1 << (n * k)))
                want = 0
                for v in range(k):
                    sv = (s >> (v * n)) & ((1 << n) - 1)
                    p1 = spec if (e & sv) == e else 1.0 - sens
                    if oracle.lib.orc_uniform(9, t, 3, (t % 40) * 64 + v) < p1:
                        want |= 1 << v
                assert oracle.lib.orc_sample_response(0, n, k, e, s, 0.99, 0.005, 9, t, t % 40) == want
