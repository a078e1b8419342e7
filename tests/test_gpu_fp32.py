"""FP32 posterior storage (BGT_GPU_FP32): exact fixed-point reductions and
FP64 normalisation, thresholds and objective comparison over FP32-stored
values.  The bar is 1e-6 absolute posterior error against the FP64 oracle;
selections agree except where the FP64 scores of the two choices are within
the FP32 error (reported, not exact)."""
import numpy as np
import pytest

import bayesiangrouptesting_gb300 as bgt
from bayesiangrouptesting_gb300.serve import serve_all

pytestmark = pytest.mark.gpu

TOL = 1e-6  # FP32 posterior tolerance against FP64 (absolute, normalised posterior)
GB = 1 << 30


def _score_gap(oracle, post, n, a, b):
    _, upset = oracle.op_bha(post, n)
    return abs(abs(upset[a] - 0.5) - abs(upset[b] - 0.5))


@pytest.mark.parametrize("dilution", [False, True])
def test_fp32_update_sequence_against_oracle(gpu, oracle, dilution):
    rng = np.random.default_rng(320 + dilution)
    n = 14
    pi0 = rng.uniform(0.01, 0.2, n)
    t = bgt.LatticeType.replicated_dilution if dilution else bgt.LatticeType.replicated_non_dilution
    lat = bgt.Lattice(t, n, pi0, precision=bgt.Precision.float32)
    table = bgt.DilutionTable(n, 0.01, 0.005) if dilution else None
    post = oracle.prior(pi0)
    np.testing.assert_allclose(lat.posterior(), post, rtol=0, atol=TOL)
    disagreements = 0
    for step in range(10):
        want = oracle.select(post, n, 1, 1)
        got = bgt.reverse_bits(lat.select_experiment(bgt.SelectorType.op_bha), n)
        if got != want:
            disagreements += 1
            assert _score_gap(oracle, post, n, got, want) <= 10 * TOL
        r = int(rng.integers(0, 2))
        lat.update(bgt.reverse_bits(want, n), r, table)
        post = oracle.update(1 if dilution else 0, n, 1, post, want, r, alpha=0.01)
        err = float(np.max(np.abs(lat.posterior() - post)))
        assert err <= TOL, (step, err)
        lat.update_classification(0.01, 0.01)
        np.testing.assert_allclose(lat.atom_masses(), oracle.atom_masses(post, n), rtol=0, atol=TOL)
    assert disagreements <= 2


def test_fp32_multinomial_updates(gpu, oracle):
    rng = np.random.default_rng(33)
    n, k = 6, 2
    pi0 = rng.uniform(0.02, 0.3, n * k)
    lat = bgt.Lattice(bgt.LatticeType.replicated_dilution, n, pi0, variants=k, precision=bgt.Precision.float32)
    table = bgt.DilutionTable(n, 0.99, 0.005)
    post = oracle.prior(pi0)
    for _ in range(4):
        e = int(rng.integers(1, 1 << n))
        r = int(rng.integers(0, 1 << k))
        lat.update(e, r, table)
        post = oracle.update(1, n, k, post, e, r)
        assert float(np.max(np.abs(lat.posterior() - post))) <= TOL


def test_fp32_session_tracks_fp64(gpu):
    rng = np.random.default_rng(34)
    agree = total = 0
    for trial in range(6):
        n = int(rng.integers(10, 17))
        pi0 = rng.uniform(0.005, 0.15, n)
        truth = int(rng.integers(0, 1 << n))
        f64 = bgt.Lattice(bgt.LatticeType.replicated_dilution, n, pi0)
        f32 = bgt.Lattice(bgt.LatticeType.replicated_dilution, n, pi0, precision=bgt.Precision.float32)
        ref = f64.run_session(12, truth, seed=trial, selector=bgt.SelectorType.op_bbpa, alpha=0.01)
        table = bgt.DilutionTable(n, 0.01, 0.005)
        for e, r in zip(ref["experiments"], ref["responses"]):
            total += 1
            agree += bgt.reverse_bits(f32.select_experiment(bgt.SelectorType.op_bbpa), n) == int(e)
            f32.update(bgt.reverse_bits(int(e), n), int(r), table)
        assert f64.max_abs_diff(f32) <= TOL
    assert agree >= 0.9 * total, (agree, total)


def test_fp32_thirty_atoms_against_fp64(gpu):
    # n = 10 subjects x k = 3 variants: 2^30 states (4 GB FP32, 8 GB FP64).
    rng = np.random.default_rng(35)
    n, k = 10, 3
    pi0 = rng.uniform(0.01, 0.10, n * k)
    f64 = bgt.Lattice(bgt.LatticeType.replicated_non_dilution, n, pi0, variants=k)
    f32 = bgt.Lattice(bgt.LatticeType.replicated_non_dilution, n, pi0, variants=k, precision=bgt.Precision.float32)
    assert f64.max_abs_diff(f32) <= TOL
    for _ in range(3):
        e = f64.select_experiment()  # both lattices take the FP64 choice (agreement: see the benchmark)
        r = int(rng.integers(0, 1 << k))
        f64.update(e, r)
        f32.update(e, r)
    assert f64.max_abs_diff(f32) <= TOL
    np.testing.assert_allclose(f32.atom_masses(), f64.atom_masses(), rtol=0, atol=TOL)


def test_fp32_served_equals_fp32_plain_loop(gpu):
    from test_gpu_serve import _requests

    reqs = _requests(24, seed=36)
    served = serve_all(reqs, memory_budget=GB, fp32=True)
    for i in (0, 7, 23):
        q = reqs[i]
        t = bgt.LatticeType.replicated_dilution if q.dilution else bgt.LatticeType.replicated_non_dilution
        lat = bgt.Lattice(t, q.subjects, q.prior, precision=bgt.Precision.float32)
        plain = lat.run_session_until_classified(40, q.true_state, seed=q.seed, session=q.session,
                                                 alpha=q.alpha, h=q.h)
        assert plain["stages"] == served[i].stages
        np.testing.assert_array_equal(plain["experiments"], served[i].experiments)
        np.testing.assert_array_equal(plain["neg"], served[i].neg_masks)
