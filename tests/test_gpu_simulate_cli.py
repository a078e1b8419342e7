"""bgt_simulate on the device, end to end: the reference's own e2e runs of
the command (CMakeLists.txt:518-529, with --provider cuda), the single-subject
golden (tests/cpp/support/assertions.hpp:80-92), a seeded tree against the
oracle, and the progress files."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _cli(*args):
    proc = subprocess.run([sys.executable, "-m", "bayesiangrouptesting_gb300.simulate", *map(str, args)],
                          capture_output=True, text=True, cwd=REPO, timeout=300)
    return proc


def _csv(path):
    lines = open(path).read().splitlines()
    assert lines[0] == "field,value"
    return dict(line.split(",", 1) for line in lines[1:])


def test_reference_e2e_scalar_prior(gpu, tmp_path):
    p = _cli("--subjects", 3, "--variants", 1, "--prior", 0.02, "--lattice", "replicated_non_dilution",
             "--mode", "local_tree", "--search-depth", 5, "--provider", "cuda", "--selector", "op_bbpa",
             "--threshold-up", 0.01, "--threshold-lo", 0.01, "--branch-threshold", 0.001, "--write-csv",
             "--output-dir", tmp_path, "--run-name", "bgt-simulate-scalar-prior")
    assert p.returncode == 0, p.stderr
    text = open(tmp_path / "bgt-simulate-scalar-prior.csv").read()
    assert "total_leaves,11" in text
    assert p.stdout.startswith("mode=0 provider=2 status=0 total_states=8 evaluated_states=8 evaluated_prior_mass=1 leaves=11")
    assert f"report={tmp_path}/bgt-simulate-scalar-prior.csv" in p.stdout


def test_reference_e2e_report_single_subject(gpu, tmp_path):
    p = _cli("--subjects", 1, "--prior", 0.2, "--provider", "cuda", "--write-csv", "--output-dir", tmp_path,
             "--run-name", "bgt-simulate-e2e")
    assert p.returncode == 0, p.stderr
    rows = _csv(tmp_path / "bgt-simulate-e2e.csv")
    assert rows["status"] == "completed" and rows["is_partial"] == "false" and rows["provider"] == "2"
    assert rows["total_states"] == "2" and rows["evaluated_states"] == "2" and rows["state_coverage_fraction"] == "1"
    want = {"total_leaves": "2", "correct_probability": "0.792", "incorrect_probability": "0.002",
            "false_positive_probability": "0", "false_negative_probability": "0.002",
            "unclassified_probability": "0.206", "expected_stages": "1", "expected_tests": "1"}
    for k, v in want.items():
        assert rows[k] == v, (k, rows[k])


def test_cli_matches_oracle(gpu, oracle, tmp_path):
    rng = np.random.default_rng(5)
    pi0 = rng.uniform(0.01, 0.15, 8)
    p = _cli("--subjects", 8, "--prior", ",".join(repr(float(x)) for x in pi0), "--lattice", "replicated_dilution",
             "--search-depth", 4, "--dilution-alpha", 0.05, "--dilution-h", 0.01, "--provider", "cuda",
             "--write-csv", "--output-dir", tmp_path, "--run-name", "seeded")
    assert p.returncode == 0, p.stderr
    rows = _csv(tmp_path / "seeded.csv")
    want = oracle.run_simulation(1, 8, 1, pi0, 4, alpha=0.05, h=0.01)
    keys = ["total_leaves", "correct_probability", "incorrect_probability", "false_positive_probability",
            "false_negative_probability", "unclassified_probability", "expected_stages", "expected_tests"]
    got = np.array([float(rows[k]) for k in keys])
    assert got[0] == want[0]
    np.testing.assert_allclose(got[1:], want[1:], rtol=1e-5, atol=1e-6)  # the report prints six digits


def test_progress_files(gpu, tmp_path):
    prog = tmp_path / "run.progress.json"
    p = _cli("--subjects", 6, "--prior", 0.05, "--search-depth", 3, "--provider", "cuda", "--progress",
             "--progress-file", prog)
    assert p.returncode == 0, p.stderr
    assert f"progress={prog}" in p.stdout
    assert "bgt progress: status=running evaluated=0/64" in p.stderr
    assert "bgt progress: status=completed evaluated=64/64" in p.stderr
    final = json.loads(open(prog).read())
    assert final["status"] == "completed" and final["evaluated_states"] == 64 and final["message"] == "completed"
    hist = [json.loads(x) for x in open(tmp_path / "run.progress.jsonl").read().splitlines()]
    assert [h["status"] for h in hist] == ["running", "completed"]
    assert hist[0]["message"] == "starting CUDA evaluation"


def test_runtime_and_cuda_provider(gpu):
    import bayesiangrouptesting_gb300 as bgt
    cfg = bgt.SimulationConfig(subjects=1, prior=[0.2], options=bgt.SimulationOptions(provider=bgt.Provider.cuda))
    res = bgt.Runtime().run_simulation(cfg)
    assert res.kernel.provider == bgt.Provider.cuda and res.kernel.selector == bgt.SelectorType.op_bha
    np.testing.assert_allclose(res.stats.as_array(), [2, 0.792, 0.002, 0.0, 0.002, 0.206, 1.0, 1.0], atol=1e-12)
    st = bgt.CudaProvider().run(bgt.LatticeType.replicated_dilution, 2, 1, [0.2, 0.4], bgt.SimulationOptions(),
                                bgt.DilutionTable(2, 0.99, 0.005))
    want = bgt.run_simulation(bgt.SimulationConfig(lattice_type=bgt.LatticeType.replicated_dilution, subjects=2,
                                                   prior=[0.2, 0.4])).stats
    np.testing.assert_allclose(st.as_array(), want.as_array(), atol=0)
