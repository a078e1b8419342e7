"""The bgt_simulate command line (examples/run_simulation.cpp) and the run
report / progress formats (src/runtime/reporting.cpp:10-45,
src/runtime/progress.cpp:48-80): option parsing, usage and error exits, the
CSV and JSON writers, and a run cancelled before evaluation (no GPU needed)."""
import json
import os

import pytest

import bayesiangrouptesting_gb300 as bgt
from bayesiangrouptesting_gb300 import reporting, simulate


def test_parse_every_option():
    cfg, prior, eprior, want_help = simulate.parse_args([
        "--subjects", "3", "--variants", "2", "--prior", "0.02,0.05", "--evaluation-prior", "0.1",
        "--lattice", "replicated_dilution", "--mode", "local_tree", "--search-depth", "5",
        "--global-tree-depth", "2", "--workload-granularity", "4", "--provider", "cuda", "--selector", "op_bbpa",
        "--true-state-policy", "trimmed", "--trim-percent", "0.5", "--threshold-up", "0.02", "--threshold-lo", "0.03",
        "--branch-threshold", "0.001", "--dilution-alpha", "0.01", "--dilution-h", "0.004", "--write-csv",
        "--output-dir", "out", "--run-name", "r", "--progress", "--progress-interval", "2",
        "--progress-file", "p.json", "--no-progress-stderr"])
    assert not want_help and prior == "0.02,0.05" and eprior == "0.1"
    assert (cfg.subjects, cfg.variants, cfg.options.search_depth) == (3, 2, 5)
    assert cfg.lattice_type == bgt.LatticeType.replicated_dilution and cfg.mode == bgt.SimulationMode.local_tree
    assert cfg.options.provider == bgt.Provider.cuda and cfg.options.selector == bgt.SelectorType.op_bbpa
    assert cfg.true_state_policy == bgt.TrueStatePolicy.trimmed and cfg.trim_percent == 0.5
    assert (cfg.global_tree_depth, cfg.workload_granularity) == (2, 4)
    assert (cfg.options.threshold_up, cfg.options.threshold_lo, cfg.options.branch_threshold) == (0.02, 0.03, 0.001)
    assert (cfg.dilution.alpha, cfg.dilution.h) == (0.01, 0.004)
    assert cfg.report.write_csv and cfg.report.output_directory == "out" and cfg.report.run_name == "r"
    assert cfg.progress.enabled and not cfg.progress.print_stderr
    assert cfg.progress.interval_seconds == 2.0 and cfg.progress.output_path == "p.json"
    assert simulate.parse_prior("0.02", 4) == [0.02] * 4
    assert simulate.parse_prior("0.1,0.2", 2) == [0.1, 0.2]


def test_usage_and_error_exits(capsys):
    assert simulate.main(["--help"]) == 0
    assert "Usage: bgt_simulate --subjects N --prior P[,P...] [options]" in capsys.readouterr().err
    assert simulate.main(["--subjects", "3"]) == 2  # no prior
    assert simulate.main(["--bogus"]) == 1
    assert "unknown argument: --bogus" in capsys.readouterr().err
    assert simulate.main(["--subjects", "2", "--prior", "0.1", "--mode", "parallel_global_tree"]) == 1
    assert "MPI" in capsys.readouterr().err
    assert simulate.main(["--subjects", "2", "--prior", "0.1", "--provider", "cpu"]) == 1
    assert "CPU provider" in capsys.readouterr().err
    assert simulate.main(["--subjects", "2", "--prior", "0.1", "--selector", "op_bha", "--variants", "2"]) == 1


def _result(status=bgt.SimulationRunStatus.completed):
    stats = bgt.TreeStats(2, 0.792, 0.002, 0.0, 0.002, 0.206, 1.0, 1.0)
    return bgt.SimulationResult(stats, bgt.Provider.cuda, 2, 2, evaluated_prior_mass=1.0, status=status,
                                timings=bgt.SimulationTimings(0.0, 0.0, 0.25, 0.5))


def test_csv_report_format(tmp_path):
    cfg = bgt.SimulationConfig(subjects=1, prior=[0.2])
    assert reporting.write_report_if_requested(cfg, _result()) == ""  # not requested
    cfg.report = bgt.ReportConfig(True, str(tmp_path), "")
    path = reporting.write_report_if_requested(cfg, _result())
    assert os.path.basename(path) == "local_tree.csv"
    lines = open(path).read().splitlines()
    assert lines[0] == "field,value"
    rows = dict(line.split(",", 1) for line in lines[1:])
    assert list(rows)[:6] == ["status", "termination_reason", "is_partial", "mode", "provider", "subjects"]
    assert rows["status"] == "completed" and rows["termination_reason"] == "none" and rows["is_partial"] == "false"
    assert rows["mode"] == "local_tree" and rows["provider"] == "2" and rows["world_size"] == "1"
    assert rows["total_leaves"] == "2" and rows["correct_probability"] == "0.792"
    assert rows["unclassified_probability"] == "0.206" and rows["state_coverage_fraction"] == "1"
    assert rows["evaluation_seconds"] == "0.25" and list(rows)[-1] == "total_seconds"
    cfg.report.run_name = "named"
    path = reporting.write_report_if_requested(cfg, _result(bgt.SimulationRunStatus.interrupted))
    assert os.path.basename(path) == "named.partial.csv"


def test_progress_snapshot_format():
    body = reporting.snapshot_json(bgt.SimulationRunStatus.running, bgt.TerminationReason.none, 8, 4, 0.5,
                                   bgt.TreeStats(3, 0.1), bgt.SimulationTimings(total_seconds=1.5), 'say "hi"')
    d = json.loads(body)
    assert list(d) == ["status", "termination_reason", "total_states", "evaluated_states", "state_coverage_fraction",
                       "evaluated_prior_mass", "stats", "timings", "message"]
    assert d["status"] == "running" and d["state_coverage_fraction"] == 0.5 and d["stats"]["total_leaves"] == 3
    assert d["message"] == 'say "hi"' and d["timings"]["total_seconds"] == 1.5
    assert '"correct_probability":0.10000000000000001' in body  # setprecision(17)


def test_cancelled_before_evaluation(tmp_path):
    cfg = bgt.SimulationConfig(subjects=3, prior=[0.05] * 3,
                               report=bgt.ReportConfig(True, str(tmp_path), "cancelled"),
                               progress=bgt.ProgressConfig(enabled=True))
    bgt.request_simulation_cancellation(bgt.TerminationReason.user_signal)
    try:
        res = bgt.run_simulation(cfg)
    finally:
        bgt.clear_simulation_cancellation()
    assert res.status == bgt.SimulationRunStatus.interrupted
    assert res.termination_reason == bgt.TerminationReason.user_signal and res.evaluated_states == 0
    assert os.path.basename(res.report_path) == "cancelled.partial.csv"
    snap = json.loads(open(res.progress_path).read())
    assert snap["status"] == "interrupted" and snap["message"] == "cancelled before evaluation started"
    hist = open(os.path.join(str(tmp_path), "cancelled.progress.jsonl")).read().splitlines()
    assert len(hist) == 1


def test_runtime_and_kernel_spec():
    # bgt::Runtime / KernelSpec (include/bgt/runtime.hpp:58-74): specs record
    # the request; no run-time compilation; CUDA disabled in the compile
    # options refuses Provider.cuda (src/runtime/simulation_runner.cpp:205-206).
    rt = bgt.Runtime("cache")
    cfg = bgt.SimulationConfig(subjects=3, variants=2, prior=[0.1] * 6,
                               lattice_type=bgt.LatticeType.replicated_dilution)
    spec = rt.make_kernel_spec(cfg)
    assert spec.dilution == bgt.DilutionMode.dilution and spec.selector == bgt.SelectorType.op_bbpa
    assert (spec.subjects, spec.variants, spec.cuda_arch) == (3, 2, "sm_103a")
    info = rt.jit_cache_info()
    assert not info.jit_enabled and info.memory_entries == 0 and info.disk_cache_directory == "cache"
    rt.clear_jit_cache()
    assert bgt.Provider.cpu in rt.available_providers()
    cfg.options.provider = bgt.Provider.cuda
    cfg.options.compile_options.enable_cuda = False
    with pytest.raises(bgt.Error):
        rt.run_simulation(cfg)
