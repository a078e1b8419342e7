"""The Python API surface a user of the reference's binding relies on
(tests/python/unit/test_public_api.py and tests/python/integration/
test_runtime.py of the reference list the expectations): exported names,
logging settings, enums, config coercion and kernel specs.  No device calls."""
import numpy as np
import pytest

import bayesiangrouptesting_gb300 as bgt
from bayesiangrouptesting_gb300 import logconfig


def test_public_exports():
    expected = {"CompileOptions", "KernelSpec", "Lattice", "LogConfig", "LogLevel", "LogSubsystem",
                "ProfileBackend", "Runtime", "ProgressConfig", "SimulationConfig", "SimulationMode",
                "SimulationRunStatus", "StatusCode", "TerminationReason", "clear_simulation_cancellation",
                "request_simulation_cancellation", "set_log_config", "set_log_level", "run_simulation",
                "select_experiment", "update", "get_log_config"}
    assert expected <= set(bgt.__all__)
    assert all(hasattr(bgt, name) for name in bgt.__all__)


@pytest.fixture
def restore_log_config():
    saved = bgt.get_log_config()
    yield
    bgt.set_log_config(saved)


def test_logging_round_trip(restore_log_config):
    cfg = bgt.LogConfig()
    assert cfg.level == bgt.LogLevel.warn and cfg.timestamps is True and cfg.color is False
    cfg.level = bgt.LogLevel.debug
    cfg.subsystems = [bgt.LogSubsystem.runtime]
    cfg.rank_filter = [0, 2]
    cfg.color = False
    cfg.timestamps = False
    bgt.set_log_config(cfg)
    got = bgt.get_log_config()
    assert got.level == bgt.LogLevel.debug
    assert got.subsystems == [bgt.LogSubsystem.runtime]
    assert got.rank_filter == [0, 2]
    assert got.color is False and got.timestamps is False
    bgt.set_log_level(bgt.LogLevel.warn)
    assert bgt.get_log_config().level == bgt.LogLevel.warn
    cfg.subsystems.append(bgt.LogSubsystem.cuda)   # the stored copy is independent
    assert bgt.get_log_config().subsystems == [bgt.LogSubsystem.runtime]


def test_log_filtering_and_output(restore_log_config, tmp_path):
    out = tmp_path / "bgt.log"
    bgt.set_log_config(bgt.LogConfig(level=bgt.LogLevel.info, subsystems=[bgt.LogSubsystem.cuda],
                                     timestamps=False, file_path=str(out)))
    assert bgt.log_enabled(bgt.LogLevel.info, bgt.LogSubsystem.cuda)
    assert not bgt.log_enabled(bgt.LogLevel.debug, bgt.LogSubsystem.cuda)
    assert not bgt.log_enabled(bgt.LogLevel.info, bgt.LogSubsystem.runtime)
    assert not bgt.log_enabled(bgt.LogLevel.off, bgt.LogSubsystem.cuda)
    bgt.log_message(bgt.LogLevel.info, bgt.LogSubsystem.cuda, "hello")
    bgt.log_message(bgt.LogLevel.debug, bgt.LogSubsystem.cuda, "hidden")
    line = out.read_text().strip()
    assert line.startswith("INFO cuda test_public_api.py:") and line.endswith(": hello")
    bgt.set_log_level(bgt.LogLevel.off)
    assert not bgt.log_enabled(bgt.LogLevel.fatal, bgt.LogSubsystem.cuda)


def test_log_names_and_parsing():
    assert bgt.parse_log_level("WARNING") == bgt.LogLevel.warn
    assert bgt.parse_log_level("Trace") == bgt.LogLevel.trace
    assert bgt.parse_log_level("nonsense") == bgt.LogLevel.warn
    assert bgt.parse_log_subsystem("JIT") == bgt.LogSubsystem.jit
    assert bgt.parse_log_subsystem("nonsense") == bgt.LogSubsystem.runtime
    assert bgt.log_level_name(bgt.LogLevel.error) == "ERROR"
    assert bgt.log_subsystem_name(bgt.LogSubsystem.perf) == "perf"


def test_log_environment(monkeypatch, restore_log_config):
    monkeypatch.setattr(logconfig, "_env_applied", False)
    monkeypatch.setattr(logconfig, "_config", logconfig.LogConfig())
    monkeypatch.setenv("BGT_LOG_LEVEL", "error")
    monkeypatch.setenv("BGT_LOG_SUBSYS", "tree,cuda")
    monkeypatch.setenv("BGT_LOG_RANKS", "1,3")
    monkeypatch.setenv("BGT_LOG_COLOR", "on")
    monkeypatch.setenv("BGT_PERF_LEVEL", "debug")
    cfg = bgt.get_log_config()
    assert cfg.level == bgt.LogLevel.debug  # raised by BGT_PERF_LEVEL
    assert cfg.subsystems == [bgt.LogSubsystem.tree, bgt.LogSubsystem.cuda, bgt.LogSubsystem.perf]
    assert cfg.rank_filter == [1, 3] and cfg.color is True


def test_status_error_and_modes():
    assert bgt.StatusCode.success.name == "success"
    assert issubclass(bgt.Error, RuntimeError)
    names = [m.name for m in bgt.SimulationMode if m != bgt.SimulationMode.local_tree]
    assert names and all(n.startswith("parallel_") for n in names)


def test_config_accepts_numpy_and_lists():
    cfg = bgt.SimulationConfig()
    cfg.subjects, cfg.variants = 1, 2
    cfg.prior = np.array([0.2, 0.4], dtype=np.float64)
    cfg.evaluation_prior = [0.3, 0.5]
    assert cfg.prior == [0.2, 0.4]
    assert cfg.evaluation_prior == [0.3, 0.5]
    assert bgt.SimulationConfig(prior=np.array([0.1])).prior == [0.1]


def test_progress_defaults():
    p = bgt.ProgressConfig()
    assert p.enabled is False and p.interval_seconds == 5.0 and p.write_jsonl is True and p.print_stderr is False


def test_kernel_specs():
    cfg = bgt.SimulationConfig(subjects=1, variants=2, prior=np.array([0.2, 0.4]))
    cfg.options.provider = bgt.Provider.cpu
    cfg.options.selector = bgt.SelectorType.op_bbpa
    spec = bgt.Runtime().make_kernel_spec(cfg)
    assert spec.provider == bgt.Provider.cpu and spec.variants == 2
    assert spec.selector == bgt.SelectorType.op_bbpa
    assert spec.precision == cfg.options.compile_options.posterior_precision
    cfg.options.compile_options.posterior_precision = bgt.Precision.float32
    cfg.options.compile_options.accumulator_precision = bgt.Precision.float32
    spec32 = bgt.Runtime().make_kernel_spec(cfg)
    assert spec32.precision == bgt.Precision.float32 and spec32.accumulator_precision == bgt.Precision.float32
    binary = bgt.SimulationConfig(subjects=2, prior=[0.2, 0.4])
    assert bgt.Runtime().make_kernel_spec(binary).selector == bgt.SelectorType.op_bha
    multi = bgt.SimulationConfig(subjects=1, variants=2, prior=[0.2, 0.4])
    assert bgt.Runtime().make_kernel_spec(multi).selector == bgt.SelectorType.op_bbpa


def test_progress_snapshot(tmp_path):
    snap = bgt.ProgressSnapshot()
    assert snap.status == bgt.SimulationRunStatus.completed and snap.reason == bgt.TerminationReason.none
    assert snap.total_states == 0 and snap.evaluated_states == 0 and snap.message == ""
    # the tracker's snapshot is the record it writes
    import json
    import time
    from bayesiangrouptesting_gb300.reporting import ProgressTracker
    cfg = bgt.SimulationConfig(subjects=2, prior=[0.2, 0.4])
    cfg.progress.enabled = True
    cfg.progress.output_path = str(tmp_path / "p.json")
    tracker = ProgressTracker(cfg, 0, 4, time.perf_counter())
    tracker.replace_state(4, 1.0, bgt.TreeStats(total_leaves=3, correct_probability=0.5))
    snap = tracker.snapshot(bgt.SimulationRunStatus.completed, bgt.TerminationReason.none, "done")
    assert (snap.total_states, snap.evaluated_states, snap.state_coverage_fraction) == (4, 4, 1.0)
    assert snap.stats.total_leaves == 3 and snap.message == "done"
    tracker.finish(bgt.SimulationRunStatus.completed, bgt.TerminationReason.none, "done")
    rec = json.loads((tmp_path / "p.json").read_text())
    assert rec["evaluated_states"] == 4 and rec["stats"]["total_leaves"] == 3 and rec["message"] == "done"
    assert rec["status"] == "completed"
