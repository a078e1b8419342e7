"""Run reports and progress snapshots of ``run_simulation``, in the reference's
formats: the ``field,value`` CSV of write_report_if_requested
(src/runtime/reporting.cpp:10-45) and the JSON snapshots of ProgressTracker
(src/runtime/progress.cpp:48-80 and 139-300), written next to it as
``<run>.progress.json`` (latest) and ``<run>.progress.jsonl`` (history).

Numbers are printed the way the reference's iostreams print them: the CSV
with the default six significant digits (``%g``), the JSON with
``setprecision(17)`` (``%.17g``).
"""
from __future__ import annotations

import json
import os
import sys
import time

from .api import (ProgressSnapshot, SimulationConfig, SimulationMode, SimulationResult, SimulationRunStatus,
                  SimulationTimings, TerminationReason, TreeStats, simulation_cancellation_reason)


def simulation_mode_name(mode: SimulationMode) -> str:
    """simulation_mode_name (src/runtime/simulation_helpers.cpp:69-87)."""
    return SimulationMode(mode).name


def simulation_run_status_name(status: SimulationRunStatus) -> str:
    """simulation_run_status_name (src/runtime/progress.cpp:111-123)."""
    return SimulationRunStatus(status).name


def termination_reason_name(reason: TerminationReason) -> str:
    """termination_reason_name (src/runtime/progress.cpp:125-137)."""
    return TerminationReason(reason).name


def _g(v: float) -> str:
    # std::ostream's default formatting of a double: six significant digits.
    return "%g" % v


def _g17(v: float) -> str:
    return "%.17g" % v


def _run_name(config: SimulationConfig) -> str:
    return config.report.run_name or simulation_mode_name(config.mode)


def write_report_if_requested(config: SimulationConfig, result: SimulationResult) -> str:
    """write_report_if_requested (src/runtime/reporting.cpp:10-45): the
    ``field,value`` CSV of a finished (or interrupted: ``.partial.csv``) run,
    or "" when no report was asked for."""
    if not config.report.write_csv or result.rank != 0:
        return ""
    os.makedirs(config.report.output_directory, exist_ok=True)
    interrupted = result.status == SimulationRunStatus.interrupted
    path = os.path.join(config.report.output_directory, _run_name(config) + (".partial.csv" if interrupted else ".csv"))
    st, tm = result.stats, result.timings
    coverage = 0.0 if result.total_states == 0 else result.evaluated_states / result.total_states
    rows = [
        ("status", simulation_run_status_name(result.status)),
        ("termination_reason", termination_reason_name(result.termination_reason)),
        ("is_partial", "true" if interrupted else "false"),
        ("mode", simulation_mode_name(result.mode)),
        ("provider", str(int(result.provider))),
        ("subjects", str(config.subjects)),
        ("variants", str(config.variants)),
        ("world_size", str(result.world_size)),
        ("total_states", str(result.total_states)),
        ("evaluated_states", str(result.evaluated_states)),
        ("state_coverage_fraction", _g(coverage)),
        ("evaluated_prior_mass", _g(result.evaluated_prior_mass)),
        ("progress_path", result.progress_path),
        ("total_leaves", str(st.total_leaves)),
        ("correct_probability", _g(st.correct_probability)),
        ("incorrect_probability", _g(st.incorrect_probability)),
        ("false_positive_probability", _g(st.false_positive_probability)),
        ("false_negative_probability", _g(st.false_negative_probability)),
        ("unclassified_probability", _g(st.unclassified_probability)),
        ("expected_stages", _g(st.expected_stages)),
        ("expected_tests", _g(st.expected_tests)),
        ("setup_seconds", _g(tm.setup_seconds)),
        ("tree_build_seconds", _g(tm.tree_build_seconds)),
        ("evaluation_seconds", _g(tm.evaluation_seconds)),
        ("total_seconds", _g(tm.total_seconds)),
    ]
    with open(path, "w") as out:
        out.write("field,value\n")
        for k, v in rows:
            out.write(f"{k},{v}\n")
    return path


def snapshot_json(status: SimulationRunStatus, reason: TerminationReason, total_states: int, evaluated_states: int,
                  prior_mass: float, stats: TreeStats, timings: SimulationTimings, message: str) -> str:
    """snapshot_json (src/runtime/progress.cpp:48-80): one progress record."""
    coverage = 0.0 if total_states == 0 else evaluated_states / total_states
    s, t = stats, timings
    return ("{"
            f"\"status\":\"{simulation_run_status_name(status)}\","
            f"\"termination_reason\":\"{termination_reason_name(reason)}\","
            f"\"total_states\":{total_states},"
            f"\"evaluated_states\":{evaluated_states},"
            f"\"state_coverage_fraction\":{_g17(coverage)},"
            f"\"evaluated_prior_mass\":{_g17(prior_mass)},"
            "\"stats\":{"
            f"\"total_leaves\":{s.total_leaves},"
            f"\"correct_probability\":{_g17(s.correct_probability)},"
            f"\"incorrect_probability\":{_g17(s.incorrect_probability)},"
            f"\"false_positive_probability\":{_g17(s.false_positive_probability)},"
            f"\"false_negative_probability\":{_g17(s.false_negative_probability)},"
            f"\"unclassified_probability\":{_g17(s.unclassified_probability)},"
            f"\"expected_stages\":{_g17(s.expected_stages)},"
            f"\"expected_tests\":{_g17(s.expected_tests)}"
            "},"
            "\"timings\":{"
            f"\"setup_seconds\":{_g17(t.setup_seconds)},"
            f"\"tree_build_seconds\":{_g17(t.tree_build_seconds)},"
            f"\"evaluation_seconds\":{_g17(t.evaluation_seconds)},"
            f"\"total_seconds\":{_g17(t.total_seconds)}"
            "},"
            f"\"message\":{json.dumps(message)}"
            "}")


class ProgressTracker:
    """ProgressTracker (src/runtime/progress.cpp:139-300) for a device run:
    a running snapshot before the tree is launched and the final one after
    it (the device tree is one graph launch, so there is nothing between)."""

    def __init__(self, config: SimulationConfig, rank: int, total_states: int, total_start: float):
        self.config = config
        self.rank = rank
        self.total_states = total_states
        self.total_start = total_start
        self.last_emit = total_start
        self.evaluated_states = 0
        self.evaluated_prior_mass = 0.0
        self.stats = TreeStats()
        self.timings = SimulationTimings()
        self.progress_path = self._latest_path() if self._enabled() else ""

    def _enabled(self) -> bool:
        return self.config.progress.enabled and self.rank == 0

    def _latest_path(self) -> str:
        if self.config.progress.output_path:
            return str(self.config.progress.output_path)
        return os.path.join(self.config.report.output_directory, _run_name(self.config) + ".progress.json")

    def _history_path(self) -> str:
        return os.path.splitext(self._latest_path())[0] + ".jsonl"

    def replace_state(self, evaluated_states: int, prior_mass: float, stats: TreeStats) -> None:
        known = self.stats.total_leaves
        self.evaluated_states = evaluated_states
        self.evaluated_prior_mass = prior_mass
        self.stats = stats
        if self.stats.total_leaves == 0:
            self.stats.total_leaves = known

    def snapshot(self, status: SimulationRunStatus, reason: TerminationReason, message: str) -> ProgressSnapshot:
        """The record the tracker writes now (ProgressTracker::snapshot,
        src/runtime/progress.cpp:217-261)."""
        timings = SimulationTimings(self.timings.setup_seconds, self.timings.tree_build_seconds,
                                    self.timings.evaluation_seconds, time.perf_counter() - self.total_start)
        coverage = 0.0 if self.total_states == 0 else self.evaluated_states / self.total_states
        return ProgressSnapshot(status, reason, self.total_states, self.evaluated_states, coverage,
                                self.evaluated_prior_mass, self.stats, timings, message)

    def _snapshot(self, status: SimulationRunStatus, reason: TerminationReason, message: str):
        snap = self.snapshot(status, reason, message)
        return snapshot_json(snap.status, snap.reason, snap.total_states, snap.evaluated_states,
                             snap.evaluated_prior_mass, snap.stats, snap.timings, snap.message), snap.timings.total_seconds

    def maybe_emit(self, message: str, force: bool = False) -> bool:
        if not self._enabled():
            return False
        now = time.perf_counter()
        if not force and now - self.last_emit < self.config.progress.interval_seconds:
            return False
        reason = simulation_cancellation_reason()
        status = SimulationRunStatus.running if reason == TerminationReason.none else SimulationRunStatus.interrupted
        self._write(status, reason, message)
        self.last_emit = now
        return True

    def finish(self, status: SimulationRunStatus, reason: TerminationReason, message: str) -> None:
        if self._enabled():
            self._write(status, reason, message)

    def _write(self, status: SimulationRunStatus, reason: TerminationReason, message: str) -> None:
        body, elapsed = self._snapshot(status, reason, message)
        latest = self._latest_path()
        if os.path.dirname(latest):
            os.makedirs(os.path.dirname(latest), exist_ok=True)
        tmp = latest + ".tmp"
        with open(tmp, "w") as out:
            out.write(body + "\n")
        os.replace(tmp, latest)
        if self.config.progress.write_jsonl:
            hist = self._history_path()
            if os.path.dirname(hist):
                os.makedirs(os.path.dirname(hist), exist_ok=True)
            with open(hist, "a") as out:
                out.write(body + "\n")
        if self.config.progress.print_stderr:
            coverage = 0.0 if self.total_states == 0 else self.evaluated_states / self.total_states
            line = (f"bgt progress: status={simulation_run_status_name(status)}"
                    f" evaluated={self.evaluated_states}/{self.total_states}"
                    f" coverage={_g(coverage)} prior_mass={_g(self.evaluated_prior_mass)} elapsed={_g(elapsed)}s")
            if message:
                line += " " + message
            sys.stderr.write(line + "\n")
