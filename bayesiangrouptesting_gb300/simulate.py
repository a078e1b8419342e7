"""``python -m bayesiangrouptesting_gb300.simulate``: the reference's
``bgt_simulate`` command line (examples/run_simulation.cpp) on the GB300
provider.  Same options, usage text, summary line, CSV report and progress
files; the run goes through ``run_simulation`` on the device.  The parallel
tree modes need the MPI backend and the CPU provider is the reference
library's own, so those requests end with an error (exit status 1), as any
other failure does; a missing --subjects or --prior prints the usage and
exits with status 2.
"""
from __future__ import annotations

import signal
import sys
from typing import List, Optional

from .api import (LatticeType, Provider, SelectorType, SimulationConfig, SimulationMode, TerminationReason,
                  TrueStatePolicy, clear_simulation_cancellation, request_simulation_cancellation, run_simulation)

_MODES = {m.name: m for m in SimulationMode}
_LATTICES = {t.name: t for t in LatticeType}
_PROVIDERS = {"auto": Provider.auto_select, "cpu": Provider.cpu, "cuda": Provider.cuda}
_SELECTORS = {"auto": SelectorType.auto_select, "op_bha": SelectorType.op_bha, "op_bbpa": SelectorType.op_bbpa}
_POLICIES = {p.name: p for p in TrueStatePolicy}


def _parse(table, value: str, what: str):
    if value not in table:
        raise ValueError(f"unknown {what}: {value}")
    return table[value]


def parse_prior(value: str, expected_size: int) -> List[float]:
    """parse_prior (examples/run_simulation.cpp:104-120): comma-separated
    values; one value is repeated for every atom."""
    prior = [float(item) for item in value.split(",") if item]
    if len(prior) == 1 and expected_size > 1:
        prior = prior * expected_size
    return prior


def usage(program: str) -> str:
    return (f"Usage: {program} --subjects N --prior P[,P...] [options]\n"
            "Options:\n"
            "  --variants K\n"
            "  --lattice replicated_non_dilution|replicated_dilution|distributed_non_dilution|distributed_dilution\n"
            "  --mode local_tree|parallel_global_tree|parallel_dynamic_tree|parallel_hybrid_tree|parallel_partial_tree"
            "|parallel_fusion_tree\n"
            "  --search-depth N\n"
            "  --global-tree-depth N\n"
            "  --workload-granularity N\n"
            "  --provider auto|cpu|cuda\n"
            "  --selector auto|op_bha|op_bbpa\n"
            "  --true-state-policy all|trimmed|symmetric\n"
            "  --evaluation-prior P[,P...]\n"
            "  --trim-percent P\n"
            "  --write-csv --output-dir DIR --run-name NAME\n"
            "  --progress [--progress-interval SECONDS] [--progress-file PATH] [--no-progress-stderr]\n")


def parse_args(argv: List[str]):
    """The option loop of main (examples/run_simulation.cpp:162-222).
    Returns (config, prior text, evaluation-prior text, help requested)."""
    config = SimulationConfig()
    prior_arg = ""
    evaluation_prior_arg = ""
    i = 0
    while i < len(argv):
        key = argv[i]

        def value(name: str) -> str:
            nonlocal i
            if i + 1 >= len(argv):
                raise ValueError(f"missing value for {name}")
            i += 1
            return argv[i]

        if key in ("--help", "-h"):
            return config, prior_arg, evaluation_prior_arg, True
        if key == "--subjects":
            config.subjects = int(value(key))
        elif key == "--variants":
            config.variants = int(value(key))
        elif key == "--prior":
            prior_arg = value(key)
        elif key == "--evaluation-prior":
            evaluation_prior_arg = value(key)
        elif key == "--lattice":
            config.lattice_type = _parse(_LATTICES, value(key), "lattice")
        elif key == "--mode":
            config.mode = _parse(_MODES, value(key), "mode")
        elif key == "--search-depth":
            config.options.search_depth = int(value(key))
        elif key == "--global-tree-depth":
            config.global_tree_depth = int(value(key))
        elif key == "--workload-granularity":
            config.workload_granularity = int(value(key))
        elif key == "--provider":
            config.options.provider = _parse(_PROVIDERS, value(key), "provider")
        elif key == "--selector":
            config.options.selector = _parse(_SELECTORS, value(key), "selector")
        elif key == "--true-state-policy":
            config.true_state_policy = _parse(_POLICIES, value(key), "true-state policy")
        elif key == "--trim-percent":
            config.trim_percent = float(value(key))
        elif key == "--threshold-up":
            config.options.threshold_up = float(value(key))
        elif key == "--threshold-lo":
            config.options.threshold_lo = float(value(key))
        elif key == "--branch-threshold":
            config.options.branch_threshold = float(value(key))
        elif key == "--dilution-alpha":
            config.dilution.alpha = float(value(key))
        elif key == "--dilution-h":
            config.dilution.h = float(value(key))
        elif key == "--write-csv":
            config.report.write_csv = True
        elif key == "--output-dir":
            config.report.output_directory = value(key)
        elif key == "--run-name":
            config.report.run_name = value(key)
        elif key == "--progress":
            config.progress.enabled = True
            config.progress.print_stderr = True
        elif key == "--progress-interval":
            config.progress.interval_seconds = float(value(key))
        elif key == "--progress-file":
            config.progress.output_path = value(key)
        elif key == "--no-progress-stderr":
            config.progress.print_stderr = False
        else:
            raise ValueError(f"unknown argument: {key}")
        i += 1
    return config, prior_arg, evaluation_prior_arg, False


def summary_line(result) -> str:
    """The summary main prints on rank 0 (examples/run_simulation.cpp:252-262)."""
    return (f"mode={int(result.mode)} provider={int(result.provider)} status={int(result.status)}"
            f" total_states={result.total_states} evaluated_states={result.evaluated_states}"
            f" evaluated_prior_mass={result.evaluated_prior_mass:g} leaves={result.stats.total_leaves}"
            f" correct={result.stats.correct_probability:g} expected_tests={result.stats.expected_tests:g}")


def main(argv: Optional[List[str]] = None, program: str = "bgt_simulate") -> int:
    argv = sys.argv[1:] if argv is None else argv
    try:
        config, prior_arg, evaluation_prior_arg, want_help = parse_args(argv)
    except ValueError as error:
        # The reference's option errors escape main as exceptions.
        sys.stderr.write(f"bgt_simulate: {error}\n")
        return 1
    if want_help:
        sys.stderr.write(usage(program))
        return 0
    if config.subjects <= 0 or not prior_arg:
        sys.stderr.write(usage(program))
        return 2
    size = config.subjects * config.variants
    config.prior = parse_prior(prior_arg, size)
    if evaluation_prior_arg:
        config.evaluation_prior = parse_prior(evaluation_prior_arg, size)

    signals = {"count": 0}

    def on_signal(signum, _frame):
        signals["count"] += 1
        if signals["count"] == 1:
            request_simulation_cancellation(TerminationReason.user_signal)
            return
        sys.exit(128 + signum)

    try:
        clear_simulation_cancellation()
        previous = {s: signal.signal(s, on_signal) for s in (signal.SIGINT, signal.SIGTERM)}
        try:
            result = run_simulation(config)
        finally:
            for s, h in previous.items():
                signal.signal(s, h)
        if result.rank == 0:
            print(summary_line(result))
            if result.report_path:
                print(f"report={result.report_path}")
            if result.progress_path:
                print(f"progress={result.progress_path}")
    except Exception as error:  # noqa: BLE001 - the reference reports every std::exception the same way
        sys.stderr.write(f"bgt_simulate: {error}\n")
        return 1
    return 0


if __name__ == "__main__":
    sys.exit(main())
