"""GB300-native CUDA provider for the BayesianGroupTesting lattice hot path.

The compute path is libbgt_gb300.so (hand-written sm_103a kernels behind the C
ABI of include/bgt_gpu.h).  This package exposes it with the reference's
Python API names (``Lattice``, ``run_simulation``, ...).
"""
from .api import (  # noqa: F401
    DilutionParameters,
    DilutionTable,
    Error,
    Lattice,
    LatticeType,
    Precision,
    ProgressConfig,
    Provider,
    ReportConfig,
    SelectorType,
    SimulationConfig,
    SimulationMode,
    SimulationOptions,
    SimulationResult,
    SimulationRunStatus,
    SimulationTimings,
    StatusCode,
    TerminationReason,
    TreeStats,
    TrueStatePolicy,
    available_providers,
    clear_simulation_cancellation,
    cuda_available,
    request_simulation_cancellation,
    simulation_cancellation_reason,
    simulation_cancellation_requested,
    reverse_bits,
    run_simulation,
    select_experiment,
    update,
)
from .build import LIB as LIBRARY_PATH  # noqa: F401
