"""spicier_gb300 — GB300 backend of Spicier's batched-sweep hot path.

Batched Newton-Raphson DC operating points (and the BatchedLuSolver trait)
on hand-written sm_103a CUDA kernels behind the C ABI in
include/spicier_gb300.h.  This package is the host-side mirror of the
reference's Rust interface; it has no CPU fallback.
"""
from . import _abi as abi  # noqa: F401
from .circuit import Circuit, Gauss, LogUniform, Pulse, Table, Uniform  # noqa: F401
from ._lib import SpicierError, load  # noqa: F401
from .api import (  # noqa: F401
    BackendSelector,
    BackendType,
    BatchedSolveResult,
    Context,
    CornerGenerator,
    Gb300BatchedSolver,
    GpuBatchConfig,
    GpuBatchedSweepResult,
    LinearSweepGenerator,
    MonteCarloGenerator,
    NewtonResult,
    ParameterVariation,
    SweepPoint,
    Topology,
    solve_batched_sweep_gpu,
    solve_newton_sweep_gpu,
)

__version__ = "0.1.0"
