"""ctypes mirror of ``include/spicier_gb300.h``.

Struct layouts, enum values and defaults here must match the header byte for
byte; ``tests/test_abi.py`` checks sizes and offsets against the compiled
library.
"""
from __future__ import annotations

import ctypes as C

# sp_status (BatchedSweepError, crates/spicier-batched-sweep/src/error.rs:7-43)
SP_OK = 0
SP_ERR_NO_BACKEND = -1
SP_ERR_BACKEND_INIT = -2
SP_ERR_MEMORY_ALLOC = -3
SP_ERR_TRANSFER = -4
SP_ERR_INVALID_DIMENSION = -5
SP_ERR_BATCH_TOO_LARGE = -6
SP_ERR_SINGULAR_BATCH = -7
SP_ERR_BACKEND = -8
SP_ERR_SOLVER = -9
SP_ERR_INVALID_ARGUMENT = -10

STATUS_NAMES = {
    SP_ERR_NO_BACKEND: "NoBackendAvailable",
    SP_ERR_BACKEND_INIT: "BackendInit",
    SP_ERR_MEMORY_ALLOC: "MemoryAlloc",
    SP_ERR_TRANSFER: "Transfer",
    SP_ERR_INVALID_DIMENSION: "InvalidDimension",
    SP_ERR_BATCH_TOO_LARGE: "BatchTooLarge",
    SP_ERR_SINGULAR_BATCH: "SingularBatch",
    SP_ERR_BACKEND: "Backend",
    SP_ERR_SOLVER: "Solver",
    SP_ERR_INVALID_ARGUMENT: "InvalidArgument",
}

# sp_backend_type (BackendType, crates/spicier-batched-sweep/src/solver.rs:79-92)
SP_BACKEND_CUDA, SP_BACKEND_METAL, SP_BACKEND_MPS = 0, 1, 2
SP_BACKEND_ACCELERATE, SP_BACKEND_FAER, SP_BACKEND_CPU, SP_BACKEND_GB300 = 3, 4, 5, 6

SP_PREC_FP64 = 0
SP_PREC_MIXED = 1
SP_PREC_FP64_EXACT = 2

# sp_element_kind
SP_EL_R, SP_EL_C, SP_EL_L, SP_EL_V, SP_EL_I = 1, 2, 3, 4, 5
SP_EL_D, SP_EL_NMOS, SP_EL_PMOS, SP_EL_NPN, SP_EL_PNP = 6, 7, 8, 9, 10
SP_EL_BSIM3N, SP_EL_BSIM3P = 11, 12
# sp_bsim3_card: the slots of a BSIM3 element from its field[0], in order
BSIM3_CARD = ("tox", "lint", "wint", "vth0", "k1", "k2", "dvt0", "dvt1", "dvt2", "nfactor",
              "k3", "k3b", "w0", "dvt0w", "dvt1w", "dvt2w", "u0", "ua", "ub", "uc", "vsat",
              "pclm", "pdiblc1", "pdiblc2", "drout", "eta0", "etab", "dsub", "pdiblcb", "pvag",
              "nch", "tnom", "kt2", "w", "l", "nf",
              "cgso", "cgdo", "cgbo", "cj", "cjsw", "cjswg", "mj", "mjsw", "mjswg", "pb", "pbsw", "pbswg",
              "as_", "ad", "ps", "pd")
SP_B3_CARD = len(BSIM3_CARD)
SP_MAX_FIELDS = 6

# sp_draw_kind
SP_DRAW_FIXED, SP_DRAW_GAUSS, SP_DRAW_UNIFORM, SP_DRAW_LOGUNIFORM, SP_DRAW_TABLE = 0, 1, 2, 3, 4

# sp_fallback_bits
SP_FALLBACK_GMIN = 1
SP_FALLBACK_SOURCE = 2

# sp_sample_status
SP_MLP_KERNEL_AUTO, SP_MLP_KERNEL_TCGEN05, SP_MLP_KERNEL_MMA_SYNC, SP_MLP_KERNEL_LAYERED = 0, 1, 2, 3
SP_MLP_KERNEL_LINEAR = 4

SP_ST_CONVERGED = 0
SP_ST_FAILED = 1
SP_ST_SINGULAR = 2
SP_ST_NONFINITE = 3
SP_ST_MASK = 0x0F
SP_ST_FLAG_WARM = 0x10
SP_ST_FLAG_COLD = 0x20
SP_ST_FLAG_GMIN = 0x40
SP_ST_FLAG_SOURCE = 0x80


class SpBatchConfig(C.Structure):
    _fields_ = [
        ("min_batch_size", C.c_uint64),
        ("min_matrix_size", C.c_uint64),
        ("max_batch_per_launch", C.c_uint64),
    ]


class SpElement(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("node", C.c_int32 * 4),
        ("branch", C.c_int32),
        ("wave", C.c_int32),
        ("field", C.c_int32 * SP_MAX_FIELDS),
    ]


class SpParam(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("rng_index", C.c_uint32),
        ("a", C.c_double),
        ("b", C.c_double),
    ]


class SpPulse(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("v1", "v2", "td", "tr", "tf", "pw", "per")]


class SpCircuit(C.Structure):
    _fields_ = [
        ("num_nodes", C.c_int32),
        ("num_branches", C.c_int32),
        ("num_elements", C.c_int32),
        ("num_params", C.c_int32),
        ("num_pulses", C.c_int32),
        ("reserved", C.c_int32),
        ("elements", C.POINTER(SpElement)),
        ("params", C.POINTER(SpParam)),
        ("pulses", C.POINTER(SpPulse)),
        ("nodeset", C.POINTER(C.c_double)),
    ]


class SpNewtonConfig(C.Structure):
    _fields_ = [
        ("v_abstol", C.c_double),
        ("v_reltol", C.c_double),
        ("i_abstol", C.c_double),
        ("gmin", C.c_double),
        ("max_iterations", C.c_int32),
        ("precision", C.c_int32),
        ("fallback", C.c_int32),
        ("refine_steps", C.c_int32),
        ("gmin_initial", C.c_double),
        ("gmin_final", C.c_double),
        ("gmin_reduction", C.c_double),
        ("gmin_max_attempts", C.c_int32),
        ("src_max_attempts", C.c_int32),
        ("src_initial", C.c_double),
        ("src_step", C.c_double),
        ("src_min_step", C.c_double),
        ("warm_max_iterations", C.c_int32),
        ("reserved", C.c_int32),
    ]


class SpMoments(C.Structure):
    _fields_ = [
        ("count", C.c_uint64),
        ("sum", C.c_double),
        ("sum_sq", C.c_double),
        ("min", C.c_double),
        ("max", C.c_double),
    ]


def newton_config(
    precision: int = SP_PREC_FP64,
    fallback: int = SP_FALLBACK_GMIN | SP_FALLBACK_SOURCE,
    max_iterations: int = 50,
    v_abstol: float = 1e-6,
    v_reltol: float = 1e-3,
    i_abstol: float = 1e-12,
    refine_steps: int = 0,
    warm_max_iterations: int = 0,
) -> SpNewtonConfig:
    """ConvergenceCriteria::default() + Gmin/SourceSteppingParams::default()
    (crates/spicier-solver/src/newton.rs:24-34, 187-196, 222-231)."""
    c = SpNewtonConfig()
    c.v_abstol, c.v_reltol, c.i_abstol, c.gmin = v_abstol, v_reltol, i_abstol, 1e-12
    c.max_iterations, c.precision, c.fallback, c.refine_steps = max_iterations, precision, fallback, refine_steps
    c.gmin_initial, c.gmin_final, c.gmin_reduction, c.gmin_max_attempts = 1e-3, 1e-12, 10.0, 5
    c.src_max_attempts, c.src_initial, c.src_step, c.src_min_step = 5, 0.1, 0.1, 0.01
    c.warm_max_iterations, c.reserved = warm_max_iterations, 0
    return c


SP_TRAN_BE, SP_TRAN_TRAP, SP_TRAN_TRBDF2 = 0, 1, 2


class SpTransientConfig(C.Structure):
    _fields_ = [("tstep", C.c_double), ("tstop", C.c_double), ("method", C.c_int32), ("probe", C.c_int32),
                ("precision", C.c_int32), ("reserved", C.c_int32)]


def transient_config(tstep: float, tstop: float, method: int = SP_TRAN_BE, probe: int = -1,
                     precision: int = SP_PREC_FP64) -> SpTransientConfig:
    """Fixed-step transient settings (TransientParams, solver.rs): step, stop time, method, the transient
    unknown recorded at every step (-1: none) and SP_PREC_FP64 or SP_PREC_FP64_EXACT."""
    return SpTransientConfig(tstep, tstop, method, probe, precision, 0)


SP_AC_LIN, SP_AC_DEC, SP_AC_OCT = 0, 1, 2


class SpAcConfig(C.Structure):
    _fields_ = [("fstart", C.c_double), ("fstop", C.c_double), ("num_points", C.c_int32), ("sweep", C.c_int32),
                ("source", C.c_int32), ("num_probe", C.c_int32), ("probe", C.c_int32 * 8), ("precision", C.c_int32),
                ("refine", C.c_int32)]


def ac_config(fstart: float, fstop: float, num_points: int, sweep: int = SP_AC_DEC, probes=(0,),
              source: int = -1, precision: int = SP_PREC_FP64, refine: int = 0) -> SpAcConfig:
    """AC sweep settings (AcParams, ac.rs:30-40): frequency range and points (total for SP_AC_LIN, per decade or
    octave otherwise), the recorded unknowns (1..8), the stimulus (-1: every V source at AC magnitude 1, as
    the reference's ac_info default; else the element index of the one source), and the precision
    (SP_PREC_FP64: the reference's LU order; SP_PREC_MIXED: FP32 LU with `refine` FP64 refinement steps)."""
    c = SpAcConfig()
    c.fstart, c.fstop, c.num_points, c.sweep, c.source = fstart, fstop, num_points, sweep, source
    c.precision, c.refine = precision, refine
    c.num_probe = len(probes)
    for k, p in enumerate(probes):
        c.probe[k] = p
    return c


class SpLadderConfig(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("tstop", "h_init", "h_min", "h_max", "lte_reltol", "lte_abstol",
                                          "v_reltol", "v_abstol", "i_abstol", "r_lo", "r_hi", "c_lo", "c_hi",
                                          "diode_is", "diode_n")] + [("pulse", SpPulse)] + [
        (k, C.c_int32) for k in ("min_sections", "max_sections", "max_iterations", "max_steps", "precision",
                                 "num_probe")]


def ladder_config(**kw) -> SpLadderConfig:
    """The 4,096-ladder workload's transient settings (AdaptiveTransientParams::
    for_tstop(100 ns), crates/spicier-solver/src/transient/types.rs:95-118, and
    the SPICE Newton tolerances); keyword arguments override fields."""
    c = SpLadderConfig()
    c.tstop, c.h_init, c.h_min, c.h_max = 100e-9, 1e-9, 1e-15, 100e-9 / 100.0
    c.lte_reltol, c.lte_abstol = 1e-3, 1e-6
    c.v_reltol, c.v_abstol, c.i_abstol = 1e-3, 1e-6, 1e-12
    c.r_lo, c.r_hi, c.c_lo, c.c_hi = 100.0, 10e3, 1e-12, 100e-12
    c.diode_is, c.diode_n = 1e-14, 1.0
    c.pulse = SpPulse(0.0, 1.8, 0.0, 1e-9, 1e-9, 10e-9, 20e-9)
    c.min_sections, c.max_sections, c.max_iterations, c.max_steps = 8, 512, 50, 200000
    c.precision, c.num_probe = SP_PREC_FP64, 101
    for k, v in kw.items():
        setattr(c, k, v)
    return c


class SpGridConfig(C.Structure):
    _fields_ = [(k, C.c_int32) for k in ("rows", "cols", "num_sinks", "max_newton", "restart", "max_krylov",
                                         "precision", "reserved")] + [
        (k, C.c_double) for k in ("r_lo", "r_hi", "r_scale_lo", "r_scale_hi", "vto_shift", "vdd", "strap_g",
                                  "vgs_lo", "vgs_hi", "vto", "kp", "lambda_", "w", "l", "v_reltol", "v_abstol",
                                  "i_abstol", "krylov_tol", "resid_target")]


def grid_config(**kw) -> SpGridConfig:
    """The 256-corner power-grid workload's settings; keyword arguments override fields."""
    c = SpGridConfig()
    c.rows, c.cols, c.num_sinks, c.max_newton, c.restart, c.max_krylov = 64, 64, 512, 30, 30, 20000
    c.precision, c.reserved = SP_PREC_FP64, 0
    c.r_lo, c.r_hi, c.r_scale_lo, c.r_scale_hi, c.vto_shift = 0.5, 2.0, 0.9, 1.1, 0.05
    c.vdd, c.strap_g, c.vgs_lo, c.vgs_hi = 1.0, 1e3, 0.8, 1.2
    c.vto, c.kp, c.lambda_, c.w, c.l = 0.7, 110e-6, 0.04, 5e-6, 0.5e-6
    c.v_reltol, c.v_abstol, c.i_abstol = 1e-3, 1e-6, 1e-12
    c.krylov_tol, c.resid_target = 1e-9, 1e-9
    for k, v in kw.items():
        setattr(c, k, v)
    return c


class SpYieldSpec(C.Structure):
    _fields_ = [("col", C.c_uint32), ("reserved", C.c_uint32), ("lower", C.c_double), ("upper", C.c_double)]
