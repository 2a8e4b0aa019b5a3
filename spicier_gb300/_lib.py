"""ctypes loader of libspicier_gb300.so.

The product path has no CPU fallback: if the shared library is missing or a
GPU is absent, calls raise instead of computing anything on the host.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import threading

from . import _abi as abi

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libspicier_gb300.so")
HEADER = os.path.join(HERE, "..", "include", "spicier_gb300.h")

_lock = threading.Lock()
_lib = None


class SpKernelTime(C.Structure):
    _fields_ = [("name", C.c_char * 48), ("launches", C.c_uint64), ("total_ms", C.c_double)]


class SpMlpDesc(C.Structure):
    _fields_ = [("n_in", C.c_int32), ("n_hidden", C.c_int32), ("n_layers", C.c_int32), ("n_out", C.c_int32),
                ("init_seed", C.c_uint64)]


class SpicierError(RuntimeError):
    """A negative sp_status from the library (BatchedSweepError mirror)."""

    def __init__(self, code: int, message: str = ""):
        self.code = code
        self.kind = abi.STATUS_NAMES.get(code, f"Status{code}")
        super().__init__(f"{self.kind}: {message}" if message else self.kind)


def header_functions() -> list:
    """Names of every function the public header declares."""
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sp_[a-z0-9_]+)\s*\(", text)))


def load(path: str = LIB_PATH):
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError(
                f"libspicier_gb300.so not found at {path}; build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'` (no CPU fallback exists)")
        L = C.CDLL(path)
        _bind(L)
        _lib = L
        return L


def _bind(L):
    P = C.POINTER
    vp, i32, u32, u64, d = C.c_void_p, C.c_int, C.c_uint32, C.c_uint64, C.c_double
    sig = {
        "sp_version": (C.c_char_p, []),
        "sp_backend_type": (i32, []),
        "sp_ctx_create": (i32, [i32, P(vp)]),
        "sp_ctx_destroy": (i32, [vp]),
        "sp_ctx_last_error": (C.c_char_p, [vp]),
        "sp_should_use_gpu": (i32, [vp, C.c_size_t, C.c_size_t]),
        "sp_get_config": (i32, [vp, P(abi.SpBatchConfig)]),
        "sp_set_config": (i32, [vp, P(abi.SpBatchConfig)]),
        "sp_solve_batch": (i32, [vp, vp, vp, C.c_size_t, C.c_size_t, vp, vp, P(u64)]),
        "sp_solve_batch_device": (i32, [vp, vp, vp, C.c_size_t, C.c_size_t, vp, vp, i32, i32, vp]),
        "sp_newton_config_default": (None, [P(abi.SpNewtonConfig)]),
        "sp_topology_create": (i32, [vp, P(abi.SpCircuit), P(vp)]),
        "sp_topology_destroy": (i32, [vp]),
        "sp_topology_size": (i32, [vp]),
        "sp_newton_dc_device": (i32, [vp, vp, P(abi.SpNewtonConfig), u64, u64, u64, vp, u32, vp, vp, vp, vp,
                                      vp, vp, vp, vp]),
        "sp_newton_dc": (i32, [vp, P(abi.SpCircuit), P(abi.SpNewtonConfig), u64, u64, u64, vp, u32, vp, vp, vp,
                               vp, vp, vp, vp]),
        "sp_draw_params_device": (i32, [vp, vp, u64, u64, u64, vp, u32, vp, vp]),
        "sp_rng_fill_device": (i32, [vp, i32, u64, u64, u32, u64, vp, vp]),
        "sp_moments_device": (i32, [vp, vp, u64, u32, u32, vp, vp, vp]),
        "sp_mlp_create": (i32, [vp, P(SpMlpDesc), P(vp)]),
        "sp_mlp_destroy": (i32, [vp]),
        "sp_mlp_num_params": (i32, [vp]),
        "sp_mlp_get_params": (i32, [vp, vp]),
        "sp_mlp_set_params": (i32, [vp, vp]),
        "sp_mlp_set_io": (i32, [vp, vp, vp, vp, vp, vp]),
        "sp_mlp_set_linear": (i32, [vp, vp]),
        "sp_mlp_set_inference_kernel": (i32, [vp, i32]),
        "sp_mlp_set_training_kernel": (i32, [vp, i32]),
        "sp_mlp_fault": (i32, [vp, P(i32)]),
        "sp_mlp_warm_start_device": (i32, [vp, vp, u64, u64, vp, vp]),
        "sp_mlp_forward_device": (i32, [vp, vp, u64, vp, vp]),
        "sp_mlp_gradients_device": (i32, [vp, vp, vp, u64, vp, vp, vp]),
        "sp_mlp_train_device": (i32, [vp, vp, vp, u64, i32, i32, C.c_float, vp, vp]),
        "sp_newton_dc_learned_device": (i32, [vp, vp, vp, P(abi.SpNewtonConfig), u64, u64, u64, vp, u32, vp, vp,
                                              vp, vp, vp, vp]),
        "sp_newton_dc_learned": (i32, [vp, P(abi.SpCircuit), vp, P(abi.SpNewtonConfig), u64, u64, u64, vp, u32,
                                       vp, vp, vp, vp, vp]),
        "sp_topology_specialize": (i32, [vp, vp, i32, i32, C.c_char_p, C.c_size_t]),
        "sp_specialize_source": (i32, [P(abi.SpCircuit), i32, i32, C.c_char_p, C.c_size_t, P(i32)]),
        "sp_ac_frequencies": (i32, [P(abi.SpAcConfig), vp, i32]),
        "sp_ac_sweep_device": (i32, [vp, vp, P(abi.SpNewtonConfig), P(abi.SpAcConfig), u64, u64, u64, vp, u32, vp, vp,
                                     vp]),
        "sp_ac_sweep": (i32, [vp, P(abi.SpCircuit), P(abi.SpNewtonConfig), P(abi.SpAcConfig), u64, u64, u64, vp, u32,
                              vp, vp]),
        "sp_transient_device": (i32, [vp, vp, P(abi.SpNewtonConfig), P(abi.SpTransientConfig), u64, u64, u64, vp,
                                      u32, vp, vp, vp, vp]),
        "sp_transient": (i32, [vp, P(abi.SpCircuit), P(abi.SpNewtonConfig), P(abi.SpTransientConfig), u64, u64, u64, vp, u32, vp,
                               vp, vp]),
        "sp_draw_params_host": (i32, [P(abi.SpCircuit), u64, u64, u64, vp, u32, vp, i32]),
        "sp_ladder_config_default": (None, [P(abi.SpLadderConfig)]),
        "sp_ladder_transient_device": (i32, [vp, P(abi.SpLadderConfig), u64, u64, u64, vp, vp, vp, vp, vp, vp, vp,
                                             vp]),
        "sp_ladder_transient_steps_device": (i32, [vp, P(abi.SpLadderConfig), u64, u64, u64, vp, vp, vp, vp, vp,
                                                   vp, vp, vp, i32, vp]),
        "sp_ladder_transient": (i32, [vp, P(abi.SpLadderConfig), u64, u64, u64, vp, vp, vp, vp, vp, vp, vp]),
        "sp_grid_config_default": (None, [P(abi.SpGridConfig)]),
        "sp_grid_solve_device": (i32, [vp, P(abi.SpGridConfig), u64, u64, u64, vp, vp, vp, vp, vp, vp]),
        "sp_grid_solve": (i32, [vp, P(abi.SpGridConfig), u64, u64, u64, vp, vp, vp, vp, vp]),
        "sp_histogram_device": (i32, [vp, vp, u64, u32, u32, vp, d, d, u32, vp, vp]),
        "sp_bsim3_eval_device": (i32, [vp, i32, vp, vp, u64, vp, vp, vp]),
        "sp_yield_device": (i32, [vp, vp, u64, u32, vp, vp, u32, vp, vp]),
        "sp_tune_set": (i32, [vp, C.c_char_p, i32]),
        "sp_tune_get": (i32, [vp, C.c_char_p, P(i32)]),
        "sp_tune_bucket": (i32, [C.c_longlong]),
        "sp_moments_merge_device": (i32, [vp, vp, vp, u32, vp]),
        "sp_moments_merge": (i32, [vp, vp, u32]),
        "sp_profile_enable": (i32, [vp, i32]),
        "sp_profile_read": (i32, [vp, P(SpKernelTime), i32, P(i32)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype, f.argtypes = res, args


def check(ctx_ptr, rc: int):
    if rc != 0:
        msg = ""
        if ctx_ptr:
            raw = load().sp_ctx_last_error(ctx_ptr)
            msg = raw.decode() if raw else ""
        raise SpicierError(rc, msg)
