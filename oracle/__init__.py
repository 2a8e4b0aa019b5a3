"""CPU oracle for the batched Newton sweep — TEST INFRASTRUCTURE ONLY.

The oracle is a C++ restatement of Spicier's own CPU path
(crates/spicier-solver/src/newton.rs, crates/spicier-devices/src/*,
crates/spicier-core/src/mna.rs, crates/spicier-batched-sweep/src/rng.rs …),
compiled with -ffp-contract=off so that its IEEE operation sequence matches
the Rust reference.  Only tests/, ``__graft_entry__.smoke()`` and bench.py's
CPU-baseline leg may load it; it is the checker, never the thing measured as
the product.

Parity pinning: the reference cannot be compiled in this environment (Rust),
so the oracle is pinned against the reference's own unit-test known answers
(tests/test_oracle_pins.py) and against golden vectors generated by
tests/golden/make_golden.py.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle_spicier.so")
SOURCES = ["oracle_capi.cpp"]
HEADERS = ["transient.hpp", "powergrid.hpp", "oracle_core.hpp", "oracle_transient.hpp", "oracle_gmres.hpp"]

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle shared library (g++, -O2, no FMA contraction)."""
    srcs = [os.path.join(HERE, s) for s in SOURCES]
    deps = srcs + [os.path.join(HERE, h) for h in HEADERS if os.path.exists(os.path.join(HERE, h))]
    deps.append(os.path.join(HERE, "..", "include", "spicier_gb300.h"))
    deps += [os.path.join(HERE, "..", "spicier_gb300", "csrc", h) for h in ("cr_math.cuh", "cr_tables.h")]
    if not force and os.path.exists(LIB_PATH):
        mt = os.path.getmtime(LIB_PATH)
        if all(os.path.getmtime(d) <= mt for d in deps):
            return LIB_PATH
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
           "-fno-fast-math", "-pthread", "-o", LIB_PATH + ".tmp"] + srcs
    subprocess.run(cmd, check=True)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            _lib = _bind(C.CDLL(LIB_PATH))
        return _lib


def _bind(L):
    from spicier_gb300 import _abi as abi
    d, u64, u32, i32, vp_ = C.c_double, C.c_uint64, C.c_uint32, C.c_int, C.c_void_p
    P = C.POINTER
    sig = {
        "or_splitmix64": (u64, [u64]),
        "or_combine_indices": (u64, [u64, u32, u32]),
        "or_uniform": (d, [u64, u32, u32]),
        "or_uniform_f32": (C.c_float, [u64, u32, u32]),
        "or_gaussian": (d, [u64, u32, u32]),
        "or_gaussian_f32": (C.c_float, [u64, u32, u32]),
        "or_rng_fill": (None, [i32, u64, u64, u32, u64, P(d)]),
        "or_mos_evaluate": (i32, [i32, P(d), d, d, P(d)]),
        "or_diode_evaluate": (None, [d, d, d, P(d)]),
        "or_bsim3_evaluate": (None, [i32, P(d), P(d), u64, P(d), P(C.c_uint8)]),
        "or_bsim3_default_card": (None, [i32, P(d)]),
        "or_limit_voltage": (d, [d, d]),
        "or_thermal_voltage": (d, [d]),
        "or_bjt_evaluate": (None, [i32, P(d), d, d, P(d)]),
        "or_stamp_dc": (i32, [P(abi.SpCircuit), P(d), P(d), i32, d, P(d), P(d)]),
        "or_lu_solve": (i32, [i32, P(d), P(d)]),
        "or_solve_batch": (None, [P(d), P(d), u64, u64, P(d), P(C.c_uint8), i32]),
        "or_draw_params": (i32, [P(abi.SpCircuit), u64, u64, u64, P(d), u32, P(d)]),
        "or_newton_single": (i32, [P(abi.SpCircuit), P(d), P(abi.SpNewtonConfig), i32, d, P(d), P(i32)]),
        "or_stepping": (i32, [P(abi.SpCircuit), P(d), P(abi.SpNewtonConfig), i32, P(d), P(i32)]),
        "or_newton_dc": (i32, [P(abi.SpCircuit), P(abi.SpNewtonConfig), u64, u64, u64, P(d), u32,
                               P(d), P(d), P(C.c_int32), P(C.c_uint8), P(d), i32]),
        "or_moments": (None, [P(d), u64, u32, u32, P(C.c_uint8), P(abi.SpMoments)]),
        "or_set_math_mode": (None, [i32]),
        "or_ladder_draw": (i32, [vp_, u64, u32, P(d), P(d)]),
        "or_grid_solve": (None, [vp_, u64, u64, u64, P(d), P(i32), P(i32), P(C.c_uint8), P(d), i32]),
        "or_grid_sinks": (None, [vp_, u64, u32, P(i32), P(d)]),
        "or_histogram": (None, [P(d), u64, u32, u32, vp_, d, d, u32, P(u64)]),
        "or_transient": (None, [P(abi.SpCircuit), P(abi.SpNewtonConfig), u64, u64, u64, P(d), u32, i32, d, d, i32,
                                P(d), P(d), P(C.c_uint8), i32]),
        "or_yield": (None, [P(d), u64, u32, vp_, vp_, u32, P(u64)]),
        "or_ladder_transient": (None, [vp_, u64, u64, u64, P(d), P(i32), P(i32), P(i32), P(i32), P(C.c_uint8),
                                       P(d), i32]),
        "or_ladder_steps": (None, [vp_, u64, u64, u64, P(d), i32, P(i32), i32]),
        "or_ladder_replay": (None, [vp_, u64, u64, u64, P(d), i32, P(i32), P(d), P(i32), P(C.c_uint8), P(d), i32]),
        "or_get_math_mode": (i32, []),
        "or_cr_log": (d, [d, P(C.c_uint)]),
        "or_cr_cos": (d, [d, P(C.c_uint)]),
        "or_cr_log_batch": (None, [P(d), u64, P(d), P(C.c_uint)]),
        "or_cr_cos_batch": (None, [P(d), u64, P(d), P(C.c_uint)]),
        "or_cr_exp_batch": (None, [P(d), u64, P(d), P(C.c_uint)]),
        "or_cr_log_full_batch": (None, [P(d), u64, P(d), P(C.c_uint)]),
        "or_cr_cos_full_batch": (None, [P(d), u64, P(d), P(C.c_uint)]),
        "or_cr_fast_misses": (u64, [i32, P(d), u64]),
        "or_ieee_int_mismatches": (u64, [u64, u64]),
        "or_ac_frequencies": (i32, [d, d, i32, i32, P(d), i32]),
        "or_ac_sweep": (i32, [vp_, vp_, u64, u64, u64, P(d), u32, P(d), i32, i32, P(C.c_int), i32, P(d),
                              P(C.c_uint8), i32]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype, f.argtypes = res, args
    return L


class math_mode:
    """Context manager selecting the Gaussian draw's ln/cos: "libm" (the host
    libm, the reference's behaviour) or "cr" (the correctly rounded functions
    of the GPU kernels)."""

    def __init__(self, mode: str):
        self.mode = {"libm": 0, "cr": 1}[mode]

    def __enter__(self):
        self.prev = lib().or_get_math_mode()
        lib().or_set_math_mode(self.mode)
        return self

    def __exit__(self, *exc):
        lib().or_set_math_mode(self.prev)


def cr_batch(fn: str, x):
    """(values, hard count) of the host build of cr_log / cr_cos / cr_exp over x."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    hard = C.c_uint(0)
    getattr(lib(), f"or_cr_{fn}_batch")(_dp(x), x.size, _dp(y), C.byref(hard))
    return y, hard.value


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def newton_dc(circuit, cfg, seed, count, first=0, table=None, x0=None, threads=0):
    """Oracle sweep: returns (x[count,n], iters[count], status[count], params[count,np])."""
    L = lib()
    n, npar = circuit.n, len(circuit.params)
    x = np.zeros((count, n))
    iters = np.zeros(count, np.int32)
    status = np.zeros(count, np.uint8)
    params = np.zeros((count, max(npar, 1)))
    cols = 0
    if table is not None:
        table = np.ascontiguousarray(table, dtype=np.float64)
        cols = table.shape[1]
    if x0 is not None:
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
    cc = circuit.to_c()
    L.or_newton_dc(C.byref(cc), C.byref(cfg), seed, first, count, _dp(table), cols, _dp(x0), _dp(x),
                   iters.ctypes.data_as(C.POINTER(C.c_int32)),
                   status.ctypes.data_as(C.POINTER(C.c_uint8)), _dp(params), threads)
    return x, iters, status, params[:, :npar]


def draw_params(circuit, seed, count, first=0, table=None):
    L = lib()
    out = np.zeros((count, max(len(circuit.params), 1)))
    cols = 0
    if table is not None:
        table = np.ascontiguousarray(table, dtype=np.float64)
        cols = table.shape[1]
    cc = circuit.to_c()
    L.or_draw_params(C.byref(cc), seed, first, count, _dp(table), cols, _dp(out))
    return out[:, :len(circuit.params)]


def solve_batch(mats, rhs, n, batch, threads=0):
    L = lib()
    mats = np.ascontiguousarray(mats, dtype=np.float64)
    rhs = np.ascontiguousarray(rhs, dtype=np.float64)
    sol = np.zeros(batch * n)
    sing = np.zeros(batch, np.uint8)
    L.or_solve_batch(_dp(mats), _dp(rhs), n, batch, _dp(sol), sing.ctypes.data_as(C.POINTER(C.c_uint8)), threads)
    return sol, sing


def ladder_transient(cfg, seed, count, first=0, threads=0):
    """Oracle ladder transients: dict of x_final[count][max_sections+2], n, accepted,
    rejected, iterations, status, probe[count][num_probe]."""
    L = lib()
    ld = cfg.max_sections + 2
    x = np.zeros((count, ld))
    n = np.zeros(count, np.int32)
    acc = np.zeros(count, np.int32)
    rej = np.zeros(count, np.int32)
    it = np.zeros(count, np.int32)
    st = np.zeros(count, np.uint8)
    pr = np.zeros((count, max(cfg.num_probe, 1)))
    i32p = C.POINTER(C.c_int32)
    L.or_ladder_transient(C.byref(cfg), seed, first, count, _dp(x), n.ctypes.data_as(i32p), acc.ctypes.data_as(i32p),
                          rej.ctypes.data_as(i32p), it.ctypes.data_as(i32p),
                          st.ctypes.data_as(C.POINTER(C.c_uint8)), _dp(pr), threads)
    return dict(x=x, n=n, accepted=acc, rejected=rej, iterations=it, status=st, probe=pr[:, :cfg.num_probe])


def ladder_steps(cfg, seed, count, first=0, max_rec=4096, threads=0):
    """Accepted step sizes of the oracle's adaptive ladder runs: (steps[count][max_rec], nsteps[count])."""
    steps = np.zeros((count, max_rec))
    ns = np.zeros(count, np.int32)
    lib().or_ladder_steps(C.byref(cfg), seed, first, count, _dp(steps), max_rec,
                          ns.ctypes.data_as(C.POINTER(C.c_int32)), threads)
    return steps, ns


def ladder_replay(cfg, seed, steps, nsteps, first=0, threads=0):
    """Oracle ladders replayed along recorded accepted step sizes
    steps[count][max_rec] (nsteps[i] of row i used): dict of x, iterations,
    status, probe."""
    L = lib()
    steps = np.ascontiguousarray(steps, dtype=np.float64)
    nsteps = np.ascontiguousarray(nsteps, dtype=np.int32)
    count, max_rec = steps.shape
    ld = cfg.max_sections + 2
    x = np.zeros((count, ld))
    it = np.zeros(count, np.int32)
    st = np.zeros(count, np.uint8)
    pr = np.zeros((count, max(cfg.num_probe, 1)))
    i32p = C.POINTER(C.c_int32)
    L.or_ladder_replay(C.byref(cfg), seed, first, count, _dp(steps), max_rec, nsteps.ctypes.data_as(i32p), _dp(x),
                       it.ctypes.data_as(i32p), st.ctypes.data_as(C.POINTER(C.c_uint8)), _dp(pr), threads)
    return dict(x=x, iterations=it, status=st, probe=pr[:, :cfg.num_probe])


def ladder_draw(cfg, seed, inst):
    R = np.zeros(cfg.max_sections)
    Cc = np.zeros(cfg.max_sections)
    N = lib().or_ladder_draw(C.byref(cfg), seed, inst, _dp(R), _dp(Cc))
    return N, R[:N], Cc[:N]


def grid_solve(cfg, seed, count, first=0, threads=0):
    """Oracle power-grid corners: dict of x[count][rows*cols+1], newton, krylov, status, resid."""
    L = lib()
    n = cfg.rows * cfg.cols + 1
    x = np.zeros((count, n))
    nw = np.zeros(count, np.int32)
    kr = np.zeros(count, np.int32)
    st = np.zeros(count, np.uint8)
    rs = np.zeros(count)
    i32p = C.POINTER(C.c_int32)
    L.or_grid_solve(C.byref(cfg), seed, first, count, _dp(x), nw.ctypes.data_as(i32p), kr.ctypes.data_as(i32p),
                    st.ctypes.data_as(C.POINTER(C.c_uint8)), _dp(rs), threads)
    return dict(x=x, newton=nw, krylov=kr, status=st, resid=rs)


def histogram(values, col, min, max, num_bins, status=None):
    v = np.ascontiguousarray(values, dtype=np.float64)
    bins = np.zeros(num_bins, np.uint64)
    st = None if status is None else np.ascontiguousarray(status, dtype=np.uint8)
    lib().or_histogram(_dp(v), v.shape[0], v.shape[1], col, None if st is None else st.ctypes.data, min, max,
                       num_bins, bins.ctypes.data_as(C.POINTER(C.c_uint64)))
    return bins


def yield_counts(values, specs, status=None):
    """specs: [(col, lower, upper)] -> pass counts per spec and for all."""
    from spicier_gb300 import abi
    v = np.ascontiguousarray(values, dtype=np.float64)
    arr = (abi.SpYieldSpec * max(len(specs), 1))(*[abi.SpYieldSpec(c, 0, lo, hi) for c, lo, hi in specs])
    out = np.zeros(len(specs) + 1, np.uint64)
    st = None if status is None else np.ascontiguousarray(status, dtype=np.uint8)
    lib().or_yield(_dp(v), v.shape[0], v.shape[1], None if st is None else st.ctypes.data, C.addressof(arr),
                   len(specs), out.ctypes.data_as(C.POINTER(C.c_uint64)))
    return out


def transient(circuit, cfg, seed, count, method, h, tstop, probe_idx=-1, first=0, table=None, threads=0):
    """Oracle fixed-step linear transients: (x[count][nt], probe[count][steps+1] or None, status)."""
    import math
    nt = circuit.num_nodes + sum(1 for e in circuit.elements if e["kind"] == 4)
    steps = int(math.ceil(tstop / h))
    x = np.zeros((count, nt))
    pr = np.zeros((count, steps + 1)) if probe_idx >= 0 else None
    st = np.zeros(count, np.uint8)
    cols = 0
    if table is not None:
        table = np.ascontiguousarray(table, dtype=np.float64)
        cols = table.shape[1]
    cc = circuit.to_c()
    lib().or_transient(C.byref(cc), C.byref(cfg), seed, first, count, _dp(table), cols, method, h, tstop, probe_idx,
                       _dp(x), _dp(pr), st.ctypes.data_as(C.POINTER(C.c_uint8)), threads)
    return x, pr, st


def bsim3_default_card(pmos=False):
    """Bsim3Params::{nmos,pmos}_default as an sp_bsim3_card vector."""
    from spicier_gb300 import _abi as abi
    out = np.zeros(abi.SP_B3_CARD)
    lib().or_bsim3_default_card(int(pmos), _dp(out))
    return out


def bsim3_evaluate(card, bias, pmos=False):
    """Oracle BSIM3 evaluation: card[count][SP_B3_CARD], bias[count][3] ->
    (out[count][6] = ids, gds, gm, gmbs, vth, vdsat; region[count])."""
    card = np.ascontiguousarray(card, dtype=np.float64)
    bias = np.ascontiguousarray(bias, dtype=np.float64)
    n = bias.shape[0]
    out = np.zeros((n, 6))
    reg = np.zeros(n, dtype=np.uint8)
    lib().or_bsim3_evaluate(int(pmos), _dp(card), _dp(bias), n, _dp(out),
                            reg.ctypes.data_as(C.POINTER(C.c_uint8)))
    return out, reg


def ac_frequencies(fstart, fstop, num_points, sweep):
    """AC frequency grid (generate_frequencies): sweep 0 linear, 1 decade, 2 octave."""
    n = lib().or_ac_frequencies(fstart, fstop, num_points, sweep, None, 0)
    out = np.zeros(max(n, 1))
    lib().or_ac_frequencies(fstart, fstop, num_points, sweep, _dp(out), n)
    return out[:n]


def ac_sweep(circuit, cfg, seed, count, freqs, probes, source=-1, first=0, table=None, threads=0):
    """Oracle batched AC sweep: (probe[count][nf][np] complex, status[count])."""
    freqs = np.ascontiguousarray(freqs, dtype=np.float64)
    pr = np.ascontiguousarray(probes, dtype=np.int32)
    out = np.zeros((count, freqs.size, pr.size, 2))
    st = np.zeros(count, np.uint8)
    cols = 0
    if table is not None:
        table = np.ascontiguousarray(table, dtype=np.float64)
        cols = table.shape[1]
    cc = circuit.to_c()
    lib().or_ac_sweep(C.cast(C.pointer(cc), C.c_void_p), C.cast(C.pointer(cfg), C.c_void_p), seed, first, count,
                      _dp(table), cols, _dp(freqs), freqs.size, source, pr.ctypes.data_as(C.POINTER(C.c_int)),
                      pr.size, _dp(out), st.ctypes.data_as(C.POINTER(C.c_uint8)), threads)
    return out[..., 0] + 1j * out[..., 1], st

