"""Batched RC-diode ladder transients (TR-BDF2 stages under the adaptive
controller, Newton per stage): the oracle on the CPU, and the GPU kernel
against it in every precision."""
import ctypes as C

import numpy as np
import pytest

import oracle
from spicier_gb300 import abi
from spicier_gb300._lib import load

GPU_COUNT = 512


def small_cfg(**kw):
    """The workload's settings with shorter ladders, so the oracle finishes in seconds."""
    kw.setdefault("max_sections", 96)
    return abi.ladder_config(**kw)


def test_default_config_matches_library():
    c = abi.SpLadderConfig()
    load().sp_ladder_config_default(C.byref(c))
    d = abi.ladder_config()
    for f, _ in abi.SpLadderConfig._fields_:
        if f != "pulse":
            assert getattr(c, f) == getattr(d, f), f
    assert bytes(c.pulse) == bytes(d.pulse)


def test_draws_follow_the_workload_distribution():
    cfg = abi.ladder_config()
    Ns, Rs, Cs = [], [], []
    for i in range(400):
        N, R, Cc = oracle.ladder_draw(cfg, 1, i)
        Ns.append(N)
        Rs.extend(R)
        Cs.extend(Cc)
    Ns, Rs, Cs = np.array(Ns), np.array(Rs), np.array(Cs)
    assert Ns.min() >= 8 and Ns.max() <= 512 and abs(Ns.mean() - 260) < 20
    assert Rs.min() >= 100 and Rs.max() <= 10e3 and abs(np.log(Rs).mean() - np.log(1e3)) < 0.05
    assert Cs.min() >= 1e-12 and Cs.max() <= 100e-12 and abs(np.log(Cs).mean() - np.log(1e-11)) < 0.05


def test_oracle_math_modes_agree_and_physics_holds():
    cfg = small_cfg()
    with oracle.math_mode("cr"):
        a = oracle.ladder_transient(cfg, 1, 48, threads=4)
    b = oracle.ladder_transient(cfg, 1, 48, threads=4)  # host libm
    assert (a["status"] == 0).all() and (b["status"] == 0).all()
    assert np.array_equal(a["accepted"], b["accepted"]) and np.array_equal(a["rejected"], b["rejected"])
    assert np.abs(a["x"] - b["x"]).max() < 1e-12
    x, n = a["x"], a["n"]
    for i in range(48):
        N = n[i] - 2
        v = x[i, :N + 1]
        assert v[0] == 0.0  # the pulse is back at v1 = 0 V at t = 100 ns (five periods)
        assert (v <= 1.8 + 1e-9).all() and (v >= -1e-3).all()
        # branch current from the KCL of the source node
        _, R, _ = oracle.ladder_draw(cfg, 1, i)
        assert abs(x[i, N + 1] - (v[1] - v[0]) / R[0]) <= 1e-12 + 1e-9 * abs(x[i, N + 1])
    assert (a["probe"][:, 0] == 0).all()
    assert a["accepted"].min() >= 100  # h_max = tstop / 100


def test_step_control_shrinks_at_the_pulse_edges():
    cfg = small_cfg(num_probe=0)
    r = oracle.ladder_transient(cfg, 1, 8, threads=2)
    # fewer steps when the integration has to resolve only smooth input (slow edges)
    slow = small_cfg(num_probe=0)
    slow.pulse.tr = slow.pulse.tf = 5e-9
    s = oracle.ladder_transient(slow, 1, 8, threads=2)
    assert s["accepted"].mean() < r["accepted"].mean()


# --------------------------------------------------------------------------- GPU
def gpu_run(ctx, cfg, seed=1, count=GPU_COUNT, first=0):
    return ctx.ladder_transient(cfg, seed, count, first=first)


@pytest.mark.gpu
def test_exact_mode_bitwise(ctx):
    cfg = small_cfg(precision=abi.SP_PREC_FP64_EXACT)
    g = gpu_run(ctx, cfg)
    with oracle.math_mode("cr"):
        o = oracle.ladder_transient(cfg, 1, GPU_COUNT)
    for k in ("n", "accepted", "rejected", "iterations", "status"):
        assert np.array_equal(g[k], o[k]), k
    assert np.array_equal(g["x"].view(np.uint64), o["x"].view(np.uint64))
    assert np.array_equal(g["probe"].view(np.uint64), o["probe"].view(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [abi.SP_PREC_FP64, abi.SP_PREC_MIXED])
def test_fast_modes_against_oracle(ctx, prec):
    cfg = small_cfg(precision=prec)
    g = gpu_run(ctx, cfg)
    with oracle.math_mode("cr"):
        o = oracle.ladder_transient(cfg, 1, GPU_COUNT)
    assert (g["status"] == 0).all() and np.array_equal(g["n"], o["n"])
    # the adaptive step sequence is a discontinuous function of the last bits;
    # most instances take exactly the oracle's steps, the rest stay within the
    # integration tolerance (reltol 1e-3 of 1.8 V)
    err = np.abs(g["x"] - o["x"])[:, :-1].max(1)
    if prec == abi.SP_PREC_FP64:
        assert (err < 1e-9).mean() > 0.5  # the oracle's step sequence, to rounding
    assert (g["accepted"] == o["accepted"]).mean() > 0.5
    assert err.max() < 5e-3
    assert np.abs(g["probe"] - o["probe"]).max() < 5e-3


@pytest.mark.gpu
def test_full_workload_sizes(ctx):
    """Full section range (8..512) on 256 instances: completes, same sizes as the oracle."""
    cfg = abi.ladder_config(precision=abi.SP_PREC_MIXED, num_probe=11)
    g = gpu_run(ctx, cfg, count=256, first=1000)
    assert (g["status"] == 0).all()
    n = np.array([oracle.ladder_draw(cfg, 1, 1000 + i)[0] + 2 for i in range(256)])
    assert np.array_equal(g["n"], n)
    assert (g["accepted"] >= 100).all()


@pytest.mark.gpu
def test_ladder_errors(ctx):
    import spicier_gb300 as sg
    with pytest.raises(sg.SpicierError):
        ctx.ladder_transient(abi.ladder_config(max_sections=5000), 1, 4)
    with pytest.raises(sg.SpicierError):
        ctx.ladder_transient(abi.ladder_config(h_min=0.0), 1, 4)
