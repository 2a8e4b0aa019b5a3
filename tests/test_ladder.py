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
    """512 shorter ladders: every instance against the oracle replayed along
    the GPU's accepted steps (FP64 1e-9 relative, MIXED the SPICE tolerance
    per node)."""
    cfg = small_cfg(precision=prec)
    g = ctx.ladder_transient_steps(cfg, 1, GPU_COUNT)
    assert (g["status"] == 0).all()
    with oracle.math_mode("cr"):
        rep = oracle.ladder_replay(small_cfg(), 1, g["steps"], g["accepted"])
    tol_units, rel = node_errors(g["x"], rep["x"], g["n"])
    if prec == abi.SP_PREC_FP64:
        assert rel.max() < 1e-9, rel.max()
    else:
        assert tol_units.max() <= 1.0, tol_units.max()


# --------------------------------------------------------------------------- full size
# 64 consecutive instances of the workload draw (8..512 sections) around the
# first 512-section ladder of seed 1 (instance 1761), so the longest ladder
# and the whole range of lengths are compared against the oracle.
FULL_FIRST, FULL_COUNT, LONGEST = 1729, 64, 1761
NODE_RELTOL, VNTOL, ABSTOL = 1e-3, 1e-6, 1e-12  # the spec SPICE tolerances


def test_full_window_holds_the_longest_ladder():
    cfg = abi.ladder_config()
    Ns = [oracle.ladder_draw(cfg, 1, FULL_FIRST + i)[0] for i in range(FULL_COUNT)]
    assert oracle.ladder_draw(cfg, 1, LONGEST)[0] == 512 and max(Ns) == 512 and min(Ns) < 64


def test_oracle_replay_reproduces_its_own_run():
    """Replaying the oracle's accepted steps gives its adaptive run bit for bit
    (the replay is the adaptive arithmetic without the step controller)."""
    cfg = abi.ladder_config(num_probe=101)
    with oracle.math_mode("cr"):
        nat = oracle.ladder_transient(cfg, 1, 8, first=LONGEST - 4)
        steps, ns = oracle.ladder_steps(cfg, 1, 8, first=LONGEST - 4)
        rep = oracle.ladder_replay(cfg, 1, steps, ns, first=LONGEST - 4)
    assert np.array_equal(ns, nat["accepted"])
    assert np.array_equal(rep["x"].view(np.uint64), nat["x"].view(np.uint64))
    assert np.array_equal(rep["probe"].view(np.uint64), nat["probe"].view(np.uint64))


def node_errors(a, b, n):
    """Per instance: the largest error in units of the SPICE tolerance
    (reltol |x| + vntol per node voltage, reltol |I| + abstol for the source
    current), and the largest relative error."""
    tol_units, rel = [], []
    for i in range(len(n)):
        N = n[i] - 2
        va, vb = a[i, :N + 1], b[i, :N + 1]
        tv = np.abs(va - vb) / (NODE_RELTOL * np.maximum(np.abs(va), np.abs(vb)) + VNTOL)
        ti = abs(a[i, N + 1] - b[i, N + 1]) / (NODE_RELTOL * max(abs(a[i, N + 1]), abs(b[i, N + 1])) + ABSTOL)
        tol_units.append(max(tv.max(), ti))
        rel.append((np.abs(a[i, :N + 2] - b[i, :N + 2]) / np.maximum(np.abs(b[i, :N + 2]), 1e-12)).max())
    return np.array(tol_units), np.array(rel)


@pytest.fixture(scope="module")
def full_oracle():
    cfg = abi.ladder_config(num_probe=101)
    with oracle.math_mode("cr"):
        o = oracle.ladder_transient(cfg, 1, FULL_COUNT, first=FULL_FIRST)
        o["steps"], _ = oracle.ladder_steps(cfg, 1, FULL_COUNT, first=FULL_FIRST)
    return o


@pytest.mark.gpu
def test_full_size_exact_bitwise(ctx, full_oracle):
    """FP64_EXACT on the full range of lengths, the longest ladder included:
    final state, probe waveform, step counts and Newton iterations bitwise."""
    cfg = abi.ladder_config(precision=abi.SP_PREC_FP64_EXACT, num_probe=101)
    g = ctx.ladder_transient_steps(cfg, 1, FULL_COUNT, first=FULL_FIRST)
    o = full_oracle
    for k in ("n", "accepted", "rejected", "iterations", "status"):
        assert np.array_equal(g[k], o[k]), k
    assert np.array_equal(g["x"].view(np.uint64), o["x"].view(np.uint64))
    assert np.array_equal(g["probe"].view(np.uint64), o["probe"].view(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [abi.SP_PREC_FP64, abi.SP_PREC_MIXED])
def test_full_size_against_oracle(ctx, full_oracle, prec):
    """FP64 and MIXED on the full range of lengths.  The adaptive step
    sequence is a discontinuous function of the last bits of the LTE, so an
    instance may take other steps than the oracle; every instance is
    therefore compared with the oracle replayed along the GPU's own accepted
    steps (same step sizes, the oracle's FP64 arithmetic): FP64 within 1e-9
    relative, MIXED within the SPICE tolerance per node.  Instances on the
    oracle's own step sequence are also compared with its adaptive run, with
    the same bars."""
    cfg = abi.ladder_config(precision=prec, num_probe=101)
    g = ctx.ladder_transient_steps(cfg, 1, FULL_COUNT, first=FULL_FIRST)
    assert (g["status"] == 0).all() and np.array_equal(g["n"], full_oracle["n"])
    assert (g["accepted"] <= g["steps"].shape[1]).all()
    with oracle.math_mode("cr"):
        rep = oracle.ladder_replay(abi.ladder_config(num_probe=101), 1, g["steps"], g["accepted"], first=FULL_FIRST)
    assert (rep["status"] == 0).all()
    tol_units, rel = node_errors(g["x"], rep["x"], g["n"])
    if prec == abi.SP_PREC_FP64:
        assert rel.max() < 1e-9, rel.max()
        assert np.abs(g["probe"] - rep["probe"]).max() < 1e-9
    else:
        assert tol_units.max() <= 1.0, tol_units.max()
        assert np.abs(g["probe"] - rep["probe"]).max() <= NODE_RELTOL * 1.8 + VNTOL
    o = full_oracle
    # on the oracle's step sequence: the same accepted and rejected counts and
    # every accepted step close to the oracle's (the step size feeds back
    # through the LTE, so rounding differences grow along the run: FP64 to
    # 1e-10 relative, MIXED to 1e-6)
    same = (g["accepted"] == o["accepted"]) & (g["rejected"] == o["rejected"])
    w = g["steps"].shape[1]
    srel = np.max(np.abs(g["steps"] - o["steps"][:, :w]) / np.maximum(np.abs(o["steps"][:, :w]), 1e-300), axis=1)
    same &= srel <= (1e-10 if prec == abi.SP_PREC_FP64 else 1e-6)
    assert same.mean() >= 0.5, same.mean()
    tol_nat, rel_nat = node_errors(g["x"][same], o["x"][same], g["n"][same])
    if prec == abi.SP_PREC_FP64:
        assert rel_nat.max() < 1e-9, rel_nat.max()
    else:
        assert tol_nat.max() <= 1.0, tol_nat.max()


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
