"""Batched fixed-step linear transients (solve_transient, transient/solver.rs):
the oracle against the reference's own RC / LC test expectations
(transient/mod.rs tests), and the GPU kernel against the oracle."""
import math

import numpy as np
import pytest

import oracle
from spicier_gb300 import abi
from spicier_gb300.circuit import Circuit, Gauss, LogUniform, Pulse

METHODS = {"be": abi.SP_TRAN_BE, "trap": abi.SP_TRAN_TRAP, "trbdf2": abi.SP_TRAN_TRBDF2}
STEP = Pulse(0.0, 5.0, 0.0, 1e-12, 1e-12, 1.0, 2.0)  # 0 -> 5 V at t = 0+, held


def rc_circuit():
    """V1 (DC 0, PULSE to 5 V) - R 1k - C 1 uF to ground: tau = 1 ms (mod.rs:100-140)."""
    c = Circuit("rc")
    c.V("V1", "in", "0", 0.0, pulse=STEP)
    c.R("R1", "in", "out", 1000.0)
    c.Cap("C1", "out", "0", 1e-6)
    return c


def rlc_circuit():
    """Underdamped series RLC (R 1 ohm, L 1 mH, C 1 uF): f0 = 5033 Hz, the LC tank of mod.rs:451."""
    c = Circuit("rlc")
    c.V("V1", "in", "0", 0.0, pulse=STEP)
    c.R("R1", "in", "a", 1.0)
    c.L("L1", "a", "b", 1e-3)
    c.Cap("C1", "b", "0", 1e-6)
    return c


def mc_circuit():
    """Monte Carlo RLC network with two V sources, a current source and a table-free draw of every value."""
    c = Circuit("mc")
    c.V("V1", "in", "0", 0.0, pulse=Pulse(0.0, 1.0, 2e-6, 1e-6, 1e-6, 10e-6, 40e-6))
    c.R("R1", "in", "a", Gauss(100.0, 5.0, 0))
    c.L("L1", "a", "b", LogUniform(1e-6, 1e-5, 1))
    c.Cap("C1", "b", "0", LogUniform(1e-9, 1e-8, 2))
    c.R("R2", "b", "c", Gauss(200.0, 10.0, 3))
    c.Cap("C2", "c", "0", LogUniform(1e-9, 1e-8, 4))
    c.R("R3", "c", "bias", 1e3)
    c.V("V2", "bias", "0", Gauss(0.5, 0.01, 5))
    c.I("I1", "0", "c", 1e-4, pulse=Pulse(0.0, 1e-4, 5e-6, 1e-6, 1e-6, 5e-6, 20e-6))
    c.L("L2", "c", "d", 2e-6)
    c.R("R4", "d", "0", Gauss(50.0, 2.0, 6))
    return c


def run_oracle(circ, method, h, tstop, probe, count=1, seed=1, mode=None):
    cfg = abi.newton_config()
    if mode:
        with oracle.math_mode(mode):
            return oracle.transient(circ, cfg, seed, count, method, h, tstop, probe_idx=probe)
    return oracle.transient(circ, cfg, seed, count, method, h, tstop, probe_idx=probe)


# ------------------------------------------------------- reference expectations
@pytest.mark.parametrize("name,final_tol,tau_tol", [("be", 0.05, 0.2), ("trap", 0.05, 0.1),
                                                     ("trbdf2", 0.15, 0.6)])
def test_rc_charging(name, final_tol, tau_tol):
    circ = rc_circuit()
    out = circ.node("out")
    x, pr, st = run_oracle(circ, METHODS[name], 10e-6, 5e-3, out)
    assert st[0] == 0
    assert abs(x[0, out] - 5.0) < final_tol
    assert pr[0, 0] == 0.0  # DC operating point: source at its DC value 0 V
    tau = 5.0 * (1.0 - math.exp(-1.0))
    assert abs(pr[0, 100] - tau) < tau_tol
    # the closed-form BE recurrence v_k = 5 (1 - (1 + h/tau)^-k)
    if name == "be":
        k = np.arange(pr.shape[1])
        np.testing.assert_allclose(pr[0], 5.0 * (1.0 - (1.0 + 0.01) ** -k), rtol=0, atol=1e-12)


def test_rlc_oscillation_frequency():
    circ = rlc_circuit()
    b = circ.node("b")
    f0 = 1.0 / (2.0 * math.pi * math.sqrt(1e-3 * 1e-6))
    per = 1.0 / f0
    h = per / 50.0
    x, pr, st = run_oracle(circ, abi.SP_TRAN_TRAP, h, 5.0 * per, b)
    assert st[0] == 0
    v = pr[0] - 5.0
    t = np.arange(v.size) * h
    cross = [t[i - 1] - v[i - 1] * (t[i] - t[i - 1]) / (v[i] - v[i - 1])
             for i in range(1, v.size) if v[i - 1] > 0 >= v[i]]
    assert len(cross) >= 2
    f = 1.0 / (cross[1] - cross[0])
    assert abs(f - f0) / f0 < 0.05
    # trapezoidal keeps the tank's energy: the swing barely decays over five periods (Q = 31.6)
    assert pr[0].max() > 9.0


def test_oracle_math_modes_agree():
    circ = mc_circuit()
    for method in METHODS.values():
        a, pa, sa = run_oracle(circ, method, 0.2e-6, 20e-6, circ.node("c"), count=16, mode="cr")
        b, pb, sb = run_oracle(circ, method, 0.2e-6, 20e-6, circ.node("c"), count=16)
        assert (sa == 0).all() and (sb == 0).all()
        assert np.abs(a - b).max() < 1e-12 and np.abs(pa - pb).max() < 1e-12


# --------------------------------------------------------------------------- GPU
GPU_COUNT = 2048


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(METHODS))
def test_exact_mode_bitwise(ctx, name):
    circ = mc_circuit()
    probe = circ.node("c")
    cfg = abi.transient_config(0.2e-6, 30e-6, METHODS[name], probe, abi.SP_PREC_FP64_EXACT)
    dc = abi.newton_config(precision=abi.SP_PREC_FP64_EXACT)
    g = ctx.transient(circ, dc, cfg, 1, GPU_COUNT)
    with oracle.math_mode("cr"):
        x, pr, st = oracle.transient(circ, dc, 1, GPU_COUNT, METHODS[name], 0.2e-6, 30e-6, probe_idx=probe)
    assert np.array_equal(g["status"], st)
    assert np.array_equal(g["x"].view(np.uint64), x.view(np.uint64))
    assert np.array_equal(g["probe"].view(np.uint64), pr.view(np.uint64))


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(METHODS))
def test_fp64_against_oracle(ctx, name):
    circ = mc_circuit()
    probe = circ.node("b")
    cfg = abi.transient_config(0.2e-6, 30e-6, METHODS[name], probe, abi.SP_PREC_FP64)
    dc = abi.newton_config()
    g = ctx.transient(circ, dc, cfg, 7, GPU_COUNT, first=100)
    x, pr, st = oracle.transient(circ, dc, 7, GPU_COUNT, METHODS[name], 0.2e-6, 30e-6, probe_idx=probe, first=100)
    assert (g["status"] == 0).all() and (st == 0).all()
    scale = np.abs(pr).max()
    assert np.abs(g["x"] - x).max() <= 1e-9 * max(1.0, np.abs(x).max())
    assert np.abs(g["probe"] - pr).max() <= 1e-9 * max(1.0, scale)


@pytest.mark.gpu
def test_device_entry_and_reference_ranges(ctx):
    import torch
    import spicier_gb300 as sg
    circ = rc_circuit()
    out = circ.node("out")
    topo = ctx.topology(circ)
    cfg = abi.transient_config(10e-6, 5e-3, abi.SP_TRAN_TRAP, out, abi.SP_PREC_FP64)
    n = 256
    x = torch.zeros(n, 2 + 1, dtype=torch.float64, device="cuda")
    st = torch.zeros(n, dtype=torch.uint8, device="cuda")
    pr = torch.zeros(n, 501, dtype=torch.float64, device="cuda")
    ctx.transient_device(topo, abi.newton_config(), cfg, 1, n, x, st, probe=pr)
    torch.cuda.synchronize()
    assert (st == 0).all()
    assert (x[:, out] - 5.0).abs().max().item() < 0.05
    assert (pr[:, 100] - 5.0 * (1.0 - math.exp(-1.0))).abs().max().item() < 0.1
    # nonlinear circuits are rejected (solve_transient takes linear stampers)
    d = Circuit("d")
    d.V("V1", "a", "0", 1.0)
    d.R("R1", "a", "b", 1e3)
    d.D("D1", "b", "0")
    with pytest.raises(sg.SpicierError):
        ctx.transient(d, abi.newton_config(), cfg, 1, 4)
    with pytest.raises(sg.SpicierError):
        ctx.transient(circ, abi.newton_config(), abi.transient_config(0.0, 1e-3), 1, 4)
