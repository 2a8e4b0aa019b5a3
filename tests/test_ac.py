"""Batched AC small-signal sweeps (solve_ac, crates/spicier-solver/src/ac.rs):
the oracle against the reference's own AC tests, and the GPU kernel against
the oracle."""
import math

import numpy as np
import pytest

import oracle
from spicier_gb300 import abi, configs
from spicier_gb300.api import Context
from spicier_gb300.circuit import Circuit, Gauss


def test_frequency_grids_match_reference():
    # ac.rs tests: 100 linear points, 3 decades x 10 -> 31, 4 octaves x 5 -> 21
    lin = oracle.ac_frequencies(1.0, 100.0, 100, 0)
    assert lin.size == 100 and abs(lin[0] - 1.0) < 1e-10 and abs(lin[99] - 100.0) < 1e-10
    dec = oracle.ac_frequencies(1.0, 1000.0, 10, 1)
    assert dec.size == 31 and abs(dec[10] - 10.0) < 1e-6 and abs(dec[20] - 100.0) < 1e-4
    octv = oracle.ac_frequencies(100.0, 1600.0, 5, 2)
    assert octv.size == 21 and abs(octv[5] - 200.0) < 1e-6
    # the library computes the same grid
    for cfg, ref in ((abi.ac_config(1.0, 100.0, 100, abi.SP_AC_LIN), lin),
                     (abi.ac_config(1.0, 1000.0, 10, abi.SP_AC_DEC), dec),
                     (abi.ac_config(100.0, 1600.0, 5, abi.SP_AC_OCT), octv)):
        assert np.array_equal(Context.ac_frequencies(cfg), ref)


def rc_lowpass():
    c = Circuit("rc")
    c.V("V1", "in", "0", 0.0)
    c.R("R1", "in", "out", 1000.0)
    c.Cap("C1", "out", "0", 1e-6)
    return c


def rl_lowpass():
    c = Circuit("rl")
    c.V("V1", "in", "0", 0.0)
    c.L("L1", "in", "out", 0.1)
    c.R("R1", "out", "0", 1000.0)
    return c


def sweep_db(circ, node, fstart, fstop, ppd):
    f = oracle.ac_frequencies(fstart, fstop, ppd, 1)
    h, st = oracle.ac_sweep(circ, abi.newton_config(), 1, 1, f, [circ.node(node)])
    assert st[0] == 0
    return f, h[0, :, 0]


def test_rc_lowpass_3db_point_and_rolloff():
    f3db = 1.0 / (2.0 * math.pi * 1000.0 * 1e-6)
    f, h = sweep_db(rc_lowpass(), "out", 1.0, 1e6, 20)
    db = 20 * np.log10(np.abs(h))
    assert abs(db[0]) < 0.1
    k = int(np.argmin(np.abs(np.log(f / f3db))))
    assert abs(db[k] + 3.01) < 1.0
    # -20 dB per decade well above the corner, phase -45 degrees at the corner
    hi = np.nonzero(f > 10 * f3db)[0]
    d = (db[hi[-1]] - db[hi[0]]) / np.log10(f[hi[-1]] / f[hi[0]])
    assert abs(d + 20.0) < 3.0
    # the exact transfer function, to rounding
    np.testing.assert_allclose(h, 1.0 / (1.0 + 2j * math.pi * f * 1e-3), rtol=1e-12)


def test_rl_lowpass():
    f3db = 1000.0 / (2.0 * math.pi * 0.1)
    f, h = sweep_db(rl_lowpass(), "out", 10.0, 1e6, 50)
    db = 20 * np.log10(np.abs(h))
    assert abs(db[0]) < 0.5
    k = int(np.argmin(np.abs(np.log(f / f3db))))
    assert abs(db[k] + 3.01) < 1.5
    np.testing.assert_allclose(h, 1000.0 / (1000.0 + 2j * math.pi * f * 0.1), rtol=1e-12)


def test_opamp_buffer_follows_its_input():
    """The Miller op-amp as a unity-gain buffer: unity gain at low frequency from VIN, rolling off above."""
    circ = configs.miller_opamp()
    vin = [i for i, e in enumerate(circ.elements) if e["name"] == "VIN"][0]
    f = oracle.ac_frequencies(10.0, 1e9, 5, 1)
    h, st = oracle.ac_sweep(circ, abi.newton_config(), 1, 32, f, [circ.node("out")], source=vin)
    assert (st == 0).all()
    g = np.abs(h[:, :, 0])
    assert np.abs(g[:, 0] - 1.0).max() < 0.01
    assert (g[:, -1] < 0.5).all()


# --------------------------------------------------------------------------- GPU
def mc_rc_mos():
    """A MOS stage with a Monte Carlo load and an RC output filter."""
    c = Circuit("cs_rc")
    c.V("VDD", "vdd", "0", 3.3)
    c.V("VG", "g", "0", Gauss(1.2, 0.05, 0))
    c.R("RD", "vdd", "d", Gauss(10e3, 500.0, 1))
    c.M("M1", "d", "g", "0", vto=Gauss(0.7, 0.02, 2), kp=110e-6, lam=0.02)
    c.R("RF", "d", "o", 1e3)
    c.Cap("CF", "o", "0", Gauss(1e-9, 5e-11, 3))
    c.L("LS", "o", "p", 1e-6)
    c.R("RL", "p", "0", 50e3)
    return c


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cs_rc", "opamp"])
def test_exact_mode_bitwise(ctx, name):
    circ = mc_rc_mos() if name == "cs_rc" else configs.miller_opamp()
    probes = [0, 2, circ.n - 1] if name == "cs_rc" else [circ.node("out"), circ.node("n1"), circ.n - 1]
    cfg = abi.ac_config(1e2, 1e9, 8, abi.SP_AC_DEC, probes)
    dc = abi.newton_config(precision=abi.SP_PREC_FP64_EXACT)
    count = 1024
    h, st = ctx.ac_sweep(circ, dc, cfg, 5, count)
    with oracle.math_mode("cr"):
        ho, so = oracle.ac_sweep(circ, dc, 5, count, Context.ac_frequencies(cfg), probes)
    assert np.array_equal(st, so)
    ok = (st & 0x0F) == 0
    assert ok.mean() > 0.95
    assert np.array_equal(h[ok].view(np.uint64), ho[ok].view(np.uint64))


@pytest.mark.gpu
def test_bjt_diode_and_device_entry(ctx):
    import torch
    circ = configs.bjt_diode_bias()
    circ.Cap("CB", "b", "0", 1e-9)
    circ.Cap("CD", "d", "0", 1e-10)
    probes = [circ.node("c"), circ.node("d")]
    cfg = abi.ac_config(1e3, 1e10, 10, abi.SP_AC_DEC, probes)
    dc = abi.newton_config(precision=abi.SP_PREC_FP64)
    h, st = ctx.ac_sweep(circ, dc, cfg, 2, 512)
    ho, so = oracle.ac_sweep(circ, dc, 2, 512, Context.ac_frequencies(cfg), probes)
    assert (st == 0).all() and (so == 0).all()
    np.testing.assert_allclose(h, ho, rtol=1e-9, atol=1e-15)
    # device-buffer entry point, same numbers
    topo = ctx.topology(circ)
    nf = len(Context.ac_frequencies(cfg))
    pd = torch.zeros(512, nf, 2, 2, dtype=torch.float64, device="cuda")
    sd = torch.zeros(512, dtype=torch.uint8, device="cuda")
    ctx.ac_sweep_device(topo, dc, cfg, 2, 512, pd, sd)
    torch.cuda.synchronize()
    g = pd.cpu().numpy()
    assert np.array_equal((g[..., 0] + 1j * g[..., 1]).view(np.uint64), h.view(np.uint64))


@pytest.mark.gpu
def test_ac_errors(ctx):
    import spicier_gb300 as sg
    circ = rc_lowpass()
    with pytest.raises(sg.SpicierError):
        ctx.ac_sweep(circ, abi.newton_config(), abi.ac_config(1.0, 10.0, 5, probes=(7,)), 1, 4)
    with pytest.raises(sg.SpicierError):
        ctx.ac_sweep(circ, abi.newton_config(), abi.ac_config(0.0, 10.0, 5), 1, 4)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["opamp", "bjt"])
def test_mixed_precision_against_fp64_oracle(ctx, name):
    """FP32 complex LU with FP64 residual refinement: within 1e-9 of the FP64 oracle."""
    if name == "opamp":
        circ = configs.miller_opamp()
        probes = [circ.node("out"), circ.node("n2"), circ.n - 1]
    else:
        circ = configs.bjt_diode_bias()
        circ.Cap("CB", "b", "0", 1e-9)
        circ.L("LC", "c", "c2", 1e-6)
        circ.R("RC2", "c2", "0", 1e5)
        probes = [circ.node("c"), circ.node("c2"), circ.n - 1]
    cfg = abi.ac_config(1e1, 1e10, 10, abi.SP_AC_DEC, probes, precision=abi.SP_PREC_MIXED)
    dc = abi.newton_config(precision=abi.SP_PREC_FP64)
    h, st = ctx.ac_sweep(circ, dc, cfg, 3, 1024)
    ho, so = oracle.ac_sweep(circ, dc, 3, 1024, Context.ac_frequencies(cfg), probes)
    ok = (so & 0x0F) == 0
    assert np.array_equal(st, so) and ok.mean() > 0.95
    scale = np.abs(ho[ok]).max(axis=1, keepdims=True)
    assert (np.abs(h[ok] - ho[ok]) <= 1e-9 * scale + 1e-18).all()
