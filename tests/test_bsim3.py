"""BSIM3v3.3 DC model (crates/spicier-devices/src/mosfet/bsim3/): the oracle
against the reference's own evaluate tests (evaluate.rs:600-930), its stated
calibration and amplifier result, and the ngspice golden netlists
(crates/spicier-parser/tests/golden_data/dc_bsim3.json, as the reference's
ngspice_validation.rs:5394-5520 runs them); then the GPU evaluation and the
Newton kernels against the oracle."""
import json
import os

import numpy as np
import pytest

import oracle
from spicier_gb300 import abi, configs
from spicier_gb300.circuit import BSIM3_DEFAULTS, Circuit, Gauss
from spicier_gb300.netlist import parse_netlist

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "bsim3_dc.json")
K = {n: i for i, n in enumerate(abi.BSIM3_CARD)}


def card(pmos=False, **kw):
    c = oracle.bsim3_default_card(pmos)
    for k, v in kw.items():
        c[K[k]] = v
    return c


def ev(c, vgs, vds, vbs=0.0, pmos=False):
    out, reg = oracle.bsim3_evaluate(c[None], np.array([[vgs, vds, vbs]]), pmos)
    o = out[0]
    return dict(ids=o[0], gds=o[1], gm=o[2], gmbs=o[3], vth=o[4], vdsat=o[5], region=int(reg[0]))


def test_default_cards_agree():
    for pmos in (False, True):
        assert np.array_equal(oracle.bsim3_default_card(pmos),
                              np.array([BSIM3_DEFAULTS[pmos][k] for k in abi.BSIM3_CARD]))


def test_reference_evaluate_tests():
    n = card()
    # test_subthreshold
    vth = ev(n, 0.5, 0.1)["vth"]
    r = ev(n, min(vth - 0.2, 0.1), 0.1)
    assert r["region"] == 0 and 0.0 < r["ids"] < 1e-5
    # test_saturation
    r = ev(n, 1.0, 1.0)
    assert r["region"] == 2 and 10e-6 < r["ids"] < 10e-3 and r["gm"] > 0 and r["gds"] > 0
    # test_linear
    r = ev(n, 1.0, 0.1)
    assert r["region"] == 1 and r["ids"] > 0 and r["gds"] > r["gm"] * 0.1
    # test_body_effect
    a, b = ev(n, 1.0, 1.0, 0.0), ev(n, 1.0, 1.0, -1.0)
    assert b["vth"] > a["vth"] and b["ids"] < a["ids"]
    # test_pmos
    r = ev(card(True), -1.0, -1.0, 0.0, pmos=True)
    assert r["region"] == 2 and r["ids"] < 0
    # test_continuity_at_vdsat
    vdsat = ev(n, 1.0, 1.0)["vdsat"]
    lo, hi = ev(n, 1.0, vdsat * 0.95), ev(n, 1.0, vdsat * 1.05)
    assert lo["region"] == 1 and hi["region"] == 2 and 0.8 < hi["ids"] / lo["ids"] < 1.2
    # test_short_channel_effect
    s, l_ = ev(card(l=50e-9), 1.0, 0.1), ev(card(l=500e-9), 1.0, 0.1)
    assert s["vth"] < l_["vth"] and s["ids"] > 0 and l_["ids"] > 0
    # test_dibl
    assert ev(n, 0.6, 1.0)["vth"] < ev(n, 0.6, 0.1)["vth"]
    # test_narrow_width_effect
    wide, narrow = ev(card(w=1e-6, k3=10.0), 1.0, 0.5), ev(card(w=100e-9, k3=10.0), 1.0, 0.5)
    assert narrow["vth"] > wide["vth"] and narrow["ids"] < wide["ids"]
    # test_enhanced_dibl_body_effect
    p = card(pdiblcb=0.5)
    a, b = ev(p, 1.0, 1.0, 0.0), ev(p, 1.0, 1.0, -0.5)
    assert a["ids"] > 0 and b["ids"] > 0 and a["gds"] > 0 and b["gds"] > 0


def test_ngspice_comparison_and_stated_calibration():
    """test_ngspice_comparison (evaluate.rs:664-708): Vth within 10 %, Vdsat
    within 20 %, Ids within 50 % of ngspice-45; calc_mobility's comment states
    the calibration reached (Ids within 5 %, Vdsat within 2 %), which pins the
    restated mobility, threshold and Vdsat expressions much tighter."""
    r = ev(card(), 1.0, 1.0)
    assert abs(r["vth"] - 0.344833) / 0.344833 < 0.10
    assert abs(r["vdsat"] - 0.313407) / 0.313407 < 0.02
    assert abs(r["ids"] - 280.769e-6) / 280.769e-6 < 0.05


def solve_netlist(text, count=1, prec=None):
    nl = parse_netlist(text)
    x, it, st, _ = oracle.newton_dc(nl.circuit, abi.newton_config(), seed=1, count=count)
    return nl.circuit, x, st


def test_reference_amplifier_result():
    """ngspice_validation.rs test_bsim3_nmos_amplifier: VDD enforced and the
    drain pulled below VDD - 0.1 V by a conducting device.  (A comment there
    quotes V(drain) = 0.44 V, i.e. 572 uA, which no longer matches the model it
    tests: that model gives 295 uA at Vgs = Vds = 1 V, the 5 % of ngspice its
    mobility comment states, and this amplifier settles at 1.30 V, 400 uA.)"""
    circ, x, st = solve_netlist("""BSIM3 NMOS Amplifier
.MODEL NMOD NMOS LEVEL=49 VTH0=0.4 K1=0.5 U0=670 TOX=9e-9 VSAT=1.5e5
VDD 1 0 DC 3.3
VGS 2 0 DC 1.0
RD 1 3 5k
M1 3 2 0 0 NMOD W=1u L=100n
.end""")
    assert st[0] == 0
    vd = x[0, circ.node("3")]
    assert abs(x[0, circ.node("1")] - 3.3) < 0.01 and 0.0 < vd < 3.3 - 0.1
    assert abs(vd - 1.298) < 0.001


def test_golden_netlists():
    """The ngspice golden netlists with the reference's model: the sources are
    enforced (the reference's assertions), and currents and node voltages lie
    within the file's tolerances where the simplified model reaches them.  It
    does not in weak inversion (about a sixth of ngspice's current), and the
    inverter netlist, whose PMOS has source and drain exchanged, does not
    converge: the exchange in evaluate (evaluate.rs:190-195, 248-262) keeps
    the current's sign, so that pull-up drives the wrong way (the reference's
    tests do not run this netlist)."""
    g = json.load(open(GOLDEN))
    within = {}
    for c in g["circuits"]:
        circ, x, st = solve_netlist(c["netlist"])
        if c["name"] == "bsim3_cmos_inverter":
            assert st[0] & abi.SP_ST_MASK == abi.SP_ST_FAILED
            continue
        assert st[0] == 0, c["name"]
        names = {nm.upper(): v for nm, v in zip(circ.unknown_names(), x[0])}
        for key, ref in c["results"].items():
            tol = c["tolerances"]["current" if key.startswith("I(") else "voltage"]
            within[c["name"]] = bool(abs(names[key.upper()] - ref) <= tol * abs(ref))
    assert within == {"bsim3_nmos_saturation": True, "bsim3_nmos_linear": True,
                      "bsim3_nmos_subthreshold": False, "bsim3_nmos_resistive_load": True}


def test_reference_inverter_transfer():
    """parse_and_simulate.rs test_bsim3_cmos_inverter: at least 4 of the 5
    inputs converge (Vin = 0.3 V, both devices in weak inversion, is the one
    the reference expects to miss), Vout high at the first converged low
    input, low at Vin = Vdd, and non-increasing within 0.05 V."""
    res = []
    for vin in (0.3, 0.5, 0.9, 1.4, 1.8):
        circ, x, st = solve_netlist(f"""BSIM3 CMOS Inverter
.MODEL NMOD NMOS LEVEL=49 VTH0=0.4 U0=400 TOX=9e-9 K1=0.5 VSAT=1.5e5
.MODEL PMOD PMOS LEVEL=49 VTH0=-0.4 U0=150 TOX=9e-9 K1=0.5 VSAT=1.0e5
Vdd vdd 0 DC 1.8
Vin in 0 DC {vin}
Mp out in vdd vdd PMOD W=2u L=100n
Mn out in 0 0 NMOD W=1u L=100n
Rload out 0 100Meg
.end""")
        res.append((vin, x[0, circ.node("out")], st[0] == 0))
    conv = [(v, o) for v, o, c in res if c]
    assert len(conv) >= 4 and not res[0][2]
    assert conv[0][1] > 1.8 * 0.6 and res[4][1] < 1.8 * 0.2 and res[4][2]
    assert all(b[1] <= a[1] + 0.05 for a, b in zip(conv, conv[1:]))


def test_netlist_card_and_variations():
    nl = parse_netlist(""".model parse
.MODEL NMOD NMOS LEVEL=8 VTHO=0.45 UO=600 DL=5n TNOM=27 VOFF=-0.1 CJ=1e-3
M1 d g 0 b NMOD W=2u L=200n NF=2
V1 d 0 1.0
V2 g 0 1.0
V3 b 0 -0.5
.end""", {"M1.vth0": Gauss(0.45, 0.01, 0)})
    c = nl.circuit
    el = [e for e in c.elements if e["name"] == "M1"][0]
    assert el["kind"] == abi.SP_EL_BSIM3N and el["node"][3] == c.node("b")
    base = el["field"][0]
    vals = {abi.BSIM3_CARD[k]: c.params[base + k] for k in range(abi.SP_B3_CARD)}
    assert vals["vth0"][0] == abi.SP_DRAW_GAUSS
    assert vals["u0"][2] == 600.0 and vals["lint"][2] == 5e-9 and vals["tnom"][2] == 27 + 273.15
    assert vals["w"][2] == 2e-6 and vals["l"][2] == 200 * 1e-9 and vals["nf"][2] == 2.0
    with pytest.raises(Exception):
        parse_netlist("x\n.MODEL N4 NMOS LEVEL=54\nM1 d g 0 0 N4\n.end")


def test_cmos_chain_oracle():
    """The Monte Carlo BSIM3 chain converges from its nodeset in the oracle
    (PMOS in the reference's source-at-VDD orientation)."""
    circ = configs.bsim3_cmos_chain()
    x, it, st, _ = oracle.newton_dc(circ, abi.newton_config(), seed=4, count=256)
    assert ((st & abi.SP_ST_MASK) == 0).all() and (st == 0).mean() > 0.9  # a few through gmin stepping
    mid, out = x[:, circ.node("mid")], x[:, circ.node("out")]
    assert (mid > 0.0).all() and (mid < 1.8).all() and (out > 0.0).all() and (out <= 1.8 + 1e-9).all()


def cs_amp_with_caps():
    """BSIM3 common-source stage with overlap and junction capacitances, a
    source-follower BSIM3 load on the output and Monte Carlo thresholds."""
    c = Circuit("bsim3_cs_ac")
    c.V("VDD", "vdd", "0", 1.8)
    c.V("VG", "g", "0", Gauss(0.75, 0.02, 0))
    c.R("RD", "vdd", "d", Gauss(5e3, 100.0, 1))
    c.B3("M1", "d", "g", "0", "0", vth0=Gauss(0.4, 0.02, 2), cgso=3e-10, cgdo=3e-10, cgbo=1e-10, cjswg=2e-10)
    c.B3("M2", "vdd", "d", "out", "0", vth0=Gauss(0.4, 0.02, 3), w=2e-6, cgso=3e-10, cgdo=3e-10)
    c.R("RS", "out", "0", 20e3)
    c.nodeset = {"d": 0.9, "out": 0.3}
    return c


def test_ac_low_frequency_gain_matches_dc_model():
    """At 1 kHz the stage gain is -gm / (gds + 1/RD + load) of the DC model at the
    operating point; at 100 GHz the capacitances have rolled it off."""
    circ = cs_amp_with_caps()
    f = oracle.ac_frequencies(1e3, 1e11, 1, 1)
    vg = [i for i, e in enumerate(circ.elements) if e["name"] == "VG"][0]
    h, st = oracle.ac_sweep(circ, abi.newton_config(), 2, 8, f, [circ.node("d")], source=vg)
    x, _, sx, P = oracle.newton_dc(circ, abi.newton_config(), seed=2, count=8)
    assert ((st & abi.SP_ST_MASK) == 0).all()
    base = circ.elements[[e["name"] for e in circ.elements].index("M1")]["field"][0]
    for k in range(8):
        cardk = P[k, base:base + abi.SP_B3_CARD]
        r = ev(cardk, x[k, circ.node("g")], x[k, circ.node("d")], 0.0)
        # the follower's gate loads nothing at DC: only gds, gm and RD shape the gain
        gain = -r["gm"] / (r["gds"] + 1.0 / P[k, [i for i, l in enumerate(circ.param_labels) if l == "RD.r"][0]])
        assert abs(h[k, 0, 0].real - gain) < 1e-6 * abs(gain) and abs(h[k, 0, 0].imag) < 1e-3 * abs(gain)
        assert abs(h[k, -1, 0]) < 0.5 * abs(gain)


# --------------------------------------------------------------------------- GPU
def random_cards(rng, n, pmos):
    base = oracle.bsim3_default_card(pmos)
    c = np.tile(base, (n, 1))
    sgn = -1.0 if pmos else 1.0
    c[:, K["vth0"]] = sgn * rng.uniform(0.25, 0.6, n)
    c[:, K["u0"]] *= rng.uniform(0.7, 1.3, n)
    c[:, K["tox"]] *= rng.uniform(0.8, 1.2, n)
    c[:, K["l"]] = rng.uniform(50e-9, 1e-6, n)
    c[:, K["w"]] = rng.uniform(100e-9, 10e-6, n)
    c[:, K["nf"]] = rng.integers(1, 4, n)
    c[:, K["k1"]] = rng.uniform(0.3, 0.7, n)
    c[:, K["k2"]] = rng.uniform(-0.05, 0.05, n)
    c[:, K["k3"]] = rng.uniform(0.0, 10.0, n)
    c[:, K["k3b"]] = rng.uniform(-5e-9, 5e-9, n)  # K3B vbs / Weff is in volts: K3B ~ Weff x 10 mV
    c[:, K["dvt0w"]] = rng.uniform(0.0, 1.0, n)
    c[:, K["dvt1w"]] = rng.uniform(0.0, 300.0, n)
    c[:, K["eta0"]] = rng.uniform(0.0, 0.2, n)
    c[:, K["pdiblcb"]] = rng.uniform(-0.5, 0.5, n)
    c[:, K["nch"]] = rng.uniform(5e16, 5e17, n)
    return c


@pytest.mark.gpu
@pytest.mark.parametrize("pmos", [False, True])
def test_device_evaluation_matches_oracle(ctx, pmos):
    """sp_bsim3_eval_device against the oracle: bit-identical above threshold
    (IEEE operations in the reference's order, correctly rounded constants),
    within 4 ulp-scale relative error in weak inversion (the device exp)."""
    import torch
    rng = np.random.default_rng(11 + pmos)
    n = 20000
    c = random_cards(rng, n, pmos)
    sgn = -1.0 if pmos else 1.0
    bias = np.stack([sgn * rng.uniform(-0.2, 1.8, n), sgn * rng.uniform(-1.0, 1.8, n),
                     sgn * rng.uniform(-1.0, 0.3, n)], axis=1)
    bias[:64, 1] = 0.0  # vds = 0 exactly
    with oracle.math_mode("cr"):
        ro, rego = oracle.bsim3_evaluate(c, bias, pmos)
    dc, db = torch.from_numpy(c).cuda(), torch.from_numpy(bias).cuda()
    out = torch.empty(n, 6, dtype=torch.float64, device="cuda")
    reg = torch.empty(n, dtype=torch.uint8, device="cuda")
    ctx.bsim3_eval_device(pmos, dc, db, out, reg)
    torch.cuda.synchronize()
    g, gr = out.cpu().numpy(), reg.cpu().numpy()
    assert np.array_equal(gr, rego)
    assert set(np.unique(rego)) == {0, 1, 2}
    strong = rego > 0
    assert np.array_equal(g[strong].view(np.uint64), ro[strong].view(np.uint64))
    np.testing.assert_allclose(g[~strong], ro[~strong], rtol=1e-14, atol=0.0)


@pytest.mark.gpu
def test_newton_bsim3_against_oracle(ctx):
    circ = configs.bsim3_cmos_chain()
    n = 4096
    with oracle.math_mode("cr"):
        xo, io, so, _ = oracle.newton_dc(circ, abi.newton_config(), seed=4, count=n)
    assert ((so & abi.SP_ST_MASK) == 0).all()
    for prec, rtol in ((abi.SP_PREC_FP64_EXACT, 1e-11), (abi.SP_PREC_FP64, 1e-9)):
        r = ctx.newton_dc(circ, abi.newton_config(precision=prec), seed=4, count=n)
        assert np.array_equal(r.status, so)
        ok = (so & abi.SP_ST_MASK) == 0
        assert np.mean(r.iters[ok] == io[ok]) > 0.99
        np.testing.assert_allclose(r.x[ok], xo[ok], rtol=rtol, atol=1e-15)
    r = ctx.newton_dc(circ, abi.newton_config(precision=abi.SP_PREC_MIXED), seed=4, count=n)
    ok = ((so & abi.SP_ST_MASK) == 0) & ((r.status & abi.SP_ST_MASK) == 0)
    assert ok.mean() > 0.99
    nn = circ.num_nodes
    tol = np.concatenate([1e-3 * np.abs(xo[:, :nn]) + 1e-6, 1e-3 * np.abs(xo[:, nn:]) + 1e-12], axis=1)
    assert (np.abs(r.x[ok] - xo[ok]) <= tol[ok]).all()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [abi.SP_PREC_FP64, abi.SP_PREC_MIXED])
def test_ac_sweep_against_oracle(ctx, prec):
    """BSIM3 small-signal sweeps (gds, gm, gmbs and the Meyer / junction
    capacitances at each sample's operating point) within 1e-9 of the oracle."""
    from spicier_gb300.api import Context
    circ = cs_amp_with_caps()
    probes = [circ.node("out"), circ.node("d")]
    cfg = abi.ac_config(1e3, 1e11, 5, abi.SP_AC_DEC, probes, precision=prec)
    dc = abi.newton_config(precision=abi.SP_PREC_FP64)
    n = 512
    h, st = ctx.ac_sweep(circ, dc, cfg, 2, n)
    with oracle.math_mode("cr"):
        ho, so = oracle.ac_sweep(circ, dc, 2, n, Context.ac_frequencies(cfg), probes)
    ok = (so & abi.SP_ST_MASK) == 0
    assert np.array_equal(st, so) and ok.mean() > 0.99
    scale = np.abs(ho[ok]).max(axis=1, keepdims=True)
    assert (np.abs(h[ok] - ho[ok]) <= 1e-9 * scale + 1e-18).all()


@pytest.mark.gpu
def test_netlist_bsim3_sweep_on_gpu(ctx):
    """A BSIM3 netlist with Monte Carlo variations by ELEMENT.field, solved on the
    GPU and by the oracle from the same text."""
    nl = parse_netlist("""BSIM3 NMOS Amplifier
.MODEL NMOD NMOS LEVEL=49 VTH0=0.4 K1=0.5 U0=670 TOX=9e-9 VSAT=1.5e5
VDD 1 0 DC 3.3
VGS 2 0 DC 1.0
RD 1 3 5k
M1 3 2 0 0 NMOD W=1u L=100n
.end""", {"M1.vth0": Gauss(0.4, 0.02, 0), "M1.l": Gauss(100e-9, 5e-9, 1), "RD.r": Gauss(5e3, 200.0, 2)})
    circ = nl.circuit
    n = 8192
    r = ctx.newton_dc(circ, abi.newton_config(precision=abi.SP_PREC_FP64), seed=9, count=n)
    with oracle.math_mode("cr"):
        xo, io, so, _ = oracle.newton_dc(circ, abi.newton_config(), seed=9, count=n)
    assert np.array_equal(r.status, so) and ((so & abi.SP_ST_MASK) == 0).all()
    np.testing.assert_allclose(r.x, xo, rtol=1e-9, atol=1e-15)


@pytest.mark.gpu
def test_nonconverging_golden_inverter_matches_oracle(ctx):
    """The golden inverter netlist (PMOS with source and drain exchanged) fails
    in the reference's model; the GPU takes the same path through Newton, gmin
    and source stepping: same status flags and iteration totals as the oracle."""
    g = json.load(open(GOLDEN))
    text = [c for c in g["circuits"] if c["name"] == "bsim3_cmos_inverter"][0]["netlist"]
    circ = parse_netlist(text).circuit
    r = ctx.newton_dc(circ, abi.newton_config(precision=abi.SP_PREC_FP64_EXACT), seed=1, count=4)
    with oracle.math_mode("cr"):
        xo, io, so, _ = oracle.newton_dc(circ, abi.newton_config(), seed=1, count=4)
    assert (so & abi.SP_ST_MASK == abi.SP_ST_FAILED).all()
    assert np.array_equal(r.status, so) and np.array_equal(r.iters, io)
