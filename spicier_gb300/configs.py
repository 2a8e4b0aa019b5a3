"""The benchmark circuits of the batched Newton sweep, built programmatically.

Each builder returns a ``Circuit`` whose random parameters are drawn by the
stateless hash RNG (crates/spicier-batched-sweep/src/rng.rs) with the rng
index order stated in its docstring.  Topology choices that the workload
descriptions leave open are stated in each docstring.
"""
from __future__ import annotations

from .circuit import Circuit, Gauss, Uniform

# Level-1 process cards of the op-amp workload.
NMOS_VTO, NMOS_KP = 0.7, 110e-6
PMOS_VTO, PMOS_KP = -0.8, 50e-6
OPAMP_LAMBDA = 0.04


def cs_nmos_amp() -> Circuit:
    """Common-source NMOS amplifier, Monte Carlo over RD, RS, VTO, KP.

    VDD = 5 V; gate divider 100k (vdd-gate) / 47k (gate-0); RD = 10k
    (vdd-drain); RS = 1k (source-0); NMOS Level-1 W/L = 10u/1u, VTO 0.7 V,
    KP 110e-6 A/V^2, LAMBDA 0.02.  Draws (seed 1 in the workload):
    rng index 0 RD ~ N(10k, 5 %), 1 RS ~ N(1k, 5 %), 2 VTO ~ N(0.7, 30 mV),
    3 KP ~ N(110e-6, 10 %); sigma absolute (gaussian_scaled).
    MNA: nodes vdd, gate, drain, source + the VDD branch = 5 unknowns.
    """
    c = Circuit("cs_nmos_amp")
    c.V("VDD", "vdd", "0", 5.0)
    c.R("R1", "vdd", "gate", 100e3)
    c.R("R2", "gate", "0", 47e3)
    c.R("RD", "vdd", "drain", Gauss(10e3, 0.05 * 10e3, 0))
    c.R("RS", "source", "0", Gauss(1e3, 0.05 * 1e3, 1))
    c.M("M1", "drain", "gate", "source", vto=Gauss(0.7, 0.03, 2),
        kp=Gauss(110e-6, 0.10 * 110e-6, 3), lam=0.02, w=10e-6, l=1e-6)
    return c


def bjt_diode_bias() -> Circuit:
    """NPN common-emitter stage (RB 430k, RC ~ N(2k, 100 ohm) at rng index 0,
    RE 200, IS 1e-15, BF 120, VAF 80) plus a 1k-fed diode from a 5 V rail:
    the exponential device models of the Newton path (diode.rs, bjt.rs)."""
    c = Circuit("bjt_diode_bias")
    c.V("VCC", "vcc", "0", 5.0)
    c.R("RB", "vcc", "b", 430e3)
    c.R("RC", "vcc", "c", Gauss(2e3, 100.0, 0))
    c.Q("Q1", "c", "b", "e", is_=1e-15, bf=120.0, vaf=80.0)
    c.R("RE", "e", "0", 200.0)
    c.R("RD", "vcc", "d", 1e3)
    c.D("D1", "d", "0", is_=1e-14, n=1.0)
    return c


# (name, drain, gate, source, pmos, W) of the two-stage Miller op-amp, netlist order.
OPAMP_DEVICES = (
    ("M1", "n1", "out", "tail", False, 20e-6),   # diff pair, inverting input (feedback)
    ("M2", "n2", "vin", "tail", False, 20e-6),   # diff pair, non-inverting input
    ("M3", "n1", "n1", "vdd", True, 20e-6),      # PMOS mirror, diode side
    ("M4", "n2", "n1", "vdd", True, 20e-6),      # PMOS mirror, output side
    ("M5", "tail", "bias", "vss", False, 20e-6),  # tail current source (40 uA)
    ("M6", "out", "n2", "vdd", True, 80e-6),     # second stage, common source
    ("M7", "out", "bias", "vss", False, 40e-6),  # second-stage sink (80 uA)
    ("M8", "bias", "bias", "vss", False, 10e-6),  # bias diode fed by IBIAS
)


def miller_opamp(vto_sigma: float = 0.020, kp_rel_sigma: float = 0.05, rbias: float = 0.0, rload: float = 0.0) -> Circuit:
    """Two-stage Miller CMOS op-amp as a unity-gain buffer.

    Supplies VDD = 3.3 V and VSS = 0 V (an explicit rail source), input
    VIN ~ U(1.0, 2.3) V, IBIAS = 20 uA from vdd into the bias diode M8.
    Eight Level-1 devices (all L = 1 um, LAMBDA 0.04; NMOS VTO 0.7, KP 110e-6;
    PMOS VTO -0.8, KP 50e-6) with W as in OPAMP_DEVICES; compensation
    Rz = 2k in series with Cc = 2 pF (n2-nz-out; Cc open at DC).
    Draws: rng index 0 VIN (uniform); then per device in netlist order
    VTO ~ N(nominal, 20 mV) at index 1 + 2k and KP ~ N(nominal, 5 %) at
    index 2 + 2k.
    MNA: 9 nodes (vdd, vss, vin, out, n1, n2, tail, bias, nz) + 3 source
    branches (VDD, VSS, VIN) = 12 unknowns.
    Newton starts from the circuit's nodeset (the nominal operating point:
    out = vin = 1.65 V, mirror nodes 2.3 V, tail 0.8 V, bias 0.9 V).  From the
    reference's zero start the unlimited Level-1 Newton of
    crates/spicier-solver/src/newton.rs diverges on this loop for most
    samples (and so do its default gmin/source-stepping schedules).
    """
    c = Circuit("miller_opamp")
    c.V("VDD", "vdd", "0", 3.3)
    c.V("VSS", "vss", "0", 0.0)
    c.V("VIN", "vin", "0", Uniform(1.0, 2.3, 0))
    if rbias > 0:
        c.R("RBIAS", "vdd", "bias", rbias)
    else:
        c.I("IBIAS", "vdd", "bias", 20e-6)
    for k, (name, d, g, s, pmos, w) in enumerate(OPAMP_DEVICES):
        vto0 = PMOS_VTO if pmos else NMOS_VTO
        kp0 = PMOS_KP if pmos else NMOS_KP
        c.M(name, d, g, s, pmos=pmos,
            vto=Gauss(vto0, vto_sigma, 1 + 2 * k),
            kp=Gauss(kp0, kp_rel_sigma * kp0, 2 + 2 * k),
            lam=OPAMP_LAMBDA, w=w, l=1e-6)
    c.R("RZ", "n2", "nz", 2e3)
    # .nodeset: the nominal operating point the Monte Carlo samples start from
    c.nodeset = dict(vdd=3.3, vss=0.0, vin=1.65, out=1.65, n1=2.3, n2=2.3, nz=2.3, tail=0.8, bias=0.9)
    if rload > 0:
        c.R("RL", "out", "vss", rload)
    c.Cap("CC", "nz", "out", 2e-12)
    return c


def bsim3_cmos_chain() -> Circuit:
    """BSIM3 (LEVEL=49, default 100 nm cards) CMOS inverter driving a common-source
    stage with a 10 kOhm load, VDD 1.8 V.  Gaussian draws (rng index): VIN 0.8 V
    sigma 50 mV (0), PMOS VTH0 -0.4 V sigma 20 mV (1), PMOS U0 250 sigma 10 (2),
    inverter NMOS VTH0 0.4 V sigma 20 mV (3) and L 100 nm sigma 5 nm (4), stage
    NMOS VTH0 0.4 V sigma 20 mV (5) and U0 670 sigma 20 (6).  Nodeset 0.9 V on the
    inverter output and the stage output."""
    c = Circuit("bsim3_cmos_chain")
    c.V("VDD", "vdd", "0", 1.8)
    c.V("VIN", "in", "0", Gauss(0.8, 0.05, 0))
    c.B3("MP", "mid", "in", "vdd", "vdd", pmos=True, vth0=Gauss(-0.4, 0.02, 1), u0=Gauss(250.0, 10.0, 2), w=2e-6)
    c.B3("MN", "mid", "in", "0", "0", vth0=Gauss(0.4, 0.02, 3), l=Gauss(100e-9, 5e-9, 4))
    c.R("RL", "vdd", "out", 10e3)
    c.B3("M2", "out", "mid", "0", "0", vth0=Gauss(0.4, 0.02, 5), u0=Gauss(670.0, 20.0, 6))
    c.nodeset = {"mid": 0.9, "out": 0.9}
    return c
