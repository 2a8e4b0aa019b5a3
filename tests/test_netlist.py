"""SPICE netlist front end (spicier_gb300/netlist.py) against the reference
parser's rules and against the programmatic workload circuits."""
import numpy as np
import pytest

import oracle
from spicier_gb300 import abi, configs
from spicier_gb300.circuit import Gauss, Uniform
from spicier_gb300.netlist import NetlistError, parse_netlist, parse_value


def test_parse_value_matches_units_rs():
    # crates/spicier-core/src/units.rs tests
    assert parse_value("1.5") == 1.5 and parse_value("-2.5") == -2.5 and parse_value("1e-3") == 1e-3
    for text, v in [("1k", 1e3), ("4.7K", 4.7e3), ("10M", 10e-3), ("10MEG", 10e6), ("100n", 100e-9), ("1u", 1e-6),
                    ("10p", 10e-12)]:
        assert abs(parse_value(text) - v) < abs(v) * 1e-10 + 1e-20
    assert parse_value("abc") is None and parse_value("") is None and parse_value("1kohm") is None
    # number times multiplier, rounded once (as value * multiplier in units.rs)
    assert parse_value("20u") == 20.0 * 1e-6 and parse_value("2mil") == 2.0 * 25.4e-6


CS_AMP = """* common-source amplifier: the first line is the title even with a star
VDD vdd 0 DC 5
R1 vdd gate 100k ; gate divider
R2 gate 0 47k
RD vdd drain 10k
RS source 0 1k
M1 drain gate source 0 NCH W=10e-6
+ L=1e-6
.MODEL NCH NMOS (VTO=0.7 KP=110e-6 LAMBDA=0.02)
.OP
.END
"""


def cs_variations():
    return {"RD.r": Gauss(10e3, 0.05 * 10e3, 0), "RS.r": Gauss(1e3, 0.05 * 1e3, 1),
            "M1.vto": Gauss(0.7, 0.03, 2), "M1.kp": Gauss(110e-6, 0.10 * 110e-6, 3)}


def test_cs_amp_netlist_equals_programmatic_circuit():
    nl = parse_netlist(CS_AMP, cs_variations())
    assert nl.title.startswith("*") and ("OP", []) in nl.commands
    a = nl.circuit
    b = configs.cs_nmos_amp()
    assert a.n == b.n == 5
    cfg = abi.newton_config()
    xa, ia, sa, _ = oracle.newton_dc(a, cfg, 1, 512, threads=2)
    xb, ib, sb, _ = oracle.newton_dc(b, cfg, 1, 512, threads=2)
    # same unknown order (nodes by first appearance, then the source branch)
    assert np.array_equal(xa.view(np.uint64), xb.view(np.uint64))
    assert np.array_equal(ia, ib) and np.array_equal(sa, sb)


def opamp_netlist():
    lines = ["two-stage Miller op-amp", "VDD vdd 0 3.3", "VSS vss 0 0", "VIN vin 0 DC 1.65", "IBIAS vdd bias 20e-6"]
    for name, d, g, s, pmos, w in configs.OPAMP_DEVICES:
        lines.append(f"{name} {d} {g} {s} {'vdd' if pmos else 'vss'} {'PCH' if pmos else 'NCH'} W={w!r} L=1e-6")
    lines += ["RZ n2 nz 2k", "CC nz out 2e-12",
              ".MODEL NCH NMOS (LEVEL=1 VTO=0.7 KP=110e-6 LAMBDA=0.04)",
              ".MODEL PCH PMOS (VTO=-0.8 KP=50e-6 LAMBDA=0.04)",
              ".NODESET V(vdd)=3.3 V(vss)=0 V(vin)=1.65 V(out)=1.65 V(n1)=2.3 V(n2)=2.3 V(nz)=2.3",
              "+ V(tail)=0.8 V(bias)=0.9", ".END"]
    var = {"VIN.v": Uniform(1.0, 2.3, 0)}
    for k, (name, _d, _g, _s, pmos, _w) in enumerate(configs.OPAMP_DEVICES):
        vto0 = configs.PMOS_VTO if pmos else configs.NMOS_VTO
        kp0 = configs.PMOS_KP if pmos else configs.NMOS_KP
        var[f"{name}.vto"] = Gauss(vto0, 0.020, 1 + 2 * k)
        var[f"{name}.kp"] = Gauss(kp0, 0.05 * kp0, 2 + 2 * k)
    return "\n".join(lines), var


def test_opamp_netlist_runs_the_workload():
    text, var = opamp_netlist()
    a = parse_netlist(text, var).circuit
    b = configs.miller_opamp()
    assert a.n == b.n == 12 and len(a.params) == len(b.params)
    assert {k: a.nodeset[k] for k in b.nodeset} == b.nodeset
    cfg = abi.newton_config()
    xa, ia, sa, _ = oracle.newton_dc(a, cfg, 1, 256, threads=2)
    xb, ib, sb, _ = oracle.newton_dc(b, cfg, 1, 256, threads=2)
    # the same equations with the same draws; the unknowns are ordered by first appearance
    order = [a.node_index[nm] for nm in b.node_index] + list(range(a.num_nodes, a.n))
    assert np.array_equal(xa[:, order].view(np.uint64), xb.view(np.uint64))
    assert np.array_equal(ia, ib) and np.array_equal(sa, sb)


def test_pulse_source_and_transient():
    text = "rc step\nV1 in 0 PULSE(0 5 0 1e-12 1e-12 1 2)\nR1 in out 1k\nC1 out 0 1u\n.TRAN 10u 5m\n.END\n"
    nl = parse_netlist(text)
    c = nl.circuit
    assert nl.commands == [("TRAN", ["10u", "5m"])]
    assert c.params[0][2] == 0.0  # DC value of a PULSE source is v1 (Waveform::dc_value)
    x, pr, st = oracle.transient(c, abi.newton_config(), 1, 1, abi.SP_TRAN_BE, 10e-6, 5e-3,
                                 probe_idx=c.node("out"))
    assert st[0] == 0 and abs(x[0, c.node("out")] - 5.0) < 0.05


def test_errors():
    with pytest.raises(NetlistError):
        parse_netlist("t\nR1 a 0 1kohm\n")
    with pytest.raises(NetlistError):
        parse_netlist("t\nE1 a 0 b 0 2\n")  # controlled sources are outside the subset
    with pytest.raises(NetlistError):
        parse_netlist("t\nR1 a 0 1k\n", {"R2.r": Gauss(1e3, 10.0, 0)})
    with pytest.raises(NetlistError):
        parse_netlist("t\n.MODEL X NMOS LEVEL=54\n")
    with pytest.raises(NetlistError):
        parse_netlist("t\nV1 a 0 SIN(0 1 1k)\n")
