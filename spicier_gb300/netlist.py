"""SPICE netlist text -> Circuit, for the element subset the batched sweep runs.

Follows the reference parser's rules for that subset
(crates/spicier-parser/src/lexer.rs, parser/elements.rs:109-632,
parser/commands.rs:600-735, crates/spicier-core/src/units.rs:15-50):

* the first line is the title, even when it starts with '*'; later lines
  starting with '*' are comments, ';' starts an inline comment, a line
  starting with '+' continues the previous one; names are case-insensitive;
* values are numbers with an optional suffix T G MEG K M MIL U N P F
  (units.rs:15-50: the suffix must match exactly, "1kohm" is an error);
* R, C, L: name n+ n- value; V: name n+ n- [DC v] [AC mag [phase]]
  [PULSE(v1 v2 [td tr tf pw per])] (a PULSE source's DC value is v1,
  Waveform::dc_value); I: name n+ n- [DC] value; D: name a k [model];
  M: name d g s b [model] [W= L= NF=] (the bulk becomes a node, as
  expect_node makes it; only a BSIM3 model connects it);
  Q: name c b e [model];
* .MODEL name D (IS N), NMOS / PMOS level 1 (VTO KP LAMBDA W L), NMOS / PMOS
  LEVEL=49 or 8 (BSIM3: the card entries of Circuit.B3 by their SPICE names,
  with the aliases DL, DW, VTHO, UO and TNOM in Celsius, parse_bsim3_params,
  parser/commands.rs:1463-1575; entries the DC model does not read are
  accepted and ignored), NPN / PNP (IS BF BR NF NR VAF); .PARAM name=value;
  .NODESET V(node)=value; .END.
  Other dot commands (.OP .DC .TRAN .AC .PRINT .OPTIONS ...) are recorded in
  Netlist.commands and otherwise ignored.

Monte Carlo variation is not part of SPICE syntax: parse_netlist takes a
mapping from "ELEMENT.field" (for example "M1.vto", "R3.r", "V1.v") to a
parameter spec (Gauss, Uniform, LogUniform, Table) that replaces the
element's nominal value.  Element types outside the subset raise
NetlistError, as do malformed lines.
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

from .circuit import BSIM3_DEFAULTS, Circuit, ParamSpec, Pulse

_BSIM3_ALIAS = {"DL": "lint", "DW": "wint", "VTHO": "vth0", "UO": "u0", "AS": "as_"}


def _bsim3_card(mp: Dict[str, float]) -> Dict[str, float]:
    """Card entries a BSIM3 .MODEL sets (parse_bsim3_params, parser/commands.rs:1463-1575):
    the defaults stay for the rest; TNOM is given in Celsius."""
    from . import _abi as abi
    card: Dict[str, float] = {}
    for key, v in mp.items():
        name = _BSIM3_ALIAS.get(key, key.lower())
        if name == "tnom":
            v = v + 273.15
        if name in abi.BSIM3_CARD:
            card[name] = v
    return card

_SUFFIX = {"T": 1e12, "G": 1e9, "MEG": 1e6, "K": 1e3, "": 1.0, "M": 1e-3, "MIL": 25.4e-6, "U": 1e-6, "N": 1e-9,
           "P": 1e-12, "F": 1e-15}
_NUM = re.compile(r"^[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?")


class NetlistError(ValueError):
    def __init__(self, line: int, message: str):
        super().__init__(f"line {line}: {message}")
        self.line = line


def parse_value(text: str) -> Optional[float]:
    """units.rs:15-50: plain float, else number + exact SI suffix (case-insensitive)."""
    s = text.strip().upper()
    try:
        return float(s)
    except ValueError:
        pass
    m = _NUM.match(s)
    if not m:
        return None
    mult = _SUFFIX.get(s[m.end():])
    if mult is None:
        return None
    return float(m.group(0)) * mult


@dataclass
class _Model:
    kind: str
    params: Dict[str, float] = field(default_factory=dict)


@dataclass
class Netlist:
    title: str
    circuit: Circuit
    commands: List[Tuple[str, List[str]]]
    nodeset: Dict[str, float]


def _logical_lines(text: str) -> List[Tuple[int, str]]:
    raw = text.splitlines()
    out: List[Tuple[int, str]] = []
    for i, line in enumerate(raw):
        no = i + 1
        if i == 0:
            out.append((no, ""))  # the title (kept apart)
            continue
        s = line.split(";", 1)[0].rstrip()
        st = s.lstrip()
        if not st or st.startswith("*"):
            continue
        if st.startswith("+"):
            if not out or len(out) == 1:
                raise NetlistError(no, "continuation line without a previous line")
            pno, prev = out[-1]
            out[-1] = (pno, prev + " " + st[1:])
            continue
        out.append((no, st))
    return out[1:]


def _tokens(s: str) -> List[str]:
    # parentheses, commas and '=' are separators that stay tokens where they matter
    s = s.replace("(", " ( ").replace(")", " ) ").replace(",", " ").replace("=", " = ")
    return s.split()


def _kv(tokens: List[str], start: int, line: int, params: Dict[str, float]) -> Dict[str, float]:
    out: Dict[str, float] = {}
    i = start
    while i < len(tokens):
        if i + 1 < len(tokens) and tokens[i + 1] == "=":
            if i + 2 >= len(tokens):
                raise NetlistError(line, f"missing value after {tokens[i]}=")
            out[tokens[i].upper()] = _val(tokens[i + 2], line, params)
            i += 3
        else:
            i += 1
    return out


def _val(tok: str, line: int, params: Dict[str, float]) -> float:
    t = tok.strip("{}")
    v = parse_value(t)
    if v is None:
        v = params.get(t.upper())
    if v is None:
        raise NetlistError(line, f"bad value {tok!r}")
    return v


def parse_netlist(text: str, variations: Optional[Dict[str, ParamSpec]] = None) -> Netlist:
    """Parse `text`; `variations` maps "ELEMENT.field" to a parameter spec."""
    lines = text.splitlines()
    title = " ".join(_tokens(lines[0])) if lines else ""
    var = {k.upper(): v for k, v in (variations or {}).items()}
    used = set()
    params: Dict[str, float] = {}
    models: Dict[str, _Model] = {}
    commands: List[Tuple[str, List[str]]] = []
    nodeset: Dict[str, float] = {}
    body = _logical_lines(text)
    elements: List[Tuple[int, List[str]]] = []
    # dot commands first (.MODEL and .PARAM may follow their use, as in SPICE decks)
    for no, s in body:
        tk = _tokens(s)
        if not tk[0].startswith("."):
            elements.append((no, tk))
            continue
        cmd = tk[0][1:].upper()
        if cmd == "END":
            break
        if cmd == "PARAM":
            for k, v in _kv(tk, 1, no, params).items():
                params[k] = v
        elif cmd == "MODEL":
            if len(tk) < 3:
                raise NetlistError(no, ".MODEL needs a name and a type")
            kind = tk[2].upper()
            if kind not in ("D", "NMOS", "PMOS", "NPN", "PNP"):
                raise NetlistError(no, f"model type {kind} is outside the supported subset")
            mp = _kv(tk, 3, no, params)
            if kind in ("NMOS", "PMOS") and int(mp.get("LEVEL", 1)) not in (1, 8, 49):
                raise NetlistError(no, "only level-1 and BSIM3 (LEVEL=49 / 8) MOSFET models are supported")
            models[tk[1].upper()] = _Model(kind, mp)
        elif cmd == "NODESET":
            i = 1
            while i < len(tk):
                if tk[i].upper() == "V" and i + 3 < len(tk) and tk[i + 1] == "(" and tk[i + 3] == ")":
                    if i + 5 >= len(tk) or tk[i + 4] != "=":
                        raise NetlistError(no, "expected V(node)=value")
                    nodeset[tk[i + 2]] = _val(tk[i + 5], no, params)
                    i += 6
                else:
                    raise NetlistError(no, "expected V(node)=value")
        else:
            commands.append((cmd, tk[1:]))

    c = Circuit(title)

    def spec(name: str, fld: str, nominal: float) -> ParamSpec:
        key = f"{name.upper()}.{fld.upper()}"
        if key in var:
            used.add(key)
            return var[key]
        return nominal

    def need(tk: List[str], k: int, no: int, what: str) -> str:
        if len(tk) <= k:
            raise NetlistError(no, f"{tk[0]}: missing {what}")
        return tk[k]

    for no, tk in elements:
        name = tk[0]
        kind = name[0].upper()
        if kind in "RCL":
            a, b = need(tk, 1, no, "node"), need(tk, 2, no, "node")
            v = _val(need(tk, 3, no, "value"), no, params)
            if kind == "R":
                c.R(name, a, b, spec(name, "r", v))
            elif kind == "C":
                c.Cap(name, a, b, spec(name, "c", v))
            else:
                c.L(name, a, b, spec(name, "l", v))
        elif kind == "V":
            a, b = need(tk, 1, no, "node"), need(tk, 2, no, "node")
            dc, pulse, i = 0.0, None, 3
            while i < len(tk):
                u = tk[i].upper()
                if u == "DC":
                    dc = _val(need(tk, i + 1, no, "DC value"), no, params)
                    i += 2
                elif u == "AC":
                    i += 2
                    if i < len(tk) and parse_value(tk[i]) is not None:
                        i += 1
                elif u == "PULSE":
                    if need(tk, i + 1, no, "(") != "(":
                        raise NetlistError(no, "expected '(' after PULSE")
                    j = i + 2
                    vals = []
                    while j < len(tk) and tk[j] != ")":
                        vals.append(_val(tk[j], no, params))
                        j += 1
                    if j >= len(tk) or len(vals) < 2 or len(vals) > 7:
                        raise NetlistError(no, "PULSE(v1 v2 [td tr tf pw per])")
                    vals += [0.0] * (7 - len(vals))
                    pulse = Pulse(*vals)
                    i = j + 1
                elif u in ("SIN", "PWL"):
                    raise NetlistError(no, f"{u} sources are outside the supported subset")
                elif parse_value(tk[i]) is not None or tk[i].upper() in params:
                    dc = _val(tk[i], no, params)
                    i += 1
                else:
                    break
            nominal = pulse.v1 if pulse is not None else dc
            c.V(name, a, b, spec(name, "v", nominal), pulse=pulse)
        elif kind == "I":
            a, b = need(tk, 1, no, "node"), need(tk, 2, no, "node")
            k = 3
            if len(tk) > k and tk[k].upper() == "DC":
                k += 1
            c.I(name, a, b, spec(name, "i", _val(need(tk, k, no, "value"), no, params)))
        elif kind == "D":
            a, b = need(tk, 1, no, "node"), need(tk, 2, no, "node")
            mp = models.get(tk[3].upper()) if len(tk) > 3 else None
            p = mp.params if mp is not None and mp.kind == "D" else {}
            c.D(name, a, b, is_=spec(name, "is", p.get("IS", 1e-14)), n=spec(name, "n", p.get("N", 1.0)))
        elif kind == "M":
            d, g, s_ = need(tk, 1, no, "drain"), need(tk, 2, no, "gate"), need(tk, 3, no, "source")
            bulk = need(tk, 4, no, "bulk")
            pmos = False
            mp: Dict[str, float] = {}
            k = 5
            if len(tk) > k and (k + 1 >= len(tk) or tk[k + 1] != "="):
                m = models.get(tk[k].upper())
                if m is not None and m.kind in ("NMOS", "PMOS"):
                    pmos = m.kind == "PMOS"
                    mp = dict(m.params)
                k += 1
            inst = _kv(tk, k, no, params)
            if int(mp.get("LEVEL", 1)) in (8, 49):
                card = dict(BSIM3_DEFAULTS[pmos])
                card.update(_bsim3_card(mp))
                for key in ("W", "L", "NF", "AS", "AD", "PS", "PD"):  # instance overrides (parser/elements.rs:455-476)
                    if key in inst:
                        card[_BSIM3_ALIAS.get(key, key.lower())] = inst[key]
                c.B3(name, d, g, s_, bulk, pmos=pmos, **{k: spec(name, k, v) for k, v in card.items()})
                continue
            vto = mp.get("VTO", -0.7 if pmos else 0.7)
            kp = mp.get("KP", 1e-5 if pmos else 2e-5)
            lam = mp.get("LAMBDA", 0.0)
            w = inst.get("W", mp.get("W", 10e-6))
            ln = inst.get("L", mp.get("L", 1e-6))
            nf = inst.get("NF", 1.0)
            c.M(name, d, g, s_, pmos=pmos, vto=spec(name, "vto", vto), kp=spec(name, "kp", kp),
                lam=spec(name, "lambda", lam), w=spec(name, "w", w), l=spec(name, "l", ln), nf=spec(name, "nf", nf))
            c.node(bulk)  # parsed as a node (expect_node) though no model uses it
        elif kind == "Q":
            cc, bb, ee = need(tk, 1, no, "collector"), need(tk, 2, no, "base"), need(tk, 3, no, "emitter")
            pnp = False
            bp: Dict[str, float] = {}
            if len(tk) > 4:
                m = models.get(tk[4].upper())
                if m is not None and m.kind in ("NPN", "PNP"):
                    pnp = m.kind == "PNP"
                    bp = m.params
            c.Q(name, cc, bb, ee, pnp=pnp, is_=spec(name, "is", bp.get("IS", 1e-16)),
                bf=spec(name, "bf", bp.get("BF", 100.0)), br=spec(name, "br", bp.get("BR", 1.0)),
                nf=spec(name, "nf", bp.get("NF", 1.0)), nr=spec(name, "nr", bp.get("NR", 1.0)),
                vaf=spec(name, "vaf", bp.get("VAF", 0.0)))
        else:
            raise NetlistError(no, f"element {name} is outside the supported subset (R C L V I D M Q)")
    missing = sorted(set(var) - used)
    if missing:
        raise NetlistError(0, f"variations name no element field: {', '.join(missing)}")
    for node, v in nodeset.items():
        if node in c.node_index:
            c.nodeset[node] = v
    return Netlist(title, c, commands, nodeset)
