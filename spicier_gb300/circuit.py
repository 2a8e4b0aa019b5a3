"""Programmatic circuit description for the batched Newton path.

A ``Circuit`` is the flat element list the GPU kernels interpret: each
element names its MNA nodes and, for every model field, a slot in the
per-sample parameter vector.  A slot holds either a fixed value or a draw
from the stateless hash RNG keyed by (seed, sweep index, rng index), exactly
as ``spicier_batched_sweep::rng`` keys them
(crates/spicier-batched-sweep/src/rng.rs:51-56, 148-150), or a column of a
caller-supplied table (the output of a host ``SweepPointGenerator``).

Element semantics follow the reference devices:
  R  passive.rs:53-59      C  passive.rs:232-240     L  passive.rs:318-325
  V  sources.rs:96-101     I  sources.rs:230-236     D  diode.rs:91-131
  M  mosfet/level1.rs:154-248                        Q  bjt.rs:176-330
MNA node indices follow the reference's node_to_index (node n -> n-1,
ground -> None): nodes are numbered in order of first use, ground is -1.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Dict, List, Optional, Sequence, Union

from . import _abi as abi

GROUND_NAMES = ("0", "gnd", "GND")


@dataclass(frozen=True)
class Gauss:
    """mean + gaussian(seed, s, index) * sigma (sigma absolute; rng.rs:148-150)."""
    mean: float
    sigma: float
    index: int


@dataclass(frozen=True)
class Uniform:
    """lo + uniform(seed, s, index) * (hi - lo)."""
    lo: float
    hi: float
    index: int


@dataclass(frozen=True)
class LogUniform:
    """lo * exp(uniform(seed, s, index) * ln(hi / lo))."""
    lo: float
    hi: float
    index: int


@dataclass(frozen=True)
class Table:
    """Column ``col`` of a per-sample parameter table."""
    col: int


ParamSpec = Union[float, int, Gauss, Uniform, LogUniform, Table]


@dataclass(frozen=True)
class Pulse:
    """PULSE(v1 v2 td tr tf pw per), waveforms.rs:159-182."""
    v1: float
    v2: float
    td: float
    tr: float
    tf: float
    pw: float
    per: float


def _bsim3_defaults(pmos: bool) -> Dict[str, float]:
    """Bsim3Params::nmos_default / pmos_default (mosfet/bsim3/params.rs:160-310),
    the entries the DC model reads."""
    d = dict(tox=9e-9, lint=0.0, wint=0.0, vth0=-0.4 if pmos else 0.4, k1=0.5, k2=0.0, dvt0=2.2,
             dvt1=0.53, dvt2=-0.032, nfactor=1.0, k3=0.0, k3b=0.0, w0=0.0, dvt0w=0.0, dvt1w=0.0,
             dvt2w=0.0, u0=250.0 if pmos else 670.0, ua=2.25e-9, ub=5.87e-19, uc=-4.65e-11,
             vsat=1.0e5 if pmos else 1.5e5, pclm=1.3, pdiblc1=0.39, pdiblc2=0.0086, drout=0.56,
             eta0=0.08, etab=-0.07, dsub=0.56, pdiblcb=0.0, pvag=1.0, nch=1.7e17, tnom=300.15,
             kt2=0.022, w=1e-6, l=100e-9, nf=1.0,
             cgso=0.0, cgdo=0.0, cgbo=0.0, cj=5e-4, cjsw=5e-10, cjswg=0.0, mj=0.5, mjsw=0.33, mjswg=0.33,
             pb=1.0, pbsw=1.0, pbswg=1.0, as_=0.0, ad=0.0, ps=0.0, pd=0.0)
    assert tuple(d) == abi.BSIM3_CARD
    return d


BSIM3_DEFAULTS = {False: _bsim3_defaults(False), True: _bsim3_defaults(True)}


class Circuit:
    def __init__(self, title: str = ""):
        self.title = title
        self.node_index: Dict[str, int] = {}
        self.elements: List[dict] = []
        self.params: List[tuple] = []  # (kind, rng_index, a, b, label)
        self.param_labels: List[str] = []
        self.pulses: List[Pulse] = []
        self.num_branches = 0
        self.nodeset: Dict[str, float] = {}
        self._c_keepalive = None

    # -- nodes and parameters ------------------------------------------------
    def node(self, name: str) -> int:
        if name in GROUND_NAMES:
            return -1
        if name not in self.node_index:
            self.node_index[name] = len(self.node_index)
        return self.node_index[name]

    @property
    def num_nodes(self) -> int:
        return len(self.node_index)

    @property
    def n(self) -> int:
        """MNA size: nodes + current variables."""
        return self.num_nodes + self.num_branches

    def param(self, spec: ParamSpec, label: str = "") -> int:
        if isinstance(spec, Gauss):
            row = (abi.SP_DRAW_GAUSS, spec.index, float(spec.mean), float(spec.sigma))
        elif isinstance(spec, Uniform):
            row = (abi.SP_DRAW_UNIFORM, spec.index, float(spec.lo), float(spec.hi))
        elif isinstance(spec, LogUniform):
            row = (abi.SP_DRAW_LOGUNIFORM, spec.index, float(spec.lo), float(spec.hi))
        elif isinstance(spec, Table):
            row = (abi.SP_DRAW_TABLE, spec.col, 0.0, 0.0)
        else:
            row = (abi.SP_DRAW_FIXED, 0, float(spec), 0.0)
        self.params.append(row)
        self.param_labels.append(label)
        return len(self.params) - 1

    def _add(self, kind: int, name: str, nodes: Sequence[str], fields: Sequence[ParamSpec],
             field_names: Sequence[str], branch: bool = False, pulse: Optional[Pulse] = None) -> int:
        idx = [self.node(nm) for nm in nodes] + [-1] * (4 - len(nodes))
        slots = [self.param(f, f"{name}.{fn}") for f, fn in zip(fields, field_names)]
        br = -1
        if branch:
            br = self.num_branches
            self.num_branches += 1
        wave = -1
        if pulse is not None:
            self.pulses.append(pulse)
            wave = len(self.pulses) - 1
        self.elements.append(dict(kind=kind, name=name, node=idx, branch=br, wave=wave, field=slots))
        self._c_keepalive = None
        return len(self.elements) - 1

    # -- elements --------------------------------------------------------------
    def R(self, name, a, b, r: ParamSpec):
        return self._add(abi.SP_EL_R, name, (a, b), (r,), ("r",))

    def Cap(self, name, a, b, c: ParamSpec):
        return self._add(abi.SP_EL_C, name, (a, b), (c,), ("c",))

    def L(self, name, a, b, l: ParamSpec):
        return self._add(abi.SP_EL_L, name, (a, b), (l,), ("l",), branch=True)

    def V(self, name, p, n, v: ParamSpec, pulse: Optional[Pulse] = None):
        return self._add(abi.SP_EL_V, name, (p, n), (v,), ("v",), branch=True, pulse=pulse)

    def I(self, name, p, n, i: ParamSpec, pulse: Optional[Pulse] = None):
        return self._add(abi.SP_EL_I, name, (p, n), (i,), ("i",), pulse=pulse)

    def D(self, name, anode, cathode, is_: ParamSpec = 1e-14, n: ParamSpec = 1.0):
        return self._add(abi.SP_EL_D, name, (anode, cathode), (is_, n), ("is", "n"))

    def M(self, name, d, g, s, pmos: bool = False, vto: ParamSpec = None, kp: ParamSpec = None,
          lam: ParamSpec = 0.0, w: ParamSpec = 10e-6, l: ParamSpec = 1e-6, nf: ParamSpec = 1.0):
        """Level-1 MOSFET; defaults are MosfetParams::{nmos,pmos}_default (level1.rs:40-66)."""
        if vto is None:
            vto = -0.7 if pmos else 0.7
        if kp is None:
            kp = 1e-5 if pmos else 2e-5
        kind = abi.SP_EL_PMOS if pmos else abi.SP_EL_NMOS
        return self._add(kind, name, (d, g, s), (vto, kp, lam, w, l, nf),
                         ("vto", "kp", "lambda", "w", "l", "nf"))

    def Q(self, name, c, b, e, pnp: bool = False, is_: ParamSpec = 1e-16, bf: ParamSpec = 100.0,
          br: ParamSpec = 1.0, nf: ParamSpec = 1.0, nr: ParamSpec = 1.0, vaf: ParamSpec = 0.0):
        """Ebers-Moll BJT; vaf <= 0 means infinite (BjtParams::npn_default, bjt.rs:55-72)."""
        kind = abi.SP_EL_PNP if pnp else abi.SP_EL_NPN
        return self._add(kind, name, (c, b, e), (is_, bf, br, nf, nr, vaf),
                         ("is", "bf", "br", "nf", "nr", "vaf"))

    def B3(self, name, d, g, s, b, pmos: bool = False, **card: ParamSpec):
        """BSIM3v3.3 MOSFET (LEVEL=49 / 8): drain, gate, source, bulk.  `card`
        sets any sp_bsim3_card entry by its lower-case name (tox, vth0, u0, ...,
        w, l, nf, cgso, ..., as_, ad, ps, pd; tnom in kelvin), each a value or a
        distribution; the rest are
        Bsim3Params::{nmos,pmos}_default (mosfet/bsim3/params.rs:160-310).  The
        entries take consecutive parameter slots, the first in field[0]."""
        vals = dict(BSIM3_DEFAULTS[bool(pmos)])
        for k, v in card.items():
            if k.lower() not in vals:
                raise ValueError(f"{name}: {k} is not a BSIM3 card entry")
            vals[k.lower()] = v
        kind = abi.SP_EL_BSIM3P if pmos else abi.SP_EL_BSIM3N
        i = self._add(kind, name, (d, g, s, b), [vals[k] for k in abi.BSIM3_CARD], abi.BSIM3_CARD)
        self.elements[i]["field"] = self.elements[i]["field"][:1]
        return i

    # -- export ------------------------------------------------------------------
    def to_c(self) -> abi.SpCircuit:
        """The sp_circuit view (arrays kept alive on this object)."""
        if self._c_keepalive is not None:
            return self._c_keepalive[0]
        ne, npar, npul = len(self.elements), len(self.params), len(self.pulses)
        els = (abi.SpElement * max(ne, 1))()
        for i, e in enumerate(self.elements):
            els[i].kind = e["kind"]
            for k in range(4):
                els[i].node[k] = e["node"][k]
            els[i].branch = e["branch"]
            els[i].wave = e["wave"]
            f = list(e["field"]) + [0] * (abi.SP_MAX_FIELDS - len(e["field"]))
            for k in range(abi.SP_MAX_FIELDS):
                els[i].field[k] = f[k]
        prm = (abi.SpParam * max(npar, 1))()
        for i, (kind, idx, a, b) in enumerate(self.params):
            prm[i].kind, prm[i].rng_index, prm[i].a, prm[i].b = kind, idx, a, b
        pul = (abi.SpPulse * max(npul, 1))()
        for i, p in enumerate(self.pulses):
            for k in ("v1", "v2", "td", "tr", "tf", "pw", "per"):
                setattr(pul[i], k, getattr(p, k))
        c = abi.SpCircuit()
        c.num_nodes, c.num_branches = self.num_nodes, self.num_branches
        c.num_elements, c.num_params, c.num_pulses = ne, npar, npul
        c.elements = C.cast(els, C.POINTER(abi.SpElement))
        c.params = C.cast(prm, C.POINTER(abi.SpParam))
        c.pulses = C.cast(pul, C.POINTER(abi.SpPulse))
        ns = None
        if self.nodeset:
            ns = (C.c_double * max(self.n, 1))()
            for nm, v in self.nodeset.items():
                ns[self.node_index[nm]] = float(v)
            c.nodeset = C.cast(ns, C.POINTER(C.c_double))
        self._c_keepalive = (c, els, prm, pul, ns)
        return c

    def nodeset_vector(self):
        """The nodeset as a list over all MNA unknowns (zeros elsewhere)."""
        v = [0.0] * self.n
        for nm, val in self.nodeset.items():
            v[self.node_index[nm]] = float(val)
        return v

    def table_cols(self) -> int:
        cols = [idx for (kind, idx, _a, _b) in self.params if kind == abi.SP_DRAW_TABLE]
        return (max(cols) + 1) if cols else 0

    def unknown_names(self) -> List[str]:
        names = [""] * self.n
        for nm, i in self.node_index.items():
            names[i] = f"V({nm})"
        for e in self.elements:
            if e["branch"] >= 0:
                names[self.num_nodes + e["branch"]] = f"I({e['name']})"
        return names
