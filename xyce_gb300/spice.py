"""SPICE-subset netlist reader and ``.prn`` / ``.mt0`` writers for the GPU
transient path.

Lets a netlist written for the reference drive the device-resident
transient (``Circuit.transient``) and produce the reference's tabular
output.  The subset is what the path simulates:

* elements ``R``, ``C``, ``L`` (no IC), ``V`` and ``I`` (DC, ``SIN``, ``PULSE``, ``PWL``),
  ``D`` (diode level 1), ``M`` (MOSFET level 1; level 54/14 = BSIM4 4.8.2),
  ``X`` (subcircuit instances, flattened);
* ``.MODEL``, ``.SUBCKT``/``.ENDS``, ``.TRAN``, ``.OPTIONS TIMEINT``
  (RELTOL, ABSTOL, METHOD=TRAP|GEAR, MAXORD), ``.OPTIONS NONLIN-TRAN``
  (RELTOL, ABSTOL, DELTAXTOL, RHSTOL, SMALLUPDATETOL, MAXSTEP),
  ``.OPTIONS LINSOL TYPE=KLU|KSPARSE``, ``.INCLUDE``, ``{expression}`` values
  (arithmetic, parameters, SPICE numbers, SQRT EXP LOG ... functions) in
  elements, sources, models and ``.PARAM``, ``.TEMP`` and ``.OPTIONS DEVICE
  TEMP= TNOM=`` (diodes and level-1 MOSFETs; the instance TEMP / DTEMP and
  the model TNOM too), ``.PARAM`` with ``{NAME}``
  references, ``.STEP`` (LIN, DEC, OCT or LIST; every point of the sweep runs as one
  circuit of a single GPU batch), ``.SAMPLING`` with ``.OPTIONS SAMPLES``
  (Latin hypercube or Monte Carlo samples of NORMAL / UNIFORM parameters,
  all samples one batch, moments of every .MEASURE), ``.EMBEDDEDSAMPLING``
  with ``.OPTIONS EMBEDDEDSAMPLES`` (the samples as one block system with one
  step control; per-point moments of each output in ``<netlist>_ensemble.prn``),
  ``.PRINT TRAN`` (FORMAT=STD,
  NOINDEX or CSV), ``.MEASURE TRAN`` (MAX, MIN, PP, AVG,
  RMS, INTEG with FROM/TO; TRIG/TARG with VAL, TD and RISE/FALL/CROSS=n|LAST;
  WHEN; FIND and DERIV ... WHEN / AT; FREQ, DUTY, ON_TIME and OFF_TIME with
  ON/OFF), ``.END``; ``*`` and ``;`` comments, ``+``
  continuation lines, engineering suffixes (T G MEG K M MIL U N P F);
* print variables ``V(n)``, ``V(a,b)``, ``I(Vname)`` / ``I(Lname)``, ``TIME``,
  ``TEMP``, ``<R|C name>:R|C`` (the element value) and ``{expressions}`` of
  V(...) / I(...), e.g. ``{V(a)-V(b)}``.

Anything outside the subset (another element letter, a model level, an
unknown model parameter, an expression) raises ``ValueError`` rather than
simulating something else.

Reference behaviour restated:
* source defaults — SIN: FREQ = 1/TSTOP, TD = THETA = PHASE = 0; PULSE:
  TD = 0, TR = TF = TSTEP, PW = PER = TSTOP
  (SinData/PulseData::initializeSource, src/DeviceModelPKG/Core/N_DEV_SourceData.C:342-355,1142-1157);
* ``.prn`` table — an Index column (fixed, width 5, left-justified, header
  "Index"), then TIME and the print variables, each scientific with 9
  digits, width 17, right-justified under a centred header, columns
  separated by one space, footer "End of Xyce(TM) Simulation"
  (src/IOInterfacePKG/N_IO_OutputterLocal.C:201-250,402-423,452-470;
  column defaults src/IOInterfacePKG/N_IO_Outputter.h:91-100,192-193;
  footer src/IOInterfacePKG/N_IO_OutputterTimePrn.C:150-160);
* measures — evaluated at every accepted time point inside [FROM, TO]:
  MAX/MIN the extreme value (src/IOInterfacePKG/Output/N_IO_MeasureExtrema.C:109-165),
  AVG the trapezoid integral over the window divided by its length
  (src/IOInterfacePKG/Output/N_IO_MeasureAverage.C:96-130), ``.mt0`` lines
  ``NAME = value`` in scientific with 6 digits
  (src/IOInterfacePKG/Output/N_IO_MeasureMax.C:141-161).
"""
from __future__ import annotations

import ast
import math
import os
from decimal import Decimal
import re
import sys
from dataclasses import dataclass, field

import numpy as np

from . import netlist as N

# decimal exponents of the engineering suffixes (MIL = 25.4e-6 separately)
_SUFFIX = {"t": 12, "g": 9, "meg": 6, "k": 3, "m": -3, "u": -6, "n": -9, "p": -12, "f": -15}
_NUM = re.compile(r"^([+-]?(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?)(meg|mil|[tgkmunpf])?[a-z]*$", re.I)


def _decimal(tok: str) -> Decimal:
    """Exact decimal value of a SPICE number (engineering suffix, unit letters)."""
    m = _NUM.match(tok.strip())
    if not m:
        raise ValueError(f"not a number: {tok!r}")
    suf = (m.group(2) or "").lower()
    if suf == "mil":
        return Decimal(m.group(1)) * Decimal("25.4e-6")
    return Decimal(m.group(1)).scaleb(_SUFFIX.get(suf, 0))


def number(tok: str) -> float:
    """SPICE number with an optional engineering suffix and unit letters
    (decimal arithmetic: "5u" is the double nearest 5e-6)."""
    return float(_decimal(tok))


def _is_number(tok: str) -> bool:
    return bool(_NUM.match(tok))


def _tokens(line: str) -> list[str]:
    """Tokens of a logical line; a {...} expression stays one token (its
    spaces dropped; its parentheses and commas are its own)."""
    out: list[str] = []
    for part in re.split(r"(\{[^{}]*\})", line):
        if part.startswith("{") and part.endswith("}"):
            out.append("{" + re.sub(r"\s+", "", part[1:-1]) + "}")
        else:
            part = re.sub(r"([(),=])", r" \1 ", part)
            out += [t for t in part.split() if t != ","]
    return out


# ---------------------------------------------------------------------------
# expressions: {...} in element, source and model values and in .PARAM
# (arithmetic, parameters, SPICE numbers, a few functions; the reference's
# expression language, src/UtilityPKG/N_UTL_Expression*, is far larger)

class _Unresolved(ValueError):
    """An expression names a parameter that has no value (yet)."""


_FUNCS = {"SQRT": math.sqrt, "EXP": math.exp, "LOG": math.log, "LN": math.log, "LOG10": math.log10,
          "ABS": abs, "MIN": min, "MAX": max, "POW": math.pow, "PWR": math.pow, "SIN": math.sin,
          "COS": math.cos, "TAN": math.tan, "ATAN": math.atan, "SINH": math.sinh, "COSH": math.cosh,
          "TANH": math.tanh, "FLOOR": math.floor, "CEIL": math.ceil}
_VFUNCS = {"SQRT": np.sqrt, "EXP": np.exp, "LOG": np.log, "LN": np.log, "LOG10": np.log10, "ABS": np.abs,
           "MIN": np.minimum, "MAX": np.maximum, "POW": np.power, "PWR": np.power, "SIN": np.sin,
           "COS": np.cos, "TAN": np.tan, "ATAN": np.arctan, "SINH": np.sinh, "COSH": np.cosh, "TANH": np.tanh,
           "FLOOR": np.floor, "CEIL": np.ceil}
_BINOPS = {ast.Add: lambda a, b: a + b, ast.Sub: lambda a, b: a - b, ast.Mult: lambda a, b: a * b,
           ast.Div: lambda a, b: a / b, ast.Pow: lambda a, b: a ** b}
_SPICE_NUM = re.compile(r"(?<![A-Za-z_0-9.])(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?([A-Za-z]+)?")


def eval_expr(expr: str, params: dict, vector: bool = False):
    """Value of an expression (without its braces) given the parameters
    (upper-case names).  Numbers may carry SPICE suffixes (1k, 2.5MEG, 10n);
    ** and ^ are powers.  vector: the parameters may be arrays (waveforms)
    and the result is an array."""
    src = _SPICE_NUM.sub(lambda m: repr(number(m.group(0))) if m.group(1) else m.group(0), expr)
    try:
        tree = ast.parse(src.replace("^", "**"), mode="eval")
    except SyntaxError as e:
        raise ValueError(f"expression {{{expr}}}: {e.msg}") from None

    def ev(n):
        if isinstance(n, ast.Constant) and isinstance(n.value, (int, float)) and not isinstance(n.value, bool):
            return float(n.value)
        if isinstance(n, ast.Name):
            k = n.id.upper()
            if k in params:
                return params[k] if vector else float(params[k])
            if k == "PI":
                return math.pi
            raise _Unresolved(n.id)
        if isinstance(n, ast.UnaryOp) and isinstance(n.op, (ast.USub, ast.UAdd)):
            v = ev(n.operand)
            return -v if isinstance(n.op, ast.USub) else v
        if isinstance(n, ast.BinOp) and type(n.op) in _BINOPS:
            return _BINOPS[type(n.op)](ev(n.left), ev(n.right))
        if (isinstance(n, ast.Call) and isinstance(n.func, ast.Name) and n.func.id.upper() in _FUNCS
                and not n.keywords):
            if vector:
                return _VFUNCS[n.func.id.upper()](*[ev(a) for a in n.args])
            return float(_FUNCS[n.func.id.upper()](*[ev(a) for a in n.args]))
        raise ValueError(f"expression {{{expr}}}: unsupported element {ast.dump(n)[:40]}")
    try:
        return ev(tree.body)
    except (ZeroDivisionError, OverflowError, TypeError) as e:
        raise ValueError(f"expression {{{expr}}}: {e}") from None


def _param_value(raw: str, params: dict) -> float:
    v = raw.strip()
    if len(v) >= 2 and v[0] in "{'\"" and v[-1] in "}'\"":
        v = v[1:-1]
    return number(v) if _is_number(v) else eval_expr(v, params)


def resolve_params(raw: dict, fixed: dict | None = None) -> dict:
    """.PARAM definitions (NAME -> text) to values, in whatever order they
    refer to each other; fixed values (a sweep point) replace definitions."""
    vals = dict(fixed or {})
    pending = {k: v for k, v in raw.items() if k not in vals}
    while pending:
        progress = False
        for k, v in list(pending.items()):
            try:
                vals[k] = _param_value(v, vals)
            except _Unresolved:
                continue
            del pending[k]
            progress = True
        if not progress:
            raise ValueError(f".PARAM: cannot resolve {sorted(pending)} (an unknown name or a cycle)")
    return vals


_INCLUDE = re.compile(r"^\s*\.INC(?:LUDE)?\s+(['\"]?)(.+?)\1\s*$", re.IGNORECASE)


def _with_includes(lines: list[str], base_dir: str | None, depth: int = 0) -> list[str]:
    """.INCLUDE / .INC lines replaced by the named file's lines (relative to
    the including file's directory; the whole file, no title line)."""
    if depth > 16:
        raise ValueError(".INCLUDE nested more than 16 deep (a cycle?)")
    out: list[str] = []
    for ln in lines:
        m = _INCLUDE.match(ln)
        if not m:
            out.append(ln)
            continue
        path = m.group(2)
        if not os.path.isabs(path):
            path = os.path.join(base_dir or os.getcwd(), path)
        try:
            with open(path) as f:
                body = f.read().splitlines()
        except OSError as e:
            raise ValueError(f".INCLUDE {m.group(2)}: {e.strerror}") from None
        out += _with_includes(body, os.path.dirname(path), depth + 1)
    return out


def _logical_lines(text: str, base_dir: str | None = None) -> tuple[str, list[str]]:
    raw = text.splitlines()
    title = raw[0].strip() if raw else ""
    out: list[str] = []
    for ln in _with_includes(raw[1:], base_dir):
        s = ln.split(";", 1)[0]
        s = re.split(r"\s\$\s", s, maxsplit=1)[0].rstrip()
        st = s.strip()
        if not st or st.startswith("*"):
            continue
        if st.startswith("+"):
            if not out:
                raise ValueError("continuation line without a line to continue")
            out[-1] += " " + st[1:]
        else:
            out.append(st)
    return title, out


def _params(toks: list[str]) -> tuple[list[str], dict[str, str]]:
    """Split a token list into positional tokens and NAME=value pairs."""
    pos, kv = [], {}
    i = 0
    while i < len(toks):
        if i + 1 < len(toks) and toks[i + 1] == "=":
            if i + 2 >= len(toks):
                raise ValueError(f"missing value after {toks[i]}=")
            kv[toks[i].upper()] = toks[i + 2]
            i += 3
        elif toks[i] in ("(", ")"):
            i += 1
        else:
            pos.append(toks[i])
            i += 1
    return pos, kv


@dataclass
class Model:
    name: str
    kind: str                 # D, NMOS, PMOS
    level: int
    params: dict[str, float]


@dataclass
class Measure:
    """func: MAX, MIN, PP, AVG, RMS, INTEG over var; or TRIGTARG, WHEN, FIND
    (spec holds their clauses).  vars: every variable the measure reads."""
    name: str
    func: str
    var: str
    frm: float | None = None
    to: float | None = None
    spec: dict = field(default_factory=dict)
    vars: list = field(default_factory=list)

    def __post_init__(self):
        if not self.vars:
            self.vars = [self.var]


@dataclass
class Deck:
    """A parsed netlist: the flat :class:`Netlist` plus output requests."""
    netlist: N.Netlist
    title: str = ""
    prints: list[str] = field(default_factory=list)
    print_format: str = "STD"                         # .PRINT TRAN FORMAT=STD|NOINDEX|CSV
    measures: list[Measure] = field(default_factory=list)
    tstep: float = 0.0
    element_values: dict[str, float] = field(default_factory=dict)
    branches: dict[str, int] = field(default_factory=dict)
    steps: list = field(default_factory=list)        # .STEP: (name, [values]), outermost first
    params: dict[str, float] = field(default_factory=dict)
    step_values: dict[str, float] = field(default_factory=dict)  # this deck's point of the sweep
    sampling: dict = field(default_factory=dict)     # .SAMPLING vectors + .OPTIONS SAMPLES
    temp_c: float = 27.0                              # .TEMP / .OPTIONS DEVICE TEMP (degrees C)
    embedded: dict = field(default_factory=dict)     # .EMBEDDEDSAMPLING + .OPTIONS EMBEDDEDSAMPLES


_DIODE_ALIASES = {"CJ0": "CJO", "CJ": "CJO", "PB": "VJ", "MJ": "M", "CJP": "CJSW", "PHP": "VJSW"}
_MOS1_MODEL = {"VTO", "KP", "GAMMA", "PHI", "LAMBDA", "RD", "RS", "CBD", "CBS", "IS", "PB", "CGSO",
               "CGDO", "CGBO", "CJ", "MJ", "CJSW", "MJSW", "JS", "TOX", "LD", "FC", "RSH", "TNOM"}
_MOS1_INST = {"W", "L", "AD", "AS", "PD", "PS", "M", "NRD", "NRS", "TEMP", "DTEMP"}
_B4_INST = {"L", "W", "AS", "AD", "PS", "PD", "M"}
_IGNORED_MODEL = {"LEVEL", "VERSION"}


class _Builder:
    def __init__(self, title: str):
        self.nl = N.Netlist(label=title)
        self.deck = Deck(netlist=self.nl, title=title)
        self.models: dict[str, Model] = {}
        self.subckts: dict[str, tuple[list[str], list[str]]] = {}
        self.tran = None
        self.overrides: dict[str, float] = {}  # element name -> swept value
        # .TEMP / .OPTIONS DEVICE TEMP and TNOM (degrees C; the reference's
        # defaults are 27)
        self.temp_c = 27.0
        self.tnom_c = 27.0

    def subst(self, toks: list[str]) -> list[str]:
        """{expression} tokens -> their value from the .PARAM values
        (expressions of waveforms, V(...) / I(...), are left for .PRINT and
        .MEASURE)."""
        out = []
        for t in toks:
            if t.startswith("{") and t.endswith("}") and not re.search(r"(?i)(?<![A-Za-z_0-9])[VI]\(", t):
                try:
                    out.append(repr(eval_expr(t[1:-1], self.deck.params)))
                except _Unresolved as e:
                    raise ValueError(f"unknown parameter {e} in {t}") from None
            else:
                out.append(t)
        return out

    # ---- nodes ----------------------------------------------------------
    def node(self, name: str) -> int:
        u = name.upper()
        if u in ("0", "GND", "GND!"):
            return -1
        if u not in self.nl.names:
            self.nl.node(u)
        return self.nl.names[u]

    # ---- waveforms --------------------------------------------------------
    def _wave(self, name: str, toks: list[str]):
        """(kind, data) of a V/I source specification; the defaults that
        depend on .TRAN are filled in later (kind, data, given flags)."""
        pos, _ = _params(toks)
        up = [t.upper() for t in pos]
        dc = None
        i = 0
        tran = None
        while i < len(up):
            t = up[i]
            if t == "DC":
                dc = number(pos[i + 1])
                i += 2
            elif t == "AC":  # small-signal magnitude and phase: no transient effect
                i += 1
                while i < len(up) and _is_number(pos[i]):
                    i += 1
            elif t in ("SIN", "PULSE", "PWL"):
                j = i + 1
                vals = []
                while j < len(pos) and _is_number(pos[j]):
                    vals.append(number(pos[j]))
                    j += 1
                tran = (t, vals)
                i = j
            elif _is_number(pos[i]):
                dc = number(pos[i])
                i += 1
            else:
                raise ValueError(f"{name}: unsupported source specification {pos[i]!r}")
        if tran is None:
            return ("DC", [dc if dc is not None else 0.0])
        return tran

    # ---- elements ---------------------------------------------------------
    def element(self, toks: list[str], prefix: str, nodemap: dict[str, str]):
        toks = self.subst(toks)
        name = (prefix + toks[0]).upper()
        letter = toks[0][0].upper()
        pos, kv = _params(toks[1:])

        def nd(t):
            t = t.upper()
            if t in nodemap:
                return self.node(nodemap[t])
            if t in ("0", "GND", "GND!"):
                return -1
            return self.node(prefix + t)

        if letter in "RC":
            if len(pos) < 3:
                raise ValueError(f"{name}: needs two nodes and a value")
            a, b, v = nd(pos[0]), nd(pos[1]), number(pos[2])
            v = self.overrides.get(name, v)
            (self.nl.R if letter == "R" else self.nl.C)(a, b, v)
            self.deck.element_values[name] = v
        elif letter == "L":
            if len(pos) < 3:
                raise ValueError(f"{name}: needs two nodes and a value")
            if kv:
                raise ValueError(f"{name}: inductor parameters {sorted(kv)} are not supported (no IC)")
            v = self.overrides.get(name, number(pos[2]))
            self.deck.branches[name] = self.nl.L(nd(pos[0]), nd(pos[1]), v, name=f"{name}#branch")
            self.deck.element_values[name] = v
        elif letter in "VI":
            if len(pos) < 2:
                raise ValueError(f"{name}: needs two nodes")
            a, b = nd(pos[0]), nd(pos[1])
            wave = self._wave(name, toks[3:])
            if name in self.overrides:
                if wave[0] != "DC":
                    raise ValueError(f".STEP of {name}: only DC sources can be stepped")
                wave = ("DC", [self.overrides[name]])
            self._pending_sources.append((letter, name, a, b, wave))
        elif letter == "D":
            if len(pos) < 3:
                raise ValueError(f"{name}: needs two nodes and a model")
            m = self._model(pos[2], "D")
            p = dict(m.params)
            area = kv.get("AREA") or (pos[3] if len(pos) > 3 else None)
            if area is not None:
                p["AREA"] = number(area)
            if "PJ" in kv:
                p["PJ"] = number(kv["PJ"])
            bad = set(kv) - {"AREA", "PJ", "TEMP", "DTEMP"}
            if bad:
                raise ValueError(f"{name}: unsupported diode instance parameter(s) {sorted(bad)}")
            p.update(self._device_temps({k: number(v) for k, v in kv.items()}, p))
            self.nl.D(nd(pos[0]), nd(pos[1]), **p)
        elif letter == "M":
            if len(pos) < 5:
                raise ValueError(f"{name}: needs four nodes and a model")
            m = self._model(pos[4], "M")
            d, g, s, b = (nd(t) for t in pos[:4])
            inst = {k: number(v) for k, v in kv.items()}
            if m.level == 1:
                bad = set(inst) - _MOS1_INST
                if bad:
                    raise ValueError(f"{name}: unsupported MOSFET instance parameter(s) {sorted(bad)}")
                p = dict(m.params)
                p.update(inst)
                p.pop("DTEMP", None)
                p.update(self._device_temps(inst, m.params))
                p["TYPE"] = 1.0 if m.kind == "NMOS" else -1.0
                self.nl.M1(d, g, s, b, **p)
            else:
                bad = set(inst) - _B4_INST
                if bad:
                    raise ValueError(f"{name}: unsupported BSIM4 instance parameter(s) {sorted(bad)}")
                if abs(self.temp_c - 27.0) > 1e-12 or abs(self.tnom_c - 27.0) > 1e-12:
                    raise ValueError(f"{name}: BSIM4 at a temperature other than 27 C is not supported")
                p = dict(m.params)
                p.update(inst)
                p["TYPE"] = 1.0 if m.kind == "NMOS" else -1.0
                self.nl.M4(d, g, s, b, **p)
        elif letter == "X":
            if not pos:
                raise ValueError(f"{name}: needs a subcircuit name")
            sub = pos[-1].upper()
            if sub not in self.subckts:
                raise ValueError(f"{name}: unknown subcircuit {pos[-1]}")
            pins, body = self.subckts[sub]
            conns = pos[:-1]
            if len(conns) != len(pins):
                raise ValueError(f"{name}: {len(conns)} nodes for {len(pins)} pins of {sub}")
            inner = prefix + toks[0].upper() + ":"
            mapping = {}
            for pin, c in zip(pins, conns):
                cu = c.upper()
                mapping[pin] = nodemap.get(cu, cu if cu in ("0", "GND", "GND!") else prefix + cu)
            for ln in body:
                self.element(_tokens(ln), inner, mapping)
        else:
            raise ValueError(f"{name}: element type {letter!r} is not supported")

    def _model(self, mname: str, letter: str) -> Model:
        m = self.models.get(mname.upper())
        if m is None:
            raise ValueError(f"unknown model {mname}")
        if letter == "D" and m.kind != "D":
            raise ValueError(f"model {mname} is not a diode model")
        if letter == "M" and m.kind not in ("NMOS", "PMOS"):
            raise ValueError(f"model {mname} is not a MOSFET model")
        return m

    def _device_temps(self, inst: dict, model_params: dict) -> dict:
        """TEMP and TNOM of a diode or level-1 MOSFET row, kelvin: the
        instance TEMP, else the circuit temperature plus DTEMP
        (Instance::processParams, N_DEV_Diode.C:392-410, N_DEV_MOSFET1.C:383-400);
        the model's TNOM, else .OPTIONS DEVICE TNOM."""
        temp_c = inst["TEMP"] if "TEMP" in inst else self.temp_c + inst.get("DTEMP", 0.0)
        return {"TEMP": temp_c + N.CTOK, "TNOM": model_params.get("TNOM", self.tnom_c + N.CTOK)}

    def model(self, toks: list[str]):
        toks = self.subst(toks)
        pos, kv = _params(toks[1:])
        if len(pos) < 2:
            raise ValueError(".MODEL needs a name and a type")
        name, kind = pos[0].upper(), pos[1].upper()
        level = int(number(kv.get("LEVEL", "1")))
        params = {}
        for k, v in kv.items():
            if k in _IGNORED_MODEL:
                continue
            if k == "TNOM" and not (kind == "D" or level == 1):
                # the BSIM4 restatement runs at TNOM = 27 C only
                if abs(number(v) - 27.0) > 1e-12:
                    raise ValueError(f"model {name}: TNOM other than 27 is not supported")
                continue
            params[k] = number(v) + N.CTOK if k == "TNOM" else number(v)
        if kind == "D":
            out = {}
            for k, v in params.items():
                k = _DIODE_ALIASES.get(k, k)
                if k not in N.DIODE_FIELDS or k in ("BVGIVEN", "NSGIVEN", "PJ", "TEMP"):
                    raise ValueError(f"model {name}: unsupported diode parameter {k}")
                out[k] = v
            params = out
        elif kind in ("NMOS", "PMOS"):
            if level == 1:
                bad = set(params) - _MOS1_MODEL
                if bad:
                    raise ValueError(f"model {name}: unsupported level-1 parameter(s) {sorted(bad)}")
            elif level in (14, 54):
                bad = set(params) - set(N.B4_FIELDS)
                if bad:
                    raise ValueError(f"model {name}: unsupported BSIM4 parameter(s) {sorted(bad)}")
            else:
                raise ValueError(f"model {name}: MOSFET level {level} is not supported")
        else:
            raise ValueError(f"model {name}: type {kind} is not supported")
        self.models[name] = Model(name, kind, level, params)

    # ---- sources need .TRAN for their defaults ----------------------------
    def finish_sources(self, tstep: float, tstop: float):
        for letter, name, a, b, (kind, vals) in self._pending_sources:
            if kind == "DC":
                k, data = N.WAVE_DC, vals
            elif kind == "SIN":
                if len(vals) < 2:
                    raise ValueError(f"{name}: SIN needs at least VO and VA")
                d = list(vals) + [None] * (6 - len(vals))
                data = [d[0], d[1], d[2] if d[2] is not None else 1.0 / tstop,
                        d[3] or 0.0, d[4] or 0.0, d[5] or 0.0]
                k = N.WAVE_SIN
            elif kind == "PULSE":
                if len(vals) < 2:
                    raise ValueError(f"{name}: PULSE needs at least V1 and V2")
                d = list(vals) + [None] * (7 - len(vals))
                data = [d[0], d[1], d[2] or 0.0,
                        d[3] if d[3] is not None else tstep, d[4] if d[4] is not None else tstep,
                        d[5] if d[5] is not None else tstop, d[6] if d[6] is not None else tstop]
                k = N.WAVE_PULSE
            else:
                if len(vals) < 2 or len(vals) % 2:
                    raise ValueError(f"{name}: PWL needs time/value pairs")
                k, data = N.WAVE_PWL, vals
            if letter == "V":
                br = self.nl.V(a, b, k, data, name=f"{name}#branch")
                self.deck.branches[name] = br
            else:
                self.nl.I(a, b, k, data)



# .OPTIONS NONLIN-TRAN keys and the transient fields they set
_NONLIN_TRAN = {"RELTOL": "nl_reltol", "ABSTOL": "nl_abstol", "DELTAXTOL": "nl_deltaxtol",
                "RHSTOL": "nl_rhstol", "SMALLUPDATETOL": "nl_smallupdatetol", "MAXSTEP": "nl_maxstep"}


def parse(text: str, overrides: dict | None = None, base_dir: str | None = None) -> Deck:
    """Parse a netlist (the first line is the title, as in SPICE).
    overrides: {parameter or element name: value} — one point of a .STEP
    sweep (parse_sweep builds them)."""
    title, lines = _logical_lines(text, base_dir)
    B = _Builder(title)
    B._pending_sources = []
    # .PARAM values first (they may be referenced before their line, and
    # refer to each other); a sweep point fixes its parameters, and every
    # parameter defined from them follows
    raw_params = {}
    for ln in lines:
        toks = _tokens(ln)
        if toks[0].upper() == ".PARAM":
            pos, kv = _params(toks[1:])
            if pos:
                raise ValueError(".PARAM takes NAME=value pairs")
            raw_params.update(kv)
    overrides = {k.upper(): float(v) for k, v in (overrides or {}).items()}
    B.deck.params = resolve_params(raw_params, {k: v for k, v in overrides.items() if k in raw_params})
    for k, v in overrides.items():
        if k not in raw_params:
            B.overrides[k] = v
    B.deck.step_values = dict(overrides)
    # pass 1: subcircuit bodies and models
    body_lines = []
    cur = None
    for ln in lines:
        toks = _tokens(ln)
        head = toks[0].upper()
        if head == ".SUBCKT":
            if cur is not None:
                raise ValueError("nested .SUBCKT definitions are not supported")
            pos, kv = _params(toks[1:])
            if kv:
                raise ValueError(".SUBCKT parameters are not supported")
            cur = (pos[0].upper(), [p.upper() for p in pos[1:]], [])
        elif head == ".ENDS":
            if cur is None:
                raise ValueError(".ENDS without .SUBCKT")
            B.subckts[cur[0]] = (cur[1], cur[2])
            cur = None
        elif cur is not None:
            if head == ".MODEL":
                B.model(toks)
            elif head.startswith("."):
                raise ValueError(f"{head} inside a subcircuit is not supported")
            else:
                cur[2].append(ln)
        elif head == ".MODEL":
            B.model(toks)
        else:
            body_lines.append((ln, toks))
    if cur is not None:
        raise ValueError(".SUBCKT without .ENDS")
    tran = None
    tstep = 0.0
    reltol = abstol = method = maxord = delmax = None
    nonlin = {}
    deck = B.deck
    # the circuit temperature applies to every device, wherever the line is
    for ln, toks in body_lines:
        head = toks[0].upper()
        if head == ".TEMP":
            vals = [number(t) for t in B.subst(toks[1:])]
            if len(vals) != 1:
                raise ValueError(".TEMP takes one temperature (no sweeps)")
            B.temp_c = deck.temp_c = vals[0]
        elif head == ".OPTIONS" and len(toks) > 1 and toks[1].upper() == "DEVICE":
            pos, kv = _params(B.subst(toks)[2:])
            for k, v in kv.items():
                if k == "TEMP":
                    B.temp_c = deck.temp_c = number(v)
                elif k == "TNOM":
                    B.tnom_c = number(v)
                else:
                    raise ValueError(f".OPTIONS DEVICE {k} is not supported")
    for ln, toks in body_lines:
        head = toks[0].upper()
        if head == ".END":
            break
        if head in (".PARAM", ".TEMP") or (head == ".OPTIONS" and len(toks) > 1 and toks[1].upper() == "DEVICE"):
            continue
        if head == ".SAMPLING":
            deck.sampling.update(_sampling_spec(ln))
            continue
        if head == ".EMBEDDEDSAMPLING":
            deck.embedded.update(_sampling_spec(ln, ".EMBEDDEDSAMPLING"))
            continue
        if head == ".OPTIONS" and len(toks) > 1 and toks[1].upper() == "EMBEDDEDSAMPLES":
            deck.embedded.update(_embedded_options(ln))
            continue
        if head == ".OPTIONS" and len(toks) > 1 and toks[1].upper() == "SAMPLES":
            pos, kv = _params(toks[2:])
            for k, v in kv.items():
                if k == "NUMSAMPLES":
                    deck.sampling["NUMSAMPLES"] = int(number(v))
                elif k == "SEED":
                    deck.sampling["SEED"] = int(number(v))
                elif k == "SAMPLE_TYPE":
                    if v.upper() not in ("LHS", "MC"):
                        raise ValueError("SAMPLE_TYPE must be LHS or MC")
                    deck.sampling["SAMPLE_TYPE"] = v.upper()
                else:
                    raise ValueError(f".OPTIONS SAMPLES {k} is not supported")
            continue
        if head == ".STEP":
            deck.steps.append(_step(toks[1:]))
            continue
        toks = B.subst(toks)
        if head == ".TRAN":
            pos, kv = _params(toks[1:])
            nums = [number(p) for p in pos if _is_number(p)]
            if len(nums) < 2:
                raise ValueError(".TRAN needs TSTEP and TSTOP")
            tstep, tstop = nums[0], nums[1]
            tstart = nums[2] if len(nums) > 2 else 0.0
            hmax = nums[3] if len(nums) > 3 else 0.0
            tran = N.Tran(tstop=tstop, tstart=tstart, hmax=hmax)
        elif head == ".OPTIONS":
            pos, kv = _params(toks[1:])
            pkg = pos[0].upper() if pos else ""
            if pkg == "TIMEINT":
                for k, v in kv.items():
                    if k == "RELTOL":
                        reltol = number(v)
                    elif k == "ABSTOL":
                        abstol = number(v)
                    elif k == "METHOD":
                        mv = v.upper()
                        methods = {"TRAP": 7, "TRAPEZOID": 7, "7": 7, "1": 7, "GEAR": 8, "8": 8}
                        if mv not in methods:
                            raise ValueError(f".OPTIONS TIMEINT METHOD={v} is not supported")
                        method = methods[mv]
                    elif k == "DELMAX":
                        # the largest step, with .TRAN's TMAX the smaller of the
                        # two (StepErrorControl, N_TIA_StepErrorControl.C:899-901)
                        delmax = number(v)
                        if not delmax > 0:
                            raise ValueError("DELMAX must be positive")
                    elif k == "MAXORD":
                        maxord = int(number(v))
                        if maxord not in (1, 2):
                            raise ValueError("MAXORD must be 1 or 2")
                    else:
                        raise ValueError(f".OPTIONS TIMEINT {k} is not supported")
            elif pkg == "NONLIN-TRAN":
                # the transient Newton's options (N_NLS_NLParams.C:191-220)
                for k, v in kv.items():
                    if k not in _NONLIN_TRAN:
                        raise ValueError(f".OPTIONS NONLIN-TRAN {k} is not supported")
                    nonlin[_NONLIN_TRAN[k]] = int(number(v)) if k == "MAXSTEP" else number(v)
            elif pkg == "LINSOL":
                # every direct solver the reference offers factors and solves the
                # same system; this path's is the GPU LU
                for k, v in kv.items():
                    if k != "TYPE" or v.upper() not in ("DEFAULT", "KLU", "KSPARSE"):
                        raise ValueError(f".OPTIONS LINSOL {k}={v} is not supported")
            else:
                raise ValueError(f".OPTIONS {pkg} is not supported")
        elif head == ".PRINT":
            if len(toks) < 2 or toks[1].upper() != "TRAN":
                raise ValueError("only .PRINT TRAN is supported")
            rest = toks[2:]
            while len(rest) >= 3 and rest[1] == "=":
                key, val = rest[0].upper(), rest[2].upper()
                if key != "FORMAT" or val not in ("STD", "NOINDEX", "CSV"):
                    raise ValueError(f".PRINT TRAN {key}={val} is not supported")
                deck.print_format = val
                rest = rest[3:]
            deck.prints.extend(_print_vars(rest))
        elif head in (".MEASURE", ".MEAS"):
            deck.measures.append(_measure(toks[1:]))
        elif head.startswith("."):
            raise ValueError(f"{head} is not supported")
        else:
            B.element(toks, "", {})
    if tran is None:
        raise ValueError("no .TRAN line")
    unknown = [k for k in B.overrides if k not in deck.element_values and k not in
               {src[1] for src in B._pending_sources}]
    if unknown:
        raise ValueError(f".STEP names no parameter or element: {unknown}")
    if reltol is not None:
        tran.reltol = reltol
    if abstol is not None:
        tran.abstol = abstol
    if method is not None:
        tran.method = method
    if maxord is not None:
        tran.max_order = maxord
    if delmax is not None:
        tran.hmax = min(tran.hmax, delmax) if tran.hmax > 0 else delmax
    for k, v in nonlin.items():
        setattr(tran, k, v)
    B.finish_sources(tstep, tran.tstop)
    B.nl.tran = tran
    B.nl.end_circuit()
    deck.tstep = tstep
    return deck


def read(path: str) -> Deck:
    with open(path) as f:
        return parse(f.read())


def _step(toks: list[str]) -> tuple[str, list[float]]:
    """.STEP [LIN] NAME start stop step | .STEP DEC|OCT NAME start stop
    points | .STEP NAME LIST v1 v2 ... (SweepParam, src/AnalysisPKG/
    N_ANP_SweepParam.C:95-135, 385-440: DEC and OCT multiply by
    exp(ln 10 / points) or exp(ln 2 / points), floor(decades * points + 1)
    values; a start above the stop gives the start alone)."""
    pos, kv = _params(toks)
    if len(pos) < 2:
        raise ValueError(".STEP needs a name and values")
    kind = pos[0].upper()
    if kind in ("DEC", "OCT"):
        if len(pos) != 5:
            raise ValueError(f".STEP {kind} NAME start stop points")
        name, a, b, pts = pos[1].upper(), number(pos[2]), number(pos[3]), number(pos[4])
        if not (a > 0 and b > 0 and pts >= 1):
            raise ValueError(f".STEP {kind}: start and stop must be positive, points at least 1")
        base = 10.0 if kind == "DEC" else 2.0
        mult = math.exp(math.log(base) / pts)
        if a > b + 2.0 * 2.220446049250313e-16:
            return name, [a]
        count = int(math.floor(abs(math.log(a) - math.log(b)) / math.log(base) * pts + 1))
        return name, [a * mult ** k for k in range(count)]
    if kind == "LIN":
        pos = pos[1:]
    name = pos[0].upper()
    if pos[1].upper() == "LIST":
        vals = [number(v) for v in pos[2:]]
        if not vals:
            raise ValueError(".STEP LIST needs values")
        return name, vals
    if len(pos) != 4:
        raise ValueError(".STEP NAME start stop step")
    a, b, st = _decimal(pos[1]), _decimal(pos[2]), _decimal(pos[3])
    if st == 0 or (b - a) / st < 0:
        raise ValueError(".STEP step must move from start towards stop")
    k = int((b - a) / st) + 1  # decimal: the end point is not lost to rounding
    return name, [float(a + i * st) for i in range(k)]


def _sampling_spec(line: str, what: str = ".SAMPLING") -> dict:
    """.SAMPLING PARAM=a,b TYPE=normal,uniform MEANS=.. STD_DEVIATIONS=..
    LOWER_BOUNDS=.. UPPER_BOUNDS=.. (vectors, one entry per parameter;
    the keys of Sampling, src/AnalysisPKG/N_ANP_Sampling.C:200-260, and of
    EmbeddedSampling::setAnalysisParams, N_ANP_EmbeddedSampling.C:291-380)."""
    body = line.split(None, 1)[1] if len(line.split(None, 1)) > 1 else ""
    out = {}
    for m in re.finditer(r"(\w+)\s*=\s*(.*?)(?=\s+\w+\s*=|$)", body):
        key = m.group(1).upper()
        vals = [v for v in re.split(r"[,\s]+", m.group(2).strip()) if v]
        if key in ("PARAM", "TYPE"):
            out[key] = [v.upper() for v in vals]
        elif key in ("MEANS", "STD_DEVIATIONS", "LOWER_BOUNDS", "UPPER_BOUNDS"):
            out[key] = [number(v) for v in vals]
        else:
            raise ValueError(f"{what} {key} is not supported")
    return out


def _embedded_options(line: str) -> dict:
    """.OPTIONS EMBEDDEDSAMPLES NUMSAMPLES= SAMPLE_TYPE=LHS|MC SEED=
    OUTPUTS={expr},{expr} OUTPUT_SAMPLE_STATS= OUTPUT_ALL_SAMPLES=
    OUTPUTFORMAT=STD|TECPLOT (EmbeddedSampling::setEmbeddedSamplingOptions,
    N_ANP_EmbeddedSampling.C:513-640; defaults :2044-2065).  The polynomial
    chaos options are not supported."""
    parts = line.split(None, 2)
    body = parts[2] if len(parts) > 2 else ""
    out = {}
    flag = lambda v: v.strip().upper() in ("1", "TRUE", "YES") or (_is_number(v) and number(v) != 0)
    for m in re.finditer(r"(\w+)\s*=\s*(.*?)(?=\s+\w+\s*=|$)", body):
        key, val = m.group(1).upper(), m.group(2).strip()
        if key == "OUTPUTS":
            outs = re.findall(r"\{([^}]*)\}", val) or [v for v in re.split(r"[,\s]+", val) if v]
            out["OUTPUTS"] = [o.strip().upper() for o in outs]
        elif key in ("NUMSAMPLES", "SEED"):
            out[key] = int(number(val))
        elif key == "SAMPLE_TYPE":
            if val.upper() not in ("LHS", "MC"):
                raise ValueError("SAMPLE_TYPE must be LHS or MC")
            out[key] = val.upper()
        elif key in ("OUTPUT_SAMPLE_STATS", "OUTPUT_ALL_SAMPLES"):
            out[key] = flag(val)
        elif key == "OUTPUTFORMAT":
            if val.upper() not in ("STD", "TECPLOT"):
                raise ValueError("OUTPUTFORMAT must be STD or TECPLOT")
            out[key] = val.upper()
        else:
            raise ValueError(f".OPTIONS EMBEDDEDSAMPLES {key} is not supported")
    if out.get("NUMSAMPLES", 1) < 1:
        raise ValueError("NUMSAMPLES on .OPTIONS EMBEDDEDSAMPLES must be > 0")
    return out


def sample_points(spec: dict) -> list[dict]:
    """Parameter values of every sample: Latin hypercube (default) or plain
    Monte Carlo, NORMAL (MEANS, STD_DEVIATIONS) or UNIFORM (LOWER_BOUNDS,
    UPPER_BOUNDS) marginals; numpy's generator seeded with SEED (0 by
    default), so the samples are reproducible but not the reference's
    (it draws from its own generator)."""
    import statistics
    names = spec.get("PARAM", [])
    types = spec.get("TYPE", [])
    n = int(spec.get("NUMSAMPLES", 1))
    if not names or len(types) != len(names):
        raise ValueError(".SAMPLING needs PARAM and one TYPE per parameter")
    if n < 1:
        raise ValueError("NUMSAMPLES must be positive")
    rng = np.random.default_rng(int(spec.get("SEED", 0)))
    lhs = spec.get("SAMPLE_TYPE", "LHS") == "LHS"
    cols = {}
    iN = iU = 0
    for name, ty in zip(names, types):
        u = (rng.permutation(n) + rng.uniform(size=n)) / n if lhs else rng.uniform(size=n)
        u = np.clip(u, 1e-12, 1 - 1e-12)
        if ty == "NORMAL":
            mu, sd = spec["MEANS"][iN], spec["STD_DEVIATIONS"][iN]
            iN += 1
            if sd < 0:
                raise ValueError("STD_DEVIATIONS must be >= 0")
            nd = statistics.NormalDist(mu, sd) if sd > 0 else None
            cols[name] = [nd.inv_cdf(float(x)) if nd else mu for x in u]
        elif ty == "UNIFORM":
            lo, hi = spec["LOWER_BOUNDS"][iU], spec["UPPER_BOUNDS"][iU]
            iU += 1
            cols[name] = [lo + float(x) * (hi - lo) for x in u]
        else:
            raise ValueError(f".SAMPLING TYPE {ty} is not supported (NORMAL, UNIFORM)")
    return [{name: cols[name][k] for name in names} for k in range(n)]


def sample_moments(values) -> dict:
    """Mean, population standard deviation and variance, skew, kurtosis,
    min and max of one output over the samples; non-finite moments read 0
    (computeMoments, src/AnalysisPKG/N_ANP_UQSupport.C:80-135)."""
    v = np.asarray(values, np.float64)
    if len(v) == 0:
        return {}
    mean = v.mean()
    var = np.mean((v - mean) ** 2)
    sd = np.sqrt(var)
    mu3 = np.mean(v ** 3) - 3 * mean * np.mean(v ** 2) + 2 * mean ** 3
    mu4 = np.mean(v ** 4) - 4 * mean * np.mean(v ** 3) + 6 * mean ** 2 * np.mean(v ** 2) - 3 * mean ** 4
    with np.errstate(divide="ignore", invalid="ignore"):
        skew, kurt = mu3 / sd ** 3, mu4 / sd ** 4
    fix = lambda x: float(x) if np.isfinite(x) else 0.0
    return dict(mean=fix(mean), stddev=fix(sd), variance=fix(var), skew=fix(skew), kurtosis=fix(kurt),
                min=float(v.min()), max=float(v.max()))


def parse_sampling(text: str, base_dir: str | None = None) -> list[Deck]:
    """One deck per sample of the deck's .SAMPLING block."""
    base = parse(text, base_dir=base_dir)
    if not base.sampling:
        return [base]
    return [parse(text, pt, base_dir) for pt in sample_points(base.sampling)]


def parse_embedded(text: str, base_dir: str | None = None) -> list[Deck]:
    """One deck per sample of the deck's .EMBEDDEDSAMPLING block (the same
    parameter vectors and sample generator as .SAMPLING)."""
    base = parse(text, base_dir=base_dir)
    if not base.embedded:
        raise ValueError("the deck has no .EMBEDDEDSAMPLING")
    if base.sampling or base.steps:
        raise ValueError(".EMBEDDEDSAMPLING with .SAMPLING or .STEP is not supported")
    return [parse(text, pt, base_dir) for pt in sample_points(base.embedded)]


def ensemble_netlist(decks: list[Deck]) -> tuple[N.Netlist, list[int]]:
    """Every sample as a block of ONE circuit, and each block's first
    unknown.  As in the reference's embedded sampling (ESLoader and the
    block vectors of N_ANP_EmbeddedSampling.C) the blocks share one
    transient: one step sequence, one Newton solve per step over the whole
    block system, error norms over every block, every sample's breakpoints.
    (.SAMPLING instead runs each sample as its own circuit of a batch, with
    its own step control.)"""
    nl = N.batch([d.netlist for d in decks], label=decks[0].title)
    bases = list(nl.offsets[:-1])
    nl.offsets = [0, nl.n]
    return nl, bases


@dataclass
class Ensemble:
    """An embedded-sampling run: the shared time points and, per output,
    every sample's values [n_samples, n_points]."""
    times: np.ndarray
    samples: dict[str, np.ndarray]
    stats: dict

    def moments(self, var: str) -> dict:
        """Mean, population standard deviation and variance over the samples
        at every time point (computeMoments, N_ANP_UQSupport.C:80-135)."""
        v = self.samples[var]
        mean = v.mean(axis=0)
        var_ = np.mean((v - mean) ** 2, axis=0)
        return dict(mean=mean, stddev=np.sqrt(var_), variance=var_)


def _gpu_transient(nl: N.Netlist, probes: list[int], cap: int, device: int = 0):
    from . import Circuit
    circ = Circuit(nl, device=device)
    try:
        counts, times, values, stats = circ.transient(nl.tran, probes=probes, cap=cap)
    finally:
        circ.close()
    n = int(counts[0])
    return times[0, :n].copy(), values[0, :n, :].copy(), stats


def run_embedded(decks: list[Deck], device: int = 0, cap: int | None = None, transient=None) -> Ensemble:
    """The samples as one block system on the GPU (ensemble_netlist).
    Outputs: OUTPUTS of .OPTIONS EMBEDDEDSAMPLES, else the .PRINT variables.
    transient(nl, probes, cap) -> (times, values[points, probes], stats)
    replaces the GPU run (a checker drives the same netlist through it)."""
    spec = decks[0].embedded
    outs = spec.get("OUTPUTS") or [v for v in decks[0].prints if v != "TIME"]
    if not outs:
        raise ValueError("embedded sampling needs OUTPUTS or .PRINT variables")
    nl, bases = ensemble_netlist(decks)
    probes, plan, slot_of = [], [], {}
    for d, base in zip(decks, bases):
        row = []
        for var in outs:
            us, f = _var_probes(d, var)
            slots = []
            for u in us:
                if base + u not in slot_of:  # each unknown is probed once
                    slot_of[base + u] = len(probes)
                    probes.append(base + u)
                slots.append(slot_of[base + u])
            row.append((us, slots, f))
        plan.append(row)
    if not probes:
        probes = [0]
    if cap is None:
        tr = nl.tran
        hmin_guess = tr.hmax if tr.hmax > 0 else tr.tstop / 50.0
        cap = int(min(2_000_000, max(4096, 20 * tr.tstop / max(hmin_guess, 1e-30))))
    run_t = transient or (lambda n_, p_, c_: _gpu_transient(n_, p_, c_, device))
    for _ in range(4):
        t, vals, stats = run_t(nl, probes, cap)
        if len(t) < cap:
            break
        cap *= 4
    else:
        raise RuntimeError(f"more than {cap} accepted steps")
    samples = {}
    for j, var in enumerate(outs):
        cols = []
        for row in plan:
            us, slots, f = row[j]
            sub_ = {u: vals[:, s] for u, s in zip(us, slots)}
            cols.append(np.broadcast_to(np.asarray(f(sub_), np.float64), t.shape))
        samples[var] = np.stack(cols)
    return Ensemble(t, samples, stats)


def write_ensemble(path: str, deck: Deck, ens: Ensemble) -> str:
    """<netlist>_ensemble.prn (OUTPUTFORMAT=STD, the default) or .dat
    (TECPLOT) in the reference's layout (EmbeddedSampling::hackEnsembleOutput,
    N_ANP_EmbeddedSampling.C:1377-1560): a TECPLOT-style header naming TIME
    and, per output, its mean, mean -/+ one and two standard deviations,
    standard deviation and variance (OUTPUT_SAMPLE_STATS) and every sample
    (OUTPUT_ALL_SAMPLES), then one row per accepted time point."""
    spec = deck.embedded
    stats_on = spec.get("OUTPUT_SAMPLE_STATS", True)
    all_on = spec.get("OUTPUT_ALL_SAMPLES", False)
    out = path + ("_ensemble.dat" if spec.get("OUTPUTFORMAT", "STD") == "TECPLOT" else "_ensemble.prn")
    names = list(ens.samples)
    with open(out, "w") as f:
        f.write('TITLE = "embedded sampling output"\tVARIABLES= \n')
        f.write('\t" TIME "\n')
        for var in names:
            if stats_on:
                for suffix in ("_mean", "_meanPlus", "_meanMinus", "_meanPlusTwoSigma", "_meanMinusTwoSigma",
                               "_stddev", "_variance"):
                    f.write(f'\t" {var}{suffix}"\n')
            if all_on:
                for i in range(ens.samples[var].shape[0]):
                    f.write(f'\t" {var}_{i}"\n')
        f.write('ZONE F=POINT  T="Xyce data"\n')
        mom = {var: ens.moments(var) for var in names}
        for k, t in enumerate(ens.times):
            cells = [f"{t:.6e}"]
            for var in names:
                if stats_on:
                    m, s, v = mom[var]["mean"][k], mom[var]["stddev"][k], mom[var]["variance"][k]
                    cells += [f"{x:.6e}" for x in (m, m + s, m - s, m + 2 * s, m - 2 * s, s, v)]
                if all_on:
                    cells += [f"{x:.6e}" for x in ens.samples[var][:, k]]
            f.write("\t".join(cells) + "\n")
    return out


def parse_sweep(text: str, base_dir: str | None = None) -> list[Deck]:
    """One deck per point of the .STEP sweep (the first .STEP line
    outermost); a single deck without .STEP."""
    base = parse(text, base_dir=base_dir)
    if not base.steps:
        return [base]
    combos = [{}]
    for name, vals in base.steps:
        combos = [dict(c, **{name: v}) for c in combos for v in vals]
    return [parse(text, c, base_dir) for c in combos]


def run_sweep(decks: list[Deck], device: int = 0, cap: int | None = None) -> list["Result"]:
    """All points of a sweep as the circuits of one batch on the GPU (each
    keeps its own step control); one Result per deck."""
    if len(decks) == 1:
        return [run(decks[0], device, cap)]
    from . import Circuit
    nl = N.batch([d.netlist for d in decks], label=decks[0].title)
    plans, probes = [], []
    for k, d in enumerate(decks):
        base = nl.offsets[k]
        wanted = list(dict.fromkeys(d.prints + [v for m in d.measures for v in m.vars]))
        local: list[int] = []
        plan = {}
        for var in wanted:
            us, f = _var_probes(d, var)
            slots = []
            for u in us:
                if u not in local:
                    local.append(u)
                slots.append(local.index(u))
            plan[var] = (us, slots, f)
        if not local:
            local = [0]
        probes += [base + u for u in local]
        plans.append((wanted, plan))
    if cap is None:
        tr = nl.tran
        hmin_guess = tr.hmax if tr.hmax > 0 else tr.tstop / 50.0
        cap = int(min(2_000_000, max(4096, 20 * tr.tstop / max(hmin_guess, 1e-30))))
    for _ in range(4):
        circ = Circuit(nl, device=device)
        try:
            counts, times, values, stats = circ.transient(nl.tran, probes=probes, cap=cap)
        finally:
            circ.close()
        if int(np.max(counts)) < cap:
            break
        cap *= 4
    else:
        raise RuntimeError(f"more than {cap} accepted steps")
    out = []
    for k, d in enumerate(decks):
        n = int(counts[k])
        out.append(_columns(d, plans[k][0], plans[k][1], times[k, :n].copy(), values[k, :n, :], stats))
    return out


def _columns(deck: Deck, wanted, plan, t, vals, stats) -> "Result":
    cols = {}
    for var in wanted:
        us, slots, f = plan[var]
        if var == "TIME":
            cols[var] = t
            continue
        sub = {u: vals[:, s] for u, s in zip(us, slots)}
        cols[var] = np.broadcast_to(np.asarray(f(sub), dtype=np.float64), t.shape).copy()
    meas = {m.name: evaluate_measure(m, t, cols) for m in deck.measures}
    return Result(t, cols, meas, stats)


def _print_vars(toks: list[str]) -> list[str]:
    """Re-join V(a,b) / I(x) tokens into column names."""
    out = []
    i = 0
    while i < len(toks):
        t = toks[i]
        if i + 1 < len(toks) and toks[i + 1] == "(":
            j = toks.index(")", i)
            args = [a for a in toks[i + 2:j]]
            out.append(f"{t.upper()}({','.join(a.upper() for a in args)})")
            i = j + 1
        else:
            out.append(t.upper())
            i += 1
    return out


_RFC = ("RISE", "FALL", "CROSS")
MINVAL = 1e-12  # the measures' MINVAL default, N_IO_MeasureBase.C:69


def _one_var(toks: list[str], i: int) -> tuple[str, int]:
    if i + 1 < len(toks) and toks[i + 1] == "(" and ")" in toks[i:]:
        j = toks.index(")", i)
        return f"{toks[i].upper()}({','.join(a.upper() for a in toks[i + 2:j])})", j + 1
    raise ValueError(f".MEASURE: expected V(...) or I(...) at {' '.join(toks[i:i + 3])}")


def _kv_run(toks: list[str], i: int) -> tuple[dict, int]:
    """KEY = VALUE pairs from toks[i] on."""
    out = {}
    while i + 2 < len(toks) + 1 and i + 1 < len(toks) and toks[i + 1] == "=" and toks[i] != "=":
        out[toks[i].upper()] = toks[i + 2]
        i += 3
    return out, i


def _rfc(kv: dict) -> tuple:
    """(RISE|FALL|CROSS or None, count); count -1 = LAST; none given: the
    first crossing."""
    given = [k for k in _RFC if k in kv]
    if len(given) > 1:
        raise ValueError(".MEASURE: give one of RISE, FALL, CROSS")
    if not given:
        return None, 0
    v = kv[given[0]].upper()
    return given[0], (-1 if v == "LAST" else int(number(v)))


def _timing_measure(name: str, toks: list[str]) -> Measure:
    """TRIG/TARG (RiseFallDelay), WHEN and FIND ... WHEN / AT (FindWhen,
    WhenAT), src/IOInterfacePKG/Output/N_IO_MeasureRiseFallDelay.C,
    N_IO_MeasureFindWhen.C, N_IO_MeasureWhenAT.C."""
    head = toks[0].upper()
    allowed = set(_RFC) | {"TD", "FROM", "TO", "VAL"}

    def clause(i):
        var, i = _one_var(toks, i)
        kv, i = _kv_run(toks, i)
        bad = set(kv) - allowed
        if bad or "VAL" not in kv:
            raise ValueError(f".MEASURE {name}: TRIG/TARG need VAL= (and only {sorted(allowed)})")
        return dict(var=var, val=number(kv["VAL"]), td=number(kv.get("TD", "0")), rfc=_rfc(kv)), i

    def when(i):
        var, i = _one_var(toks, i)
        if i + 1 >= len(toks) or toks[i] != "=":
            raise ValueError(f".MEASURE {name}: WHEN <var>=<value>")
        val = number(toks[i + 1])
        kv, i = _kv_run(toks, i + 2)
        bad = set(kv) - (allowed - {"VAL"})
        if bad:
            raise ValueError(f".MEASURE {name}: unsupported {sorted(bad)}")
        spec = dict(var=var, val=val, rfc=_rfc(kv), td=number(kv.get("TD", "0")),
                    frm=number(kv["FROM"]) if "FROM" in kv else None, to=number(kv["TO"]) if "TO" in kv else None)
        return spec, i

    if head == "TRIG":
        trig, i = clause(1)
        if i >= len(toks) or toks[i].upper() != "TARG":
            raise ValueError(f".MEASURE {name}: TRIG ... TARG ...")
        targ, i = clause(i + 1)
        if i != len(toks):
            raise ValueError(f".MEASURE {name}: unexpected {' '.join(toks[i:])}")
        return Measure(name, "TRIGTARG", trig["var"], spec=dict(trig=trig, targ=targ), vars=[trig["var"], targ["var"]])
    if head == "WHEN":
        w, i = when(1)
        if i != len(toks):
            raise ValueError(f".MEASURE {name}: unexpected {' '.join(toks[i:])}")
        return Measure(name, "WHEN", w["var"], spec=dict(when=w), vars=[w["var"]])
    # FIND|DERIV <var> WHEN ... | FIND|DERIV <var> AT=<t>
    func = "FIND" if head == "FIND" else "DERIV"
    fvar, i = _one_var(toks, 1)
    if i < len(toks) and toks[i].upper() == "WHEN":
        w, i = when(i + 1)
        if i != len(toks):
            raise ValueError(f".MEASURE {name}: unexpected {' '.join(toks[i:])}")
        return Measure(name, func, fvar, spec=dict(when=w), vars=[fvar, w["var"]])
    kv, i = _kv_run(toks, i)
    if set(kv) != {"AT"} or i != len(toks):
        raise ValueError(f".MEASURE {name}: {head} <var> WHEN ... or {head} <var> AT=<time>")
    return Measure(name, func, fvar, spec=dict(at=number(kv["AT"])), vars=[fvar])


def _measure(toks: list[str]) -> Measure:
    if len(toks) >= 3 and toks[0].upper() == "TRAN" and toks[2].upper() in ("TRIG", "WHEN", "FIND", "DERIV",
                                                                             "DERIVATIVE"):
        return _timing_measure(toks[1].upper(), toks[2:])
    pos, kv = _params(toks)
    if len(pos) < 3 or pos[0].upper() != "TRAN":
        raise ValueError(".MEASURE TRAN <name> <func> <var> is the supported form")
    name, func = pos[1].upper(), pos[2].upper()
    if func in ("FREQ", "DUTY", "ON_TIME", "OFF_TIME"):
        var = _print_vars(toks[toks.index(pos[2]) + 1:])
        bad = set(kv) - {"ON", "OFF", "FROM", "TO"}
        if not var or bad:
            raise ValueError(f".MEASURE {name}: {func} <var> ON= OFF= [FROM= TO=]")
        return Measure(name, func, var[0], number(kv["FROM"]) if "FROM" in kv else None,
                       number(kv["TO"]) if "TO" in kv else None,
                       spec=dict(on=number(kv.get("ON", "0")), off=number(kv.get("OFF", "0"))))
    if func not in ("MAX", "MIN", "PP", "AVG", "RMS", "INTEG"):
        raise ValueError(f".MEASURE {func} is not supported")
    var = _print_vars(toks[toks.index(pos[2]) + 1:])
    if not var:
        raise ValueError(f".MEASURE {name}: no variable")
    frm = number(kv["FROM"]) if "FROM" in kv else None
    to = number(kv["TO"]) if "TO" in kv else None
    return Measure(name, func, var[0], frm, to)


# ---------------------------------------------------------------------------
# evaluation of print variables on the probe waveforms

def _var_probes(deck: Deck, var: str) -> tuple[list[int], callable]:
    """Unknowns a variable needs and how to combine them (probe values ->
    column).  Ground reads as 0."""
    names = deck.netlist.names
    m = re.match(r"^V\(([^,()]+)(?:,([^,()]+))?\)$", var)
    if m:
        def idx(nm):
            if nm in ("0", "GND", "GND!"):
                return None
            if nm not in names:
                raise ValueError(f"{var}: unknown node {nm}")
            return names[nm]
        a, b = idx(m.group(1)), idx(m.group(2)) if m.group(2) else None
        us = [u for u in (a, b) if u is not None]

        def f(vals, a=a, b=b):
            va = vals[a] if a is not None else 0.0
            vb = vals[b] if b is not None else 0.0
            return va - vb
        return us, f
    m = re.match(r"^I\(([^,()]+)\)$", var)
    if m:
        src = m.group(1)
        if src not in deck.branches:
            raise ValueError(f"{var}: only voltage-source and inductor currents are supported")
        br = deck.branches[src]
        return [br], lambda vals, br=br: vals[br]
    if var == "TEMP":
        return [], lambda vals, tc=deck.temp_c: tc
    m = re.match(r"^([RC][^:]*):([RC])$", var)
    if m and m.group(1) in deck.element_values and m.group(1)[0] == m.group(2):
        v = deck.element_values[m.group(1)]
        return [], lambda vals, v=v: v
    if var == "TIME":
        return [], None
    if var.startswith("{") and var.endswith("}"):
        # an expression of V(...) / I(...) columns, e.g. {V(A)-V(B)} or {I(V1)*V(IN)}
        body = var[1:-1]
        refs = list(dict.fromkeys(re.findall(r"[VI]\([^()]*\)", body)))
        parts = [_var_probes(deck, r) for r in refs]
        expr = body
        for k, r in enumerate(refs):
            expr = expr.replace(r, f"__R{k}")
        eval_expr(expr, {f"__R{k}": 0.0 for k in range(len(refs))})  # syntax and names, early
        us = list(dict.fromkeys(u for ps, _ in parts for u in ps))

        def f(vals, parts=parts, expr=expr):
            env = {f"__R{k}": np.asarray(g(vals), np.float64) for k, (ps, g) in enumerate(parts)}
            return eval_expr(expr, env, vector=True)
        return us, f
    raise ValueError(f"print variable {var} is not supported")


@dataclass
class Result:
    times: np.ndarray
    columns: dict[str, np.ndarray]
    measures: dict[str, float]
    stats: dict


def _rfc_event_time(t, v, val, rfc, td):
    """TRIG or TARG: the time of the counted crossing of val (RISE: v - val
    from < 0 to >= 0; FALL: from > 0 to <= 0; CROSS: either; none given:
    the first crossing), over the points at or after TD, interpolated
    linearly between the two points around it; LAST: the last such
    crossing (Base::withinRiseFallCrossWindow, N_IO_MeasureBase.C:781-880;
    RiseFallDelay::updateTran, N_IO_MeasureRiseFallDelay.C:220-470)."""
    kind, count = rfc
    sel = t >= td * (1 - MINVAL)
    t, v = t[sel], v[sel]
    nr = nf = nc = 0
    found = float("nan")
    for k in range(1, len(t)):
        a, b = v[k - 1] - val, v[k] - val
        rise, fall = (b >= 0.0 and a < 0.0), (b <= 0.0 and a > 0.0)
        if not (rise or fall):
            continue
        nr += rise
        nf += fall
        nc += 1
        hit = ((kind is None and nc == 1) or (kind == "RISE" and rise and (nr == count or count < 0)) or
               (kind == "FALL" and fall and (nf == count or count < 0)) or
               (kind == "CROSS" and (nc == count or count < 0)))
        if hit:
            dv = v[k] - v[k - 1]
            found = t[k - 1] if abs(dv) < MINVAL else t[k - 1] + (t[k] - t[k - 1]) * (val - v[k - 1]) / dv
            if count >= 0:
                break
    return found


def _when(t, v, f, w):
    """WHEN (and FIND ... WHEN): the interpolated time at which v reaches
    w["val"], counted as RISE/FALL/CROSS among the crossings inside
    TD/FROM/TO, with f (the FIND variable) interpolated at that time
    (FindWhenBase::updateTran, WhenAT::isWHENcondition /
    interpolateCalculationInstant / withinRFCWindowForWhen,
    N_IO_MeasureFindWhen.C:108-175,420-480, N_IO_MeasureWhenAT.C:107-250)."""
    val, (kind, count) = w["val"], w["rfc"]
    td, frm, to = w["td"], w["frm"], w["to"]
    nr = nf = nc = 0
    res_t = res_f = res_d = float("nan")
    for k in range(1, len(t)):
        lv, cv = v[k - 1], v[k]
        if cv == lv:
            continue
        if not (abs(cv - val) < MINVAL or (lv - val < 0.0 < cv - val) or (lv - val > 0.0 > cv - val)):
            continue
        a = (cv - lv) / (t[k] - t[k - 1])
        tw = (val - (cv - a * t[k])) / a
        if (tw < td * (1 - MINVAL) or (frm is not None and tw < frm * (1 - MINVAL)) or
                (to is not None and tw > to * (1 + MINVAL))):
            continue
        nc += 1
        rising = cv > lv
        nr += rising
        nf += not rising
        ok = ((kind == "RISE" and rising and nr >= count) or (kind == "FALL" and not rising and nf >= count) or
              (kind not in ("RISE", "FALL") and nc >= count))
        if not ok:
            continue
        res_t = tw
        if f is not None:
            res_f = f[k] if abs(cv - val) < MINVAL else f[k] - (t[k] - tw) * (f[k] - f[k - 1]) / (t[k] - t[k - 1])
            # DERIV: the backward difference over the step that met the
            # condition (DerivativeEvaluationBase::getDerivativeValue,
            # N_IO_MeasureDerivativeEvaluation.C)
            res_d = (f[k] - f[k - 1]) / (t[k] - t[k - 1])
        if count >= 0:
            break
    return res_t, res_f, res_d


def _tran_stats(func, t, v, on, off, frm, to) -> float:
    """FREQ: half the number of OFF->ON and ON->OFF transitions per unit of
    time; DUTY: the fraction of the time spent ON (above ON, or above OFF
    once on); ON_TIME / OFF_TIME: the time at or above ON (at or below OFF)
    per entry into that state; over the points inside FROM/TO, the first of
    which only sets the state (TranStats::updateTran, Frequency / Duty /
    OnTime / OffTime::updateMeasureVars,
    src/IOInterfacePKG/Output/N_IO_MeasureTranStats.C:90-117,
    N_IO_MeasureFrequency.C:80-127, N_IO_MeasureDuty.C:80-118,
    N_IO_MeasureOnTime.C:80-105, N_IO_MeasureOffTime.C:80-105)."""
    sel = np.ones(len(t), bool)
    if frm is not None:
        sel &= t >= frm * (1 - MINVAL)
    if to is not None:
        sel &= t <= to * (1 + MINVAL)
    t, v = t[sel], v[sel]
    window = on_time = 0.0
    ups = downs = cycles = 0
    in_on = False
    for k in range(1, len(t)):
        dt, x, last = t[k] - t[k - 1], v[k], v[k - 1]
        window += dt
        if func == "FREQ":
            ups += (x + MINVAL > on) and (last < on)
            downs += (x - MINVAL < off) and (last > off)
        elif func == "ON_TIME":
            if x + MINVAL >= on:
                on_time += dt
                cycles += last < on
        elif func == "OFF_TIME":
            if x - MINVAL <= off:
                on_time += dt
                cycles += last > off
        elif (x + MINVAL > on) or (in_on and x + MINVAL > off):
            on_time += dt
            in_on = True
        else:
            in_on = False
    if not window > 0:
        return float("nan")
    if func in ("ON_TIME", "OFF_TIME"):
        return float(on_time / cycles if cycles > 0 else on_time)
    return float(0.5 * (ups + downs) / window if func == "FREQ" else on_time / window)


def evaluate_measure(m: Measure, t: np.ndarray, cols: dict) -> float:
    """One .MEASURE from the columns of its variables at the accepted points;
    NaN when it fails (written FAILED)."""
    if m.func == "TRIGTARG":
        tr, tg = m.spec["trig"], m.spec["targ"]
        t1 = _rfc_event_time(t, cols[tr["var"]], tr["val"], tr["rfc"], tr["td"])
        t2 = _rfc_event_time(t, cols[tg["var"]], tg["val"], tg["rfc"], tg["td"])
        return float(t2 - t1)
    if m.func in ("FREQ", "DUTY", "ON_TIME", "OFF_TIME"):
        return _tran_stats(m.func, t, cols[m.var], m.spec["on"], m.spec["off"], m.frm, m.to)
    if m.func == "WHEN":
        return float(_when(t, cols[m.var], None, m.spec["when"])[0])
    if m.func == "DERIV":
        f = cols[m.var]
        if "at" in m.spec:
            at = m.spec["at"]
            for k in range(1, len(t)):
                b, c = t[k - 1] - at, t[k] - at
                if (b < 0.0 < c) or abs(b) < MINVAL or abs(c) < MINVAL:
                    return float((f[k] - f[k - 1]) / (t[k] - t[k - 1]))
            return float("nan")
        w = m.spec["when"]
        return float(_when(t, cols[w["var"]], f, w)[2])
    if m.func == "FIND":
        if "at" in m.spec:
            at = m.spec["at"]
            if len(t) == 0 or at < t[0] or at > t[-1]:
                return float("nan")
            return float(np.interp(at, t, cols[m.var]))
        w = m.spec["when"]
        return float(_when(t, cols[w["var"]], cols[m.var], w)[1])
    return measure(m.func, t, cols[m.var], m.frm, m.to)


def measure(func: str, t: np.ndarray, v: np.ndarray, frm=None, to=None) -> float:
    """One .MEASURE over the accepted points inside [frm, to]."""
    sel = np.ones(len(t), bool)
    if frm is not None:
        sel &= t >= frm
    if to is not None:
        sel &= t <= to
    t, v = t[sel], v[sel]
    if len(t) == 0:
        return float("nan")
    if func == "MAX":
        return float(v.max())
    if func == "MIN":
        return float(v.min())
    if func == "PP":
        return float(v.max() - v.min())
    if len(t) < 2:
        return float("nan")
    dt = np.diff(t)
    if func == "INTEG":
        return float(np.sum(0.5 * dt * (v[1:] + v[:-1])))
    if func == "AVG":
        return float(np.sum(0.5 * dt * (v[1:] + v[:-1])) / (t[-1] - t[0]))
    # RMS: square root of the trapezoid integral of v^2 over the window
    return float(math.sqrt(np.sum(0.5 * dt * (v[1:] ** 2 + v[:-1] ** 2)) / (t[-1] - t[0])))


def run(deck: Deck, device: int = 0, cap: int | None = None) -> Result:
    """Transient of the deck on the GPU; columns of every .PRINT and
    .MEASURE variable at the accepted time points."""
    from . import Circuit
    nl = deck.netlist
    wanted = list(dict.fromkeys(deck.prints + [v for m in deck.measures for v in m.vars]))
    plan = {}
    probes: list[int] = []
    for var in wanted:
        us, f = _var_probes(deck, var)
        slots = []
        for u in us:
            if u not in probes:
                probes.append(u)
            slots.append(probes.index(u))
        plan[var] = (us, slots, f)
    if cap is None:
        tr = nl.tran
        hmin_guess = tr.hmax if tr.hmax > 0 else tr.tstop / 50.0
        cap = int(min(2_000_000, max(4096, 20 * tr.tstop / max(hmin_guess, 1e-30))))
    for _ in range(4):
        circ = Circuit(nl, device=device)
        try:
            counts, times, values, stats = circ.transient(nl.tran, probes=probes or [0], cap=cap)
        finally:
            circ.close()
        n = int(counts[0])
        if n < cap:
            break
        cap *= 4  # the waveform buffer filled up: run again with a larger one
    else:
        raise RuntimeError(f"more than {cap} accepted steps")
    return _columns(deck, wanted, plan, times[0, :n].copy(), values[0, :n, :], stats)


def write_prn(path: str, deck: Deck, res) -> None:
    """The reference's .prn table: Index, TIME, then the .PRINT columns.
    res: one Result, or a list of them for a .STEP sweep — then the steps
    follow one another under one header, the Index restarting at 0 for each
    step, and the footer reads "End of Xyce(TM) Parameter Sweep"
    (TimePrn::doStartStep / doSteppingComplete,
    src/IOInterfacePKG/N_IO_OutputterTimePrn.C:165-230).  FORMAT=NOINDEX
    drops the Index column (printIndexColumn_, N_IO_OutputMgr.C:1655)."""
    results = res if isinstance(res, list) else [res]
    names = ["TIME"] + [p for p in deck.prints if p != "TIME"]
    index = deck.print_format != "NOINDEX"

    def head(name, width=17):
        if width <= len(name):
            return name
        left = (width - len(name)) // 2
        return " " * left + name + " " * (width - left - len(name))
    with open(path, "w") as f:
        f.write(" ".join((["Index"] if index else []) + [head(n) for n in names]) + "\n")
        for r in results:
            cols = [r.times] + [r.columns[p] for p in names[1:]]
            for i in range(len(r.times)):
                row = ([f"{i:<5d}"] if index else []) + [f"{c[i]:>17.9e}" for c in cols]
                f.write(" ".join(row) + "\n")
        f.write("End of Xyce(TM) Parameter Sweep\n" if isinstance(res, list) and len(results) > 1
                else "End of Xyce(TM) Simulation\n")


def write_csv(path: str, deck: Deck, res) -> None:
    """FORMAT=CSV: TIME and the .PRINT columns, comma-delimited, names and
    values unpadded, 9 digits after the point, no Index column and no footer
    (TimeCSV, src/IOInterfacePKG/N_IO_OutputterTimeCSV.C:100-170; columns
    and delimiter N_IO_OutputterLocal.C:201-215, 402-425, 452-470).  A sweep's
    steps follow one another under the one header."""
    results = res if isinstance(res, list) else [res]
    names = ["TIME"] + [p for p in deck.prints if p != "TIME"]
    with open(path, "w") as f:
        f.write(",".join(names) + "\n")
        for r in results:
            cols = [r.times] + [r.columns[p] for p in names[1:]]
            for i in range(len(r.times)):
                f.write(",".join(f"{c[i]:.9e}" for c in cols) + "\n")


def write_print(path: str, deck: Deck, res) -> str:
    """The .PRINT TRAN output in the deck's format; returns the file written
    (path + ".csv" for FORMAT=CSV, else path + ".prn")."""
    if deck.print_format == "CSV":
        write_csv(path + ".csv", deck, res)
        return path + ".csv"
    write_prn(path + ".prn", deck, res)
    return path + ".prn"


def read_prn(path: str) -> tuple[list[str], np.ndarray]:
    """Column names and values of a .prn table (Index column included)."""
    with open(path) as f:
        lines = f.read().splitlines()
    names = lines[0].split()
    rows = [list(map(float, ln.split())) for ln in lines[1:] if ln and not ln.startswith("End of")]
    return names, np.array(rows).reshape(-1, len(names))


def write_mt0(path: str, deck: Deck, res: Result) -> None:
    with open(path, "w") as f:
        for m in deck.measures:
            v = res.measures[m.name]
            f.write(f"{m.name} = FAILED\n" if not np.isfinite(v) else f"{m.name} = {v:.6e}\n")


def main(argv=None) -> int:
    """``python -m xyce_gb300.spice netlist.cir`` — run the transient on the
    GPU and write ``netlist.cir.prn`` (``.csv`` for FORMAT=CSV; and
    ``netlist.cir.mt0`` with .MEASURE)."""
    argv = sys.argv[1:] if argv is None else argv
    if len(argv) != 1:
        print("usage: python -m xyce_gb300.spice <netlist>", file=sys.stderr)
        return 2
    path = argv[0]
    with open(path) as f:
        text = f.read()
    where = os.path.dirname(os.path.abspath(path))
    base = parse(text, base_dir=where)
    if base.embedded:
        decks = parse_embedded(text, where)
        ens = run_embedded(decks)
        out = write_ensemble(path, decks[0], ens)
        print(f"{len(decks)} samples as one block system, {len(ens.times)} shared time points; "
              f"output {os.path.basename(out)}")
        return 0
    if base.sampling:
        if base.steps:
            raise ValueError(".SAMPLING and .STEP together are not supported")
        decks = parse_sampling(text, where)
        results = run_sweep(decks)
        out = write_print(path, base, results) if base.prints else path + ".ms0"
        with open(path + ".ms0", "w") as f:
            for m in base.measures:
                st = sample_moments([r.measures[m.name] for r in results])
                line = f"{m.name}: " + ", ".join(f"{k} = {v:.6e}" for k, v in st.items())
                f.write(line + "\n")
                print(line)
        print(f"{len(decks)} samples run as one batch; output {os.path.basename(out)}")
        return 0
    decks = parse_sweep(text, where)
    deck = decks[0]
    if len(decks) == 1:
        res = run(deck)
        out = write_print(path, deck, res) if deck.prints else path + ".mt0"
        if deck.measures:
            write_mt0(path + ".mt0", deck, res)
            for m in deck.measures:
                print(f"{m.name} = {res.measures[m.name]:.6e}")
        print(f"{len(res.times)} accepted time points, {res.stats.get('rejected', 0)} rejected; "
              f"output {os.path.basename(out)}")
        return 0
    results = run_sweep(decks)
    out = write_print(path, deck, results) if deck.prints else path + ".mt0"
    if deck.measures:  # one measure file per step: .mt0, .mt1, ...
        for k, (d, r) in enumerate(zip(decks, results)):
            write_mt0(path + f".mt{k}", d, r)
    print(f"{len(decks)} sweep points run as one batch; output {os.path.basename(out)}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
