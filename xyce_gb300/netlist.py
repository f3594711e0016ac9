"""Circuit descriptions and seeded synthetic generators.

A :class:`Netlist` is the flat, array-of-devices description that the C-ABI
(``include/xyce_gb300.h``) uploads: unknown indices are 0-based MNA
unknowns, ground is ``-1``.  Several independent circuits may be packed
into one netlist (the batched Monte-Carlo form); ``offsets`` gives the
contiguous unknown range of each circuit.

Device parameter rows follow the layouts declared in the C header
(``XG_DIODE_*`` and ``XG_MOS1_*``), which mirror the instance/model
parameters of Xyce's Diode (src/DeviceModelPKG/OpenModels/N_DEV_Diode.C:100-345)
and MOSFET level 1 (src/DeviceModelPKG/OpenModels/N_DEV_MOSFET1.C:61-331).

The generators build the synthetic workloads with numpy ``default_rng``
seeds: the diode-RC ladder, CMOS ring oscillators, the power-grid mesh and
the batch of uneven Monte-Carlo rings.  No public benchmark netlists are
involved.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

WAVE_DC, WAVE_SIN, WAVE_PULSE, WAVE_PWL = 0, 1, 2, 3

# Diode parameter row (N_DEV_Diode.C addPar defaults).
DIODE_FIELDS = ["IS", "N", "RS", "CJO", "VJ", "M", "FC", "TT", "BV", "IBV", "NBV",
                "IKF", "ISR", "NR", "EG", "XTI", "AREA", "BVGIVEN",
                "JSW", "NS", "NSGIVEN", "CJSW", "VJSW", "MJSW", "FCS", "PJ",
                "TNOM", "TEMP", "TIKF", "TBV1", "TBV2", "TRS1", "TRS2"]
DIODE_DEFAULTS = dict(IS=1e-14, N=1.0, RS=0.0, CJO=0.0, VJ=1.0, M=0.5, FC=0.5, TT=0.0,
                      BV=1e99, IBV=1e-3, NBV=None, IKF=0.0, ISR=0.0, NR=2.0, EG=1.11,
                      XTI=3.0, AREA=1.0, BVGIVEN=0.0,
                      JSW=0.0, NS=1.0, NSGIVEN=0.0, CJSW=0.0, VJSW=1.0, MJSW=0.33, FCS=0.5, PJ=0.0,
                      TNOM=300.15, TEMP=300.15, TIKF=0.0, TBV1=0.0, TBV2=0.0, TRS1=0.0, TRS2=0.0)
# TNOM and TEMP in the rows are kelvin (the netlist's degrees Celsius + 273.15,
# as the reference's parameter layer converts them); 300.15 K = 27 C, the
# reference's default for both.
CTOK = 273.15

# MOSFET level-1 parameter row (model + instance; N_DEV_MOSFET1.C addPar defaults).
MOS1_FIELDS = ["TYPE", "VTO", "KP", "GAMMA", "PHI", "LAMBDA", "RD", "RS", "CBD", "CBS",
               "IS", "PB", "CGSO", "CGDO", "CGBO", "CJ", "MJ", "CJSW", "MJSW", "JS",
               "TOX", "LD", "FC", "W", "L", "AD", "AS", "PD", "PS", "M", "RSH", "NRD", "NRS",
               "TNOM", "TEMP"]
MOS1_DEFAULTS = dict(TYPE=1.0, VTO=0.0, KP=2e-5, GAMMA=0.0, PHI=0.6, LAMBDA=0.0, RD=0.0,
                     RS=0.0, CBD=0.0, CBS=0.0, IS=1e-14, PB=0.8, CGSO=0.0, CGDO=0.0,
                     CGBO=0.0, CJ=0.0, MJ=0.5, CJSW=0.0, MJSW=0.5, JS=0.0, TOX=0.0, LD=0.0,
                     FC=0.5, W=1e-4, L=1e-4, AD=0.0, AS=0.0, PD=0.0, PS=0.0, M=1.0, RSH=0.0,
                     NRD=1.0, NRS=1.0, TNOM=300.15, TEMP=300.15)


def at_temperature(nl: "Netlist", temp_c: float, tnom_c: float = 27.0, **diode_coeffs) -> "Netlist":
    """Every diode and level-1 MOSFET of nl at temp_c with model TNOM tnom_c
    (degrees C; the rows hold kelvin); diode_coeffs (TIKF, TBV1, TBV2, TRS1,
    TRS2) are set on every diode."""
    fd, fm = DIODE_FIELDS.index, MOS1_FIELDS.index
    for k, (a, b, p, row) in enumerate(nl.diode):
        row = np.array(row, dtype=np.float64)
        row[fd("TEMP")], row[fd("TNOM")] = temp_c + CTOK, tnom_c + CTOK
        for name, v in diode_coeffs.items():
            row[fd(name)] = v
        nl.diode[k] = (a, b, p, row)
    for k, m in enumerate(nl.mos1):
        row = np.array(m[4], dtype=np.float64)
        row[fm("TEMP")], row[fm("TNOM")] = temp_c + CTOK, tnom_c + CTOK
        nl.mos1[k] = m[:4] + (row,) + m[5:]
    return nl


def mos1_series(row) -> tuple:
    """(drain, source) series conductances of a MOSFET-1 row
    (Instance::processParams, N_DEV_MOSFET1.C:410-450): 1/RD when RD is
    nonzero, else 1/(RSH*NRD) when RSH is nonzero, else 0 (no internal node)."""
    f = MOS1_FIELDS.index

    def g(r, sq):
        if row[f(r)] != 0.0:
            return 1.0 / row[f(r)]
        return 1.0 / (row[f("RSH")] * row[f(sq)]) if row[f("RSH")] != 0.0 else 0.0
    return g("RD", "NRD"), g("RS", "NRS")


# BSIM4 (level 54) parameter row: instance + model parameters in the order of
# XG_B4_* (include/xyce_gb300.h).  NaN = not given: the model derives it as the
# reference does (Model::processParams4p82_, N_DEV_MOSFET_B4p82.C:7769-8136).
B4_FIELDS = (
    "TYPE L W AS AD PS PD M TOXE TOXP TOXM DTOX EPSROX VTH0 VFB K1 K2 K3 K3B W0 "
    "LPE0 LPEB DVT0 DVT1 DVT2 DVT0W DVT1W DVT2W DSUB DROUT NDEP NSUB NSD NGATE PHIN XJ XT "
    "VBM VBX GAMMA1 GAMMA2 CDSC CDSCB CDSCD CIT NFACTOR ETA0 ETAB VOFF VOFFL MINV DVTP0 DVTP1 "
    "U0 UA UB UC UD UP LP VSAT A0 AGS A1 A2 B0 B1 KETA DWG DWB RDSW RDSWMIN PRWG PRWB WR PCLM "
    "PDIBLC1 PDIBLC2 PDIBLCB PVAG DELTA FPROUT PDITS PDITSD PDITSL PSCBE1 PSCBE2 ALPHA0 "
    "ALPHA1 BETA0 AGIDL BGIDL CGIDL EGIDL AGISL BGISL CGISL EGISL CGSO CGDO CGBO CGSL CGDL "
    "CKAPPAS CKAPPAD CF CLC CLE DLC DWC DWJ LINT WINT XL XW NOFF VOFFCV ACDE MOIN ADOS BDOS "
    "XPART MINVCV VOFFCVL CJS CJD CJSWS CJSWD CJSWGS CJSWGD MJS MJD MJSWS MJSWD MJSWGS MJSWGD "
    "PBS PBD PBSWS PBSWD PBSWGS PBSWGD JSS JSD JSWS JSWD JSWGS JSWGD NJS NJD IJTHSFWD IJTHDFWD "
    "DMCG DMCI DMDG DMCGT").split()


def b4_row(**kw) -> np.ndarray:
    """BSIM4 row: every parameter not named is 'not given' (NaN)."""
    row = np.full(len(B4_FIELDS), np.nan)
    row[B4_FIELDS.index("M")] = 1.0
    for k, v in kw.items():
        row[B4_FIELDS.index(k)] = float(v)
    return row


def diode_row(**kw) -> np.ndarray:
    p = dict(DIODE_DEFAULTS)
    p.update(kw)
    if p["NBV"] is None:
        p["NBV"] = p["N"]
    if "BV" in kw:
        p["BVGIVEN"] = 1.0
    if "NS" in kw:
        p["NSGIVEN"] = 1.0
    return np.array([p[f] for f in DIODE_FIELDS], dtype=np.float64)


def mos1_row(**kw) -> np.ndarray:
    p = dict(MOS1_DEFAULTS)
    p.update(kw)
    return np.array([p[f] for f in MOS1_FIELDS], dtype=np.float64)


@dataclass
class Tran:
    """Transient options: .TRAN and .OPTIONS TIMEINT / NONLIN-TRAN values.

    Defaults follow TIAParams (src/TimeIntegrationPKG/N_TIA_TIAParams.C:95-115)
    and the NONLIN-TRAN table (src/NonlinearSolverPKG/N_NLS_Manager.C:1056-1066).
    """
    tstop: float
    hmax: float = 0.0
    tstart: float = 0.0
    hmin: float = 0.0
    reltol: float = 1e-3
    abstol: float = 1e-6
    nl_reltol: float = 1e-2
    nl_abstol: float = 1e-6
    nl_deltaxtol: float = 0.33
    nl_rhstol: float = 1e-2
    nl_smallupdatetol: float = 1e-6
    nl_maxstep: int = 20
    max_order: int = 2
    max_steps: int = 0
    method: int = 7  # 7 = OneStep (trapezoid), 8 = Gear12 (BDF2): TIMEINT METHOD


@dataclass
class Netlist:
    n: int = 0
    offsets: list = field(default_factory=lambda: [0])
    res: list = field(default_factory=list)      # (p, n, R)
    cap: list = field(default_factory=list)      # (p, n, C)
    vsrc: list = field(default_factory=list)     # (p, n, branch, kind, data)
    isrc: list = field(default_factory=list)     # (p, n, kind, data)
    ind: list = field(default_factory=list)      # (p, n, branch, L)
    diode: list = field(default_factory=list)    # (p, n, pri, row)
    mos1: list = field(default_factory=list)     # (d, g, s, b, row, d', s')
    bsim4: list = field(default_factory=list)    # (d, g, s, b, row)
    names: dict = field(default_factory=dict)
    tran: Tran | None = None
    label: str = ""

    # ---- construction ---------------------------------------------------
    def node(self, name: str | None = None) -> int:
        i = self.n
        self.n += 1
        if name is not None:
            self.names[name] = i
        return i

    def end_circuit(self):
        """Close the current circuit: unknowns allocated so far belong to it."""
        if self.offsets[-1] != self.n:
            self.offsets.append(self.n)

    def R(self, a, b, r):
        self.res.append((a, b, float(r)))

    def C(self, a, b, c):
        self.cap.append((a, b, float(c)))

    def V(self, a, b, kind, data, name=None):
        br = self.node(name)
        self.vsrc.append((a, b, br, kind, [float(x) for x in data]))
        return br

    def L(self, a, b, value, name=None):
        """Inductor (henry); its branch current is a new unknown, returned."""
        br = self.node(name)
        self.ind.append((a, b, br, float(value)))
        return br

    def I(self, a, b, kind, data):
        self.isrc.append((a, b, kind, [float(x) for x in data]))

    def D(self, a, b, **params):
        row = diode_row(**params)
        pri = a
        if row[DIODE_FIELDS.index("RS")] != 0.0:
            pri = self.node()
        self.diode.append((a, b, pri, row))

    def M1(self, d, g, s, b, **params):
        """MOSFET level 1; drain' / source' internal nodes are made when the
        series resistance (RD / RS, or RSH with NRD / NRS) is nonzero.
        Stored as (d, g, s, b, row, d', s')."""
        row = mos1_row(**params)
        gd, gs = mos1_series(row)
        dp = self.node() if gd != 0.0 else d
        sp = self.node() if gs != 0.0 else s
        self.mos1.append((d, g, s, b, row, dp, sp))

    def M4(self, d, g, s, b, **params):
        """BSIM4 (level 54) instance; parameters not named are not given."""
        self.bsim4.append((d, g, s, b, b4_row(**params)))

    # ---- flat arrays (C-ABI order) ------------------------------------
    def arrays(self) -> dict:
        self.end_circuit()
        i32 = lambda x: np.ascontiguousarray(np.asarray(x, dtype=np.int32))
        f64 = lambda x: np.ascontiguousarray(np.asarray(x, dtype=np.float64))

        def waves(lst, k_kind, k_data):
            kinds = [w[k_kind] for w in lst]
            off = [0]
            data = []
            for w in lst:
                data.extend(w[k_data])
                off.append(len(data))
            return i32(kinds), i32(off), f64(data if data else [0.0])

        out = dict(n=self.n, offsets=i32(self.offsets))
        out["res"] = (i32([r[0] for r in self.res]), i32([r[1] for r in self.res]),
                      f64([r[2] for r in self.res]))
        out["cap"] = (i32([c[0] for c in self.cap]), i32([c[1] for c in self.cap]),
                      f64([c[2] for c in self.cap]))
        vk, vo, vd = waves(self.vsrc, 3, 4)
        out["vsrc"] = (i32([v[0] for v in self.vsrc]), i32([v[1] for v in self.vsrc]),
                       i32([v[2] for v in self.vsrc]), vk, vo, vd)
        ik, io, idat = waves(self.isrc, 2, 3)
        out["isrc"] = (i32([v[0] for v in self.isrc]), i32([v[1] for v in self.isrc]), ik, io, idat)
        out["ind"] = (i32([v[0] for v in self.ind]), i32([v[1] for v in self.ind]), i32([v[2] for v in self.ind]),
                      f64([v[3] for v in self.ind]))
        out["diode"] = (i32([d[0] for d in self.diode]), i32([d[1] for d in self.diode]),
                        i32([d[2] for d in self.diode]),
                        f64(np.array([d[3] for d in self.diode]).reshape(-1, len(DIODE_FIELDS))))
        out["mos1"] = (i32([m[0] for m in self.mos1]), i32([m[1] for m in self.mos1]),
                       i32([m[2] for m in self.mos1]), i32([m[3] for m in self.mos1]),
                       i32([m[5] for m in self.mos1]), i32([m[6] for m in self.mos1]),
                       f64(np.array([m[4] for m in self.mos1]).reshape(-1, len(MOS1_FIELDS))))
        out["bsim4"] = (i32([m[0] for m in self.bsim4]), i32([m[1] for m in self.bsim4]),
                        i32([m[2] for m in self.bsim4]), i32([m[3] for m in self.bsim4]),
                        f64(np.array([m[4] for m in self.bsim4]).reshape(-1, len(B4_FIELDS))))
        return out

    @property
    def n_circuits(self) -> int:
        self.end_circuit()
        return len(self.offsets) - 1

    def circuit_of(self, u: int) -> int:
        """Index of the circuit that owns unknown u."""
        self.end_circuit()
        return int(np.searchsorted(self.offsets, u, side="right") - 1)

    def device_count(self) -> int:
        return len(self.res) + len(self.cap) + len(self.vsrc) + len(self.isrc) + len(self.ind) + \
            len(self.diode) + len(self.mos1) + len(self.bsim4)


# ---------------------------------------------------------------------------
# Small known-answer circuits.

def test_netlist1() -> Netlist:
    """V1 1 0 5; R1 1 0 1; .TRAN 0 1 — V(1) = 5 exactly."""
    nl = Netlist(label="testnetlist1")
    n1 = nl.node("1")
    nl.V(n1, -1, WAVE_DC, [5.0], name="V1#branch")
    nl.R(n1, -1, 1.0)
    nl.tran = Tran(tstop=1.0)
    return nl


def test_netlist2() -> Netlist:
    """V1 1 0 SIN(0 1 1); R1 1 2 50; R2 2 0 100; C1 1 0 1e-6; .TRAN 0 1.

    V(1) = sin(2 pi t) and V(2) = V(1) * 100/150 exactly.
    """
    nl = Netlist(label="testnetlist2")
    n1, n2 = nl.node("1"), nl.node("2")
    nl.V(n1, -1, WAVE_SIN, [0.0, 1.0, 1.0, 0.0, 0.0, 0.0], name="V1#branch")
    nl.R(n1, n2, 50.0)
    nl.R(n2, -1, 100.0)
    nl.C(n1, -1, 1e-6)
    nl.tran = Tran(tstop=1.0)
    return nl


def rc_step(r=1e3, c=1e-9, v=1.0, tstop=5e-6) -> Netlist:
    """PULSE-driven RC low-pass: V(out) = v (1 - exp(-t/RC)) after the edge."""
    nl = Netlist(label="rc_step")
    a, o = nl.node("in"), nl.node("out")
    nl.V(a, -1, WAVE_PULSE, [0.0, v, 0.0, 1e-12, 1e-12, 1.0, 0.0])
    nl.R(a, o, r)
    nl.C(o, -1, c)
    nl.tran = Tran(tstop=tstop, hmax=tstop / 200)
    return nl


# ---------------------------------------------------------------------------
# Synthetic workloads.

# Diode cards with sidewall junctions (JSW / NS / CJSW / VJSW / MJSW / FCS,
# perimeter PJ): own sidewall characteristic, sidewall current merged into
# the bottom one (NS not given), and sidewall charge beside a bottom one.
SIDEWALL_DIODES = (
    dict(IS=1e-14, N=1.0, RS=10.0, CJO=0.2e-12, JSW=2e-15, NS=1.3, CJSW=0.05e-12, VJSW=0.8, MJSW=0.4,
         FCS=0.6, PJ=3.0, BV=4.0),
    dict(IS=1e-14, N=1.0, RS=10.0, CJO=0.1e-12, JSW=5e-15, CJSW=0.03e-12, PJ=2.0),
    dict(IS=2e-14, N=1.1, RS=0.0, CJO=0.3e-12, TT=1e-10, CJSW=0.1e-12, MJSW=0.25, PJ=1.5),
)


def diode_ladder(n_nodes=1000, seed=1, sidewall=False) -> Netlist:
    """Diode-RC ladder: chain of n_nodes, R_i ~ U[500,2000] ohm, C_i ~ U[0.1,1] pF,
    a level-1 diode (IS=1e-14, N=1, RS=10) from every node to ground, node 1
    driven by SIN(1 1 1MEG); .TRAN 0 5u, max step 10 n, RELTOL 1e-3 ABSTOL 1e-12.
    sidewall: the diodes cycle through SIDEWALL_DIODES instead, and the
    source swings between -5.5 V and 3.5 V so the reverse and breakdown
    (BV = 4 V) regimes are reached."""
    rng = np.random.default_rng(seed)
    nl = Netlist(label=f"diode_ladder_{n_nodes}")
    nodes = [nl.node(f"n{i + 1}") for i in range(n_nodes)]
    rv = rng.uniform(500.0, 2000.0, n_nodes - 1)
    cv = rng.uniform(0.1e-12, 1e-12, n_nodes)
    amp = [-1.0, 4.5] if sidewall else [1.0, 1.0]
    nl.V(nodes[0], -1, WAVE_SIN, [amp[0], amp[1], 1e6, 0.0, 0.0, 0.0], name="V1#branch")
    for i in range(n_nodes - 1):
        nl.R(nodes[i], nodes[i + 1], rv[i])
    for i in range(n_nodes):
        nl.C(nodes[i], -1, cv[i])
        if sidewall:
            nl.D(nodes[i], -1, **SIDEWALL_DIODES[i % len(SIDEWALL_DIODES)])
        else:
            nl.D(nodes[i], -1, IS=1e-14, N=1.0, RS=10.0)
    nl.tran = Tran(tstop=5e-6, hmax=10e-9, reltol=1e-3, abstol=1e-12)
    return nl


NMOS_CARD = dict(TYPE=1.0, VTO=0.5, KP=120e-6, W=2e-6, L=0.18e-6)
PMOS_CARD = dict(TYPE=-1.0, VTO=-0.5, KP=40e-6, W=4e-6, L=0.18e-6)


def _ring(nl: Netlist, stages: int, vdd=1.8, cload=5e-15, nmos=None, pmos=None,
          kick=100e-6, prefix="") -> None:
    nmos = nmos or NMOS_CARD
    pmos = pmos or PMOS_CARD
    outs = [nl.node(f"{prefix}n{i + 1}") for i in range(stages)]
    vdd_n = nl.node(f"{prefix}vdd")
    nl.V(vdd_n, -1, WAVE_DC, [vdd], name=f"{prefix}VDD#branch")
    for i in range(stages):
        inp = outs[i - 1]
        out = outs[i]
        cl = cload[i] if hasattr(cload, "__len__") else cload
        nc = nmos[i] if isinstance(nmos, list) else nmos
        pc = pmos[i] if isinstance(pmos, list) else pmos
        nl.M1(out, inp, -1, -1, **nc)
        nl.M1(out, inp, vdd_n, vdd_n, **pc)
        nl.C(out, -1, cl)
    # 1 ns current kick into the first node (PWL source from ground to n1)
    nl.I(-1, outs[0], WAVE_PWL, [0.0, 0.0, 10e-12, kick, 990e-12, kick, 1e-9, 0.0])


def ring_oscillator(stages=101, caps=False, series=False) -> Netlist:
    """CMOS ring oscillator of MOSFET level-1 inverters: VDD=1.8 V, NMOS VTO=0.5
    KP=120u, PMOS VTO=-0.5 KP=40u, W/L=2u/0.18u (PMOS W=4u), 5 fF per stage, a
    1 ns PWL kick on node 1; .TRAN 0 20n, max step 5 p.

    caps=True adds gate oxide (TOX), overlap and bulk-junction capacitances so
    that the Meyer and junction-charge paths of the model are exercised.

    series=True adds series resistances: RD = 400, RS = 250 ohm on the NMOS;
    RSH = 50 ohm with NRD = 2, NRS = 1.5 squares on the PMOS, which are also
    two in parallel (M = 2)."""
    assert stages % 2 == 1
    nl = Netlist(label=f"ring_{stages}" + ("_caps" if caps else "") + ("_rs" if series else ""))
    nmos, pmos = dict(NMOS_CARD), dict(PMOS_CARD)
    if caps:
        extra = dict(TOX=4e-9, CGSO=2e-10, CGDO=2e-10, CGBO=1e-10, CJ=1e-3, CJSW=2e-10,
                     MJ=0.45, MJSW=0.33, AD=1e-12, AS=1e-12, PD=4e-6, PS=4e-6, GAMMA=0.4,
                     LAMBDA=0.05, PHI=0.7)
        nmos.update(extra)
        pmos.update(extra)
    if series:
        nmos.update(RD=400.0, RS=250.0)
        pmos.update(RSH=50.0, NRD=2.0, NRS=1.5, M=2.0)
    if caps or series:
        _ring(nl, stages, nmos=nmos, pmos=pmos)
    else:
        _ring(nl, stages)
    nl.tran = Tran(tstop=20e-9, hmax=5e-12)
    return nl


def rlc_ladder(n=20, seed=1) -> Netlist:
    """A driven RLC ladder: node 1 driven by PULSE(0 1 0.1n 0.1n 0.1n 5n 10n)
    through 50 ohm, then n sections of a series inductor L ~ U[1,3] nH into
    a shunt capacitor C ~ U[0.5,2] pF with a 1 kohm shunt; .TRAN 0 20n,
    max step 20 ps."""
    rng = np.random.default_rng(seed)
    nl = Netlist(label=f"rlc_ladder_{n}")
    src, first = nl.node("src"), nl.node("n0")
    nl.V(src, -1, WAVE_PULSE, [0.0, 1.0, 0.1e-9, 0.1e-9, 0.1e-9, 5e-9, 10e-9], name="V1#branch")
    nl.R(src, first, 50.0)
    prev = first
    for i in range(n):
        node = nl.node(f"n{i + 1}")
        nl.L(prev, node, rng.uniform(1e-9, 3e-9), name=f"L{i + 1}#branch")
        nl.C(node, -1, rng.uniform(0.5e-12, 2e-12))
        nl.R(node, -1, 1e3)
        prev = node
    nl.tran = Tran(tstop=20e-9, hmax=20e-12)
    return nl


def power_grid(k=500, n_sinks=2000, seed=3) -> Netlist:
    """k x k resistive mesh, R ~ U[0.05,0.2] ohm, decaps ~ U[1,10] fF, n_sinks
    seed-placed PWL current sinks ramping to U[0,5] mA over 100 ps windows,
    four corner pads tied to 1.0 V through 0.01 ohm; .TRAN 0 2n step 1 p."""
    rng = np.random.default_rng(seed)
    nl = Netlist(label=f"power_grid_{k}")
    base = nl.n
    nl.n += k * k
    idx = lambda r, c: base + r * k + c
    rh = rng.uniform(0.05, 0.2, (k, k - 1))
    rvv = rng.uniform(0.05, 0.2, (k - 1, k))
    for r in range(k):
        for c in range(k - 1):
            nl.R(idx(r, c), idx(r, c + 1), rh[r, c])
    for r in range(k - 1):
        for c in range(k):
            nl.R(idx(r, c), idx(r + 1, c), rvv[r, c])
    cv = rng.uniform(1e-15, 10e-15, k * k)
    for i in range(k * k):
        nl.C(base + i, -1, cv[i])
    for (r, c) in [(0, 0), (0, k - 1), (k - 1, 0), (k - 1, k - 1)]:
        pad = nl.node()
        nl.V(pad, -1, WAVE_DC, [1.0])
        nl.R(pad, idx(r, c), 0.01)
    where = rng.choice(k * k, size=min(n_sinks, k * k), replace=False)
    amp = rng.uniform(0.0, 5e-3, len(where))
    start = rng.uniform(0.0, 1.8e-9, len(where))
    for i, node in enumerate(where):
        t0 = start[i]
        nl.I(base + int(node), -1, WAVE_PWL, [t0, 0.0, t0 + 100e-12, amp[i]])
    nl.names["center"] = idx(k // 2, k // 2)
    nl.tran = Tran(tstop=2e-9, hmax=1e-12)
    return nl


def monte_carlo_rings(count=4096, min_stages=11, max_stages=301, seed=4) -> Netlist:
    """Batch of independent ring oscillators with uneven sizes: odd stage
    counts uniform in [min_stages, max_stages], per-instance VTO ~ N(+-0.5,
    0.03), KP ~ N(nominal, 5%), load C ~ U[3,7] fF; .TRAN 0 10n."""
    rng = np.random.default_rng(seed)
    nl = Netlist(label=f"mc_rings_{count}")
    odd = np.arange(min_stages, max_stages + 1, 2)
    sizes = rng.choice(odd, size=count)
    for ci, st in enumerate(sizes):
        st = int(st)
        nm = [dict(NMOS_CARD, VTO=rng.normal(0.5, 0.03), KP=rng.normal(120e-6, 0.05 * 120e-6))
              for _ in range(st)]
        pm = [dict(PMOS_CARD, VTO=rng.normal(-0.5, 0.03), KP=rng.normal(40e-6, 0.05 * 40e-6))
              for _ in range(st)]
        cl = rng.uniform(3e-15, 7e-15, st)
        _ring(nl, st, cload=cl, nmos=nm, pmos=pm, prefix=f"c{ci}.")
        nl.end_circuit()
    nl.tran = Tran(tstop=10e-9, hmax=5e-12)
    return nl


def batch(nls: list, label: str = "batch") -> Netlist:
    """Independent netlists as the circuits of one batched netlist (unknowns
    renumbered into consecutive ranges; node names prefixed "<k>:"); the
    transient options are the first netlist's."""
    out = Netlist(label=label)
    for k, nl in enumerate(nls):
        nl.end_circuit()
        base = out.n

        def sh(u, base=base):
            return -1 if u < 0 else u + base
        out.n += nl.n
        out.names.update({f"{k}:{name}": i + base for name, i in nl.names.items()})
        out.res += [(sh(a), sh(b), r) for (a, b, r) in nl.res]
        out.cap += [(sh(a), sh(b), c) for (a, b, c) in nl.cap]
        out.vsrc += [(sh(a), sh(b), sh(br), kd, list(d)) for (a, b, br, kd, d) in nl.vsrc]
        out.isrc += [(sh(a), sh(b), kd, list(d)) for (a, b, kd, d) in nl.isrc]
        out.ind += [(sh(a), sh(b), sh(br), lv) for (a, b, br, lv) in nl.ind]
        out.diode += [(sh(a), sh(b), sh(p), row) for (a, b, p, row) in nl.diode]
        out.mos1 += [(sh(d), sh(g), sh(s_), sh(b), row, sh(dp), sh(sp))
                     for (d, g, s_, b, row, dp, sp) in nl.mos1]
        out.bsim4 += [(sh(d), sh(g), sh(s_), sh(b), row) for (d, g, s_, b, row) in nl.bsim4]
        out.offsets += [o + base for o in nl.offsets[1:]]
    out.tran = nls[0].tran if nls else None
    return out


def extract_circuit(nl: Netlist, ci: int) -> Netlist:
    """Circuit ci of a batch as a netlist of its own (unknowns renumbered from
    0, ground kept at -1), with the batch's transient options."""
    nl.end_circuit()
    off0, off1 = nl.offsets[ci], nl.offsets[ci + 1]
    inside = lambda *us: any(off0 <= u < off1 for u in us)
    rm = lambda u: -1 if u < 0 else u - off0
    out = Netlist(label=f"{nl.label}.c{ci}")
    out.n = off1 - off0
    out.names = {k: v - off0 for k, v in nl.names.items() if off0 <= v < off1}
    out.res = [(rm(a), rm(b), r) for (a, b, r) in nl.res if inside(a, b)]
    out.cap = [(rm(a), rm(b), c) for (a, b, c) in nl.cap if inside(a, b)]
    out.vsrc = [(rm(a), rm(b), rm(br), k, d) for (a, b, br, k, d) in nl.vsrc if inside(br)]
    out.isrc = [(rm(a), rm(b), k, d) for (a, b, k, d) in nl.isrc if inside(a, b)]
    out.ind = [(rm(a), rm(b), rm(br), lv) for (a, b, br, lv) in nl.ind if inside(br)]
    out.diode = [(rm(a), rm(b), rm(r), row) for (a, b, r, row) in nl.diode if inside(a, b, r)]
    out.mos1 = [(rm(d), rm(g), rm(s), rm(b), row, rm(dp), rm(sp))
                for (d, g, s, b, row, dp, sp) in nl.mos1 if inside(d, g, s, b)]
    out.bsim4 = [(rm(d), rm(g), rm(s), rm(b), row) for (d, g, s, b, row) in nl.bsim4 if inside(d, g, s, b)]
    out.tran = nl.tran
    return out


# 45 nm-like BSIM4 cards: TOXE 1.8 nm, VTH0 +-0.4 V, L 45 nm; every other
# parameter keeps the BSIM4 default.
B4_NMOS = dict(TYPE=1.0, L=45e-9, W=90e-9, TOXE=1.8e-9, VTH0=0.4)
B4_PMOS = dict(TYPE=-1.0, L=45e-9, W=180e-9, TOXE=1.8e-9, VTH0=-0.4)


def _bit_stream_pwl(bits, period=1e-9, edge=20e-12, vdd=1.0):
    """PWL points of a bit stream: one bit per period, edges of `edge` s."""
    pts = [0.0, vdd * bits[0]]
    for k in range(1, len(bits)):
        if bits[k] != bits[k - 1]:
            t0 = k * period
            pts += [t0, vdd * bits[k - 1], t0 + edge, vdd * bits[k]]
    return pts


def bsim4_inverter_chain(stages=3, vdd=1.0, cload=2e-15) -> Netlist:
    """Small BSIM4 inverter chain driven by a PULSE: the FD-Jacobian and
    parity case of the level-54 path."""
    nl = Netlist(label=f"b4_chain_{stages}")
    vdd_n = nl.node("vdd")
    nl.V(vdd_n, -1, WAVE_DC, [vdd], name="VDD#branch")
    inp = nl.node("in")
    nl.V(inp, -1, WAVE_PULSE, [0.0, vdd, 50e-12, 20e-12, 20e-12, 300e-12, 700e-12], name="VIN#branch")
    prev = inp
    for i in range(stages):
        out = nl.node(f"n{i + 1}")
        nl.M4(out, prev, -1, -1, **B4_NMOS)
        nl.M4(out, prev, vdd_n, vdd_n, **B4_PMOS)
        nl.C(out, -1, cload)
        prev = out
    nl.tran = Tran(tstop=1e-9, hmax=5e-12)
    return nl


def bsim4_logic_dag(n_transistors=50000, n_inputs=64, seed=5, vdd=1.0, wire_c=2e-15,
                    tstop=5e-9) -> Netlist:
    """Random CMOS logic DAG of INV / NAND2 / NOR2 gates with BSIM4 (level 54)
    transistors: each gate draws its inputs from the primary inputs and the
    outputs of earlier gates (seeded fan-in), every gate output carries a
    wire load; the primary inputs are random PWL bit streams at 1 GHz with
    20 ps edges; .TRAN 0 5n."""
    rng = np.random.default_rng(seed)
    nl = Netlist(label=f"b4_dag_{n_transistors}")
    vdd_n = nl.node("vdd")
    nl.V(vdd_n, -1, WAVE_DC, [vdd], name="VDD#branch")
    nbits = int(np.ceil(tstop / 1e-9)) + 1
    sources = []
    for k in range(n_inputs):
        pi = nl.node(f"pi{k}")
        nl.V(pi, -1, WAVE_PWL, _bit_stream_pwl(rng.integers(0, 2, nbits), vdd=vdd))
        sources.append(pi)
    n_t = 0
    g = 0
    while n_t < n_transistors:
        kind = rng.choice(3, p=[0.34, 0.33, 0.33])  # 0 INV, 1 NAND2, 2 NOR2
        # fan-in from a window of recent signals keeps logic depth moderate
        lo = max(0, len(sources) - 64)
        a, b = (sources[int(i)] for i in rng.integers(lo, len(sources), 2))
        out = nl.node(f"g{g}")
        if kind == 0:
            nl.M4(out, a, -1, -1, **B4_NMOS)
            nl.M4(out, a, vdd_n, vdd_n, **B4_PMOS)
            n_t += 2
        elif kind == 1:  # NAND2: series NMOS, parallel PMOS
            mid = nl.node()
            nl.M4(out, a, mid, -1, **B4_NMOS)
            nl.M4(mid, b, -1, -1, **B4_NMOS)
            nl.M4(out, a, vdd_n, vdd_n, **B4_PMOS)
            nl.M4(out, b, vdd_n, vdd_n, **B4_PMOS)
            n_t += 4
        else:  # NOR2: parallel NMOS, series PMOS
            mid = nl.node()
            nl.M4(out, a, -1, -1, **B4_NMOS)
            nl.M4(out, b, -1, -1, **B4_NMOS)
            nl.M4(mid, a, vdd_n, vdd_n, **B4_PMOS)
            nl.M4(out, b, mid, vdd_n, **B4_PMOS)
            n_t += 4
        nl.C(out, -1, wire_c)
        sources.append(out)
        g += 1
    nl.tran = Tran(tstop=tstop, hmax=5e-12)
    return nl
