"""SPICE-subset reader, .prn / .mt0 writers and measures (CPU only)."""
import os

import numpy as np
import pytest

import oracle

from xyce_gb300 import netlist as N
from xyce_gb300 import spice as S

# the reference checkout's test netlists, read only when present
REF_TESTS = os.path.join(oracle.REFERENCE_ROOT, "test", "CircuitPKG")


@pytest.mark.parametrize("tok,val", [
    ("5", 5.0), ("1MEG", 1e6), ("1meg", 1e6), ("1m", 1e-3), ("1M", 1e-3), ("10pF", 10e-12),
    ("2.5u", 2.5e-6), ("1e-3", 1e-3), ("3k", 3e3), ("1F", 1e-15), ("4n", 4e-9), ("2mil", 50.8e-6),
    ("-0.5", -0.5), (".5", 0.5), ("1.8V", 1.8), ("1T", 1e12), ("2G", 2e9),
])
def test_numbers(tok, val):
    assert S.number(tok) == pytest.approx(val, rel=1e-15)


def test_not_a_number():
    with pytest.raises(ValueError):
        S.number("abc")


RC = """RC low-pass driven by a pulse
* comment line
V1 in 0 PULSE(0 1 1n)   ; TR, TF, PW, PER from .TRAN
R1 in out 1k
C1 out 0 1n
.TRAN 10p 5u 0 25n
.OPTIONS TIMEINT RELTOL=1e-4 ABSTOL=1e-9
.PRINT TRAN V(out) V(in,out) I(V1)
.MEASURE TRAN vmax MAX V(out)
.MEASURE TRAN vavg AVG V(out) FROM=1u TO=4u
.END
"""


def test_rc_deck():
    d = S.parse(RC)
    nl = d.netlist
    assert d.title == "RC low-pass driven by a pulse"
    a = nl.arrays()
    assert nl.n == 3  # in, out, V1 branch
    np.testing.assert_array_equal(a["res"][2], [1e3])
    np.testing.assert_array_equal(a["cap"][2], [1e-9])
    kinds, offs, data = a["vsrc"][3], a["vsrc"][4], a["vsrc"][5]
    assert kinds[0] == N.WAVE_PULSE
    # PULSE(V1 V2 TD) + TR = TF = TSTEP, PW = PER = TSTOP
    np.testing.assert_array_equal(data[offs[0]:offs[1]], [0, 1, 1e-9, 10e-12, 10e-12, 5e-6, 5e-6])
    assert nl.tran.tstop == 5e-6 and nl.tran.hmax == 25e-9
    assert nl.tran.reltol == 1e-4 and nl.tran.abstol == 1e-9
    assert d.prints == ["V(OUT)", "V(IN,OUT)", "I(V1)"]
    assert [(m.name, m.func, m.var, m.frm, m.to) for m in d.measures] == [
        ("VMAX", "MAX", "V(OUT)", None, None), ("VAVG", "AVG", "V(OUT)", 1e-6, 4e-6)]
    assert d.branches["V1"] == nl.names["V1#branch"]


def test_sin_defaults_and_continuation():
    d = S.parse("t\nV1 a 0 SIN(0.5 2\n+ )\nR1 a 0 1\n.TRAN 1n 2u\n.END\n")
    a = d.netlist.arrays()
    offs, data = a["vsrc"][4], a["vsrc"][5]
    # FREQ = 1/TSTOP, TD = THETA = PHASE = 0
    np.testing.assert_array_equal(data[offs[0]:offs[1]], [0.5, 2.0, 1 / 2e-6, 0, 0, 0])


INV_RING = """three-stage ring from an inverter subcircuit
.SUBCKT INV in out vdd
MN out in 0 0 nch W=2u L=0.18u
MP out in vdd vdd pch W=4u L=0.18u
C1 out 0 5f
.ENDS
.MODEL nch NMOS (VTO=0.5 KP=120u)
.MODEL pch PMOS (LEVEL=1 VTO=-0.5 KP=40u)
VDD vdd 0 1.8
X1 n1 n2 vdd INV
X2 n2 n3 vdd INV
X3 n3 n1 vdd INV
I1 0 n1 PWL(0 0 10p 100u 990p 100u 1n 0)
.TRAN 1p 2n 0 5p
.PRINT TRAN V(n1)
.END
"""


def test_subcircuit_flattening():
    d = S.parse(INV_RING)
    nl = d.netlist
    assert len(nl.mos1) == 6 and len(nl.cap) == 3
    assert {"N1", "N2", "N3", "VDD"} <= set(nl.names)
    rows = np.array([m[4] for m in nl.mos1])
    t = N.MOS1_FIELDS.index
    np.testing.assert_array_equal(rows[:, t("TYPE")], [1, -1] * 3)
    np.testing.assert_array_equal(rows[:, t("KP")], [120e-6, 40e-6] * 3)
    np.testing.assert_array_equal(rows[:, t("W")], [2e-6, 4e-6] * 3)
    # X1's NMOS: drain n2, gate n1, source/bulk ground
    d0, g0, s0, b0 = nl.mos1[0][:4]
    assert (d0, g0, s0, b0) == (nl.names["N2"], nl.names["N1"], -1, -1)
    # PMOS bulk/source on the shared supply node
    assert nl.mos1[1][2] == nl.names["VDD"] == nl.mos1[1][3]


@pytest.mark.parametrize("bad,msg", [
    ("t\nL1 a 0 1n\nL2 b 0 1n\nK1 L1 L2 0.5\n.TRAN 1n 1u\n.END\n", "not supported"),
    ("t\nM1 d g 0 0 m1\n.MODEL m1 NMOS (LEVEL=3)\n.TRAN 1n 1u\n.END\n", "level 3"),
    ("t\nM1 d g 0 0 m1\n.MODEL m1 NMOS (UO=600)\n.TRAN 1n 1u\n.END\n", "UO"),
    ("t\nR1 a 0 1\n.END\n", ".TRAN"),
    ("t\nR1 a 0 1\n.AC DEC 10 1 1k\n.TRAN 1n 1u\n.END\n", ".AC"),
])
def test_unsupported_input_raises(bad, msg):
    with pytest.raises(ValueError, match=msg):
        S.parse(bad)


def test_measures():
    t = np.array([0.0, 1.0, 2.0, 4.0])
    v = np.array([0.0, 2.0, -1.0, 3.0])
    assert S.measure("MAX", t, v) == 3.0
    assert S.measure("MIN", t, v) == -1.0
    assert S.measure("PP", t, v) == 4.0
    integ = 0.5 * 1 * 2 + 0.5 * 1 * 1 + 0.5 * 2 * 2
    assert S.measure("INTEG", t, v) == pytest.approx(integ)
    assert S.measure("AVG", t, v) == pytest.approx(integ / 4)
    rms = np.sqrt((0.5 * 1 * 4 + 0.5 * 1 * 5 + 0.5 * 2 * 10) / 4)
    assert S.measure("RMS", t, v) == pytest.approx(rms)
    assert S.measure("MAX", t, v, frm=0.5, to=2.5) == 2.0


@pytest.mark.parametrize("fmt", ["CSV", "NOINDEX"])
def test_print_formats(tmp_path, fmt):
    """.PRINT TRAN FORMAT=CSV writes <deck>.csv (comma-delimited, unpadded,
    no Index, no footer); FORMAT=NOINDEX the .prn table without Index."""
    d = S.parse(RC.replace(".PRINT TRAN", f".PRINT TRAN FORMAT={fmt}"))
    assert d.print_format == fmt and d.prints[:1] == ["V(OUT)"]
    t = np.array([0.0, 1e-9])
    cols = {k: np.array([0.5, -1.25e-3]) for k in d.prints}
    res = S.Result(t, cols, {}, {})
    out = S.write_print(str(tmp_path / "rc.cir"), d, res)
    lines = open(out).read().splitlines()
    if fmt == "CSV":
        assert out.endswith("rc.cir.csv")
        assert lines[0] == ",".join(["TIME"] + d.prints)
        assert lines[1].split(",")[:2] == ["0.000000000e+00", "5.000000000e-01"]
        assert lines[2].split(",")[1] == "-1.250000000e-03" and len(lines) == 3
    else:
        assert out.endswith("rc.cir.prn")
        assert lines[0].split() == ["TIME"] + d.prints and lines[-1] == "End of Xyce(TM) Simulation"
        assert lines[1] == "  0.000000000e+00" + " " + "  5.000000000e-01" + " " + \
            " ".join(["  5.000000000e-01"] * (len(d.prints) - 1))
    with pytest.raises(ValueError, match="WIDTH"):
        S.parse(RC.replace(".PRINT TRAN", ".PRINT TRAN WIDTH=12"))


def test_prn_layout_and_round_trip(tmp_path):
    d = S.parse(RC)
    t = np.array([0.0, 1e-9, 2.5e-9])
    res = S.Result(t, {"V(OUT)": np.array([0.0, 0.25, -1e-20]), "V(IN,OUT)": np.array([1.0, 0.75, 0.5]),
                       "I(V1)": np.array([-1e-3, -7.5e-4, -5e-4])},
                   {"VMAX": 0.25, "VAVG": float("nan")}, {})
    p = tmp_path / "rc.cir.prn"
    S.write_prn(str(p), d, res)
    lines = p.read_text().splitlines()
    # header: Index, then 17-wide centred names separated by one space
    assert lines[0] == "Index" + " " + "      TIME       " + " " + "     V(OUT)      " + " " + \
        "    V(IN,OUT)    " + " " + "      I(V1)      "
    assert lines[1] == "0    " + " " + "  0.000000000e+00" + " " + "  0.000000000e+00" + " " + \
        "  1.000000000e+00" + " " + " -1.000000000e-03"
    assert lines[-1] == "End of Xyce(TM) Simulation"
    names, vals = S.read_prn(str(p))
    assert names == ["Index", "TIME", "V(OUT)", "V(IN,OUT)", "I(V1)"]
    np.testing.assert_array_equal(vals[:, 1], t)
    np.testing.assert_array_equal(vals[:, 2], res.columns["V(OUT)"])
    m = tmp_path / "rc.cir.mt0"
    S.write_mt0(str(m), d, res)
    assert m.read_text().splitlines() == ["VMAX = 2.500000e-01", "VAVG = FAILED"]


@pytest.mark.skipif(not os.path.isdir(REF_TESTS), reason="reference test netlists not present")
@pytest.mark.parametrize("fname,maker", [("TestNetlist1.cir", N.test_netlist1),
                                         ("TestNetlist2.cir", N.test_netlist2)])
def test_reference_test_netlists_parse_to_the_known_answer_circuits(fname, maker):
    d = S.read(os.path.join(REF_TESTS, fname))
    got, want = d.netlist.arrays(), maker().arrays()
    assert d.netlist.n == maker().n
    for k in ("res", "cap", "vsrc", "isrc"):
        for g, w in zip(got[k], want[k]):
            np.testing.assert_array_equal(g, w)
    assert d.netlist.tran.tstop == 1.0
    assert [m.name for m in d.measures][:2] == ["MAXV1", "MINV1"]


@pytest.mark.parametrize("opt,method,order", [("METHOD=GEAR", 8, 2), ("METHOD=8 MAXORD=1", 8, 1),
                                              ("METHOD=TRAP", 7, 2), ("", 7, 2)])
def test_timeint_method(opt, method, order):
    d = S.parse(f"t\nR1 a 0 1\nC1 a 0 1n\nI1 0 a PULSE(0 1m 1n)\n.TRAN 1n 1u\n.OPTIONS TIMEINT {opt}\n.END\n"
                if opt else "t\nR1 a 0 1\n.TRAN 1n 1u\n.END\n")
    assert d.netlist.tran.method == method and d.netlist.tran.max_order == order


def test_nonlin_tran_and_linsol_options():
    """.OPTIONS NONLIN-TRAN sets the transient Newton's tolerances (the keys of
    N_NLS_NLParams.C:191-220); .OPTIONS LINSOL accepts the direct solvers."""
    d = S.parse("t\nR1 a 0 1\nC1 a 0 1n\nI1 0 a PULSE(0 1m 1n)\n.TRAN 1n 1u\n"
                ".OPTIONS NONLIN-TRAN RELTOL=1e-4 ABSTOL=1e-9 DELTAXTOL=0.1 RHSTOL=1e-3\n"
                "+ SMALLUPDATETOL=1e-8 MAXSTEP=40\n.OPTIONS LINSOL TYPE=KLU\n.END\n")
    tr = d.netlist.tran
    assert (tr.nl_reltol, tr.nl_abstol, tr.nl_deltaxtol, tr.nl_rhstol) == (1e-4, 1e-9, 0.1, 1e-3)
    assert tr.nl_smallupdatetol == 1e-8 and tr.nl_maxstep == 40 and isinstance(tr.nl_maxstep, int)
    assert tr.reltol == 1e-3  # TIMEINT untouched
    for bad, msg in (("NONLIN-TRAN NLSTRATEGY=1", "NONLIN-TRAN NLSTRATEGY"),
                     ("LINSOL TYPE=AZTECOO", "LINSOL TYPE=AZTECOO"), ("LINSOL TYPE=IR", "LINSOL TYPE=IR")):
        with pytest.raises(ValueError, match=msg):
            S.parse(f"t\nR1 a 0 1\n.TRAN 1n 1u\n.OPTIONS {bad}\n.END\n")


def test_nested_subcircuits_and_diode_model():
    d = S.parse("""nested subcircuits
.SUBCKT LEAF a b
R1 a m 1k
D1 m b dmod 2
.ENDS
.SUBCKT PAIR x y
XL1 x mid LEAF
XL2 mid y LEAF
.ENDS
.MODEL dmod D (IS=1e-14 N=1.5 CJ0=1p)
X1 in 0 PAIR
V1 in 0 PWL(0 0 1n 1 2n 0)
.TRAN 10p 2n
.END
""")
    nl = d.netlist
    assert len(nl.res) == 2 and len(nl.diode) == 2
    # internal nodes are prefixed by the instance path
    assert {"X1:MID", "X1:XL1:M", "X1:XL2:M"} <= set(nl.names)
    row = nl.diode[0][3]
    f = N.DIODE_FIELDS.index
    assert row[f("IS")] == 1e-14 and row[f("N")] == 1.5 and row[f("CJO")] == 1e-12 and row[f("AREA")] == 2.0
    # the diode of XL2 ends on ground (PAIR's y = 0)
    assert nl.diode[1][1] == -1


def test_diode_sidewall_card():
    d = S.parse("""sidewall
.MODEL dsw D (IS=1e-14 JSW=2e-15 NS=1.2 CJP=0.1p PHP=0.7 MJSW=0.3 FCS=0.4)
.MODEL dmerged D (IS=1e-14 JSW=2e-15)
V1 a 0 SIN(0 1 1MEG)
D1 a 0 dsw PJ=3
D2 a 0 dmerged
.TRAN 1n 1u
.END
""")
    f = N.DIODE_FIELDS.index
    r1, r2 = d.netlist.diode[0][3], d.netlist.diode[1][3]
    assert r1[f("JSW")] == 2e-15 and r1[f("NS")] == 1.2 and r1[f("NSGIVEN")] == 1.0
    assert r1[f("CJSW")] == 1e-13 and r1[f("VJSW")] == 0.7 and r1[f("MJSW")] == 0.3
    assert r1[f("FCS")] == 0.4 and r1[f("PJ")] == 3.0
    # NS not given: the sidewall current merges into the bottom characteristic
    assert r2[f("NSGIVEN")] == 0.0 and r2[f("NS")] == 1.0 and r2[f("PJ")] == 0.0
    with pytest.raises(ValueError):
        S.parse("bad\n.MODEL d1 D (NSGIVEN=1)\nD1 a 0 d1\nV1 a 0 1\n.TRAN 1n 1u\n.END\n")


def test_mosfet1_series_resistance_card():
    d = S.parse("""series
.MODEL nrs NMOS (LEVEL=1 VTO=0.5 KP=120u RD=40 RS=25)
.MODEL psh PMOS (LEVEL=1 VTO=-0.5 KP=40u RSH=50)
VDD vdd 0 1.8
M1 out in 0 0 nrs W=2u L=0.18u
M2 out in vdd vdd psh W=4u L=0.18u NRD=2 NRS=1.5
V1 in 0 PULSE(0 1.8 0 10p 10p 100p 200p)
.TRAN 1p 100p
.END
""")
    nl = d.netlist
    f = N.MOS1_FIELDS.index
    (d1, g1, s1, b1, r1, dp1, sp1), (d2, g2, s2, b2, r2, dp2, sp2) = nl.mos1
    assert r1[f("RD")] == 40.0 and r1[f("RS")] == 25.0 and dp1 != d1 and sp1 != s1
    assert r2[f("RSH")] == 50.0 and r2[f("NRD")] == 2.0 and r2[f("NRS")] == 1.5
    assert dp2 != d2 and sp2 != s2
    assert N.mos1_series(r2) == (1.0 / 100.0, 1.0 / 75.0)


def test_temperature_statements():
    d = S.parse("""temperatures
.TEMP 85
.OPTIONS DEVICE TNOM=25
.MODEL d1 D (IS=1e-14)
.MODEL d2 D (IS=1e-14 TNOM=50 TRS1=1m)
.MODEL n1 NMOS (LEVEL=1 VTO=0.5 KP=100u)
V1 a 0 1
D1 a 0 d1
D2 a 0 d2 DTEMP=10
D3 a 0 d1 TEMP=-40
M1 a a 0 0 n1 W=1u L=1u
.PRINT TRAN V(a) TEMP
.TRAN 1n 10n
.END
""")
    nl = d.netlist
    fd, fm = N.DIODE_FIELDS.index, N.MOS1_FIELDS.index
    k = lambda c: c + N.CTOK
    (r1, r2, r3) = (nl.diode[i][3] for i in range(3))
    assert r1[fd("TEMP")] == k(85.0) and r1[fd("TNOM")] == k(25.0)
    assert r2[fd("TEMP")] == k(95.0) and r2[fd("TNOM")] == k(50.0) and r2[fd("TRS1")] == 1e-3
    assert r3[fd("TEMP")] == k(-40.0)
    m = nl.mos1[0][4]
    assert m[fm("TEMP")] == k(85.0) and m[fm("TNOM")] == k(25.0)
    assert d.temp_c == 85.0
    with pytest.raises(ValueError):  # the BSIM4 restatement runs at 27 C only
        S.parse(".title\n.TEMP 50\n.MODEL n4 NMOS (LEVEL=54)\nV1 a 0 1\nM1 a a 0 0 n4 L=45n W=90n\n"
                ".TRAN 1p 10p\n.END\n")


def test_inductor_element():
    d = S.parse("rl\nV1 a 0 PULSE(0 1 0 1p 1p 1 2)\nR1 a b 100\nL1 b 0 1u\n.PRINT TRAN I(L1) V(b)\n"
                ".TRAN 1n 50n\n.END\n")
    nl = d.netlist
    assert len(nl.ind) == 1 and nl.ind[0][3] == 1e-6 and d.branches["L1"] == nl.ind[0][2]
    assert d.element_values["L1"] == 1e-6
    with pytest.raises(ValueError):
        S.parse("rl\nV1 a 0 1\nL1 a 0 1u IC=1m\n.TRAN 1n 50n\n.END\n")


def test_bsim4_model_card_and_instance():
    d = S.parse("""bsim4 inverter
.MODEL n1 NMOS (LEVEL=54 VERSION=4.8.2 TOXE=1.8n VTH0=0.4)
.MODEL p1 PMOS (LEVEL=54 TOXE=1.8n VTH0=-0.4)
VDD vdd 0 1.0
VIN in 0 PULSE(0 1 10p 20p 20p 100p 240p)
MN out in 0 0 n1 L=45n W=90n
MP out in vdd vdd p1 L=45n W=180n
C1 out 0 2f
.TRAN 1p 500p
.END
""")
    nl = d.netlist
    assert len(nl.bsim4) == 2 and not nl.mos1
    f = N.B4_FIELDS.index
    rn, rp = nl.bsim4[0][4], nl.bsim4[1][4]
    assert rn[f("TYPE")] == 1 and rp[f("TYPE")] == -1
    assert rn[f("TOXE")] == 1.8e-9 and rn[f("VTH0")] == 0.4 and rp[f("VTH0")] == -0.4
    assert rn[f("L")] == 45e-9 and rp[f("W")] == 180e-9
    assert np.isnan(rn[f("K1")])  # not given: derived by the model as the reference does


def test_dollar_comments_and_ac_spec_ignored():
    d = S.parse("t\nV1 a 0 DC 2 AC 1 0 $ a comment\nR1 a 0 1k ; another\n.TRAN 1n 1u\n.END\n")
    a = d.netlist.arrays()
    assert a["vsrc"][3][0] == N.WAVE_DC and a["vsrc"][5][0] == 2.0


def test_print_of_unknown_node_raises():
    d = S.parse("t\nR1 a 0 1k\nI1 0 a 1m\n.TRAN 1n 1u\n.PRINT TRAN V(b)\n.END\n")
    with pytest.raises(ValueError, match="unknown node"):
        S._var_probes(d, "V(B)")


SWEEP = """RC sweep
.PARAM rval=1k
V1 in 0 PULSE(0 1 1n)
R1 in out {rval}
C1 out 0 1n
.TRAN 10p 2u 0 25n
.STEP rval LIST 1k 2k 4k
.PRINT TRAN V(out)
.MEASURE TRAN vmax MAX V(out)
.END
"""


def test_param_reference_and_step_list():
    decks = S.parse_sweep(SWEEP)
    assert [d.netlist.res[0][2] for d in decks] == [1e3, 2e3, 4e3]
    assert [d.step_values for d in decks] == [{"RVAL": 1e3}, {"RVAL": 2e3}, {"RVAL": 4e3}]
    assert decks[0].steps == [("RVAL", [1e3, 2e3, 4e3])]


def test_nested_linear_steps_outermost_first():
    text = SWEEP.replace(".STEP rval LIST 1k 2k 4k", ".STEP rval 1k 2k 1k\n.STEP C1 1n 3n 1n")
    decks = S.parse_sweep(text)
    got = [(d.netlist.res[0][2], d.netlist.cap[0][2]) for d in decks]
    assert got == [(1e3, 1e-9), (1e3, 2e-9), (1e3, 3e-9), (2e3, 1e-9), (2e3, 2e-9), (2e3, 3e-9)]


def test_step_of_unknown_name_raises():
    with pytest.raises(ValueError, match="no parameter or element"):
        S.parse_sweep(SWEEP.replace(".STEP rval", ".STEP rx"))
    with pytest.raises(ValueError, match="unknown parameter"):
        S.parse(SWEEP.replace("{rval}", "{nope}"))


def test_run_sweep_splits_the_batch(monkeypatch):
    """The sweep runs as one batch; each step gets its own circuit's rows
    (a stand-in for the GPU transient returns per-circuit waveforms)."""
    import xyce_gb300

    class FakeCircuit:
        def __init__(self, nl, device=0, arrays=None):
            self.nl = nl

        def transient(self, tran, probes=(), cap=0):
            nc = len(self.nl.offsets) - 1
            counts = np.array([3 + c for c in range(nc)], np.int32)
            times = np.zeros((nc, cap))
            values = np.zeros((nc, cap, 1))
            for c in range(nc):
                times[c, :counts[c]] = np.arange(counts[c]) * 1e-9
                values[c, :counts[c], 0] = 10.0 * (c + 1) + np.arange(counts[c])
            return counts, times, values, {"status": 0, "rejected": 0}

        def close(self):
            pass

    monkeypatch.setattr(xyce_gb300, "Circuit", FakeCircuit)
    decks = S.parse_sweep(SWEEP)
    res = S.run_sweep(decks, cap=64)
    assert [len(r.times) for r in res] == [3, 4, 5]
    np.testing.assert_array_equal(res[1].columns["V(OUT)"], [20, 21, 22, 23])
    assert [r.measures["VMAX"] for r in res] == [12.0, 23.0, 34.0]


def test_sweep_prn_layout(tmp_path):
    d = S.parse(SWEEP)
    rs = [S.Result(np.array([0.0, 1e-9]), {"V(OUT)": np.array([0.0, 0.5 + k])}, {}, {}) for k in range(2)]
    p = tmp_path / "s.prn"
    S.write_prn(str(p), d, rs)
    lines = p.read_text().splitlines()
    assert lines[0].split() == ["Index", "TIME", "V(OUT)"]
    assert [ln.split()[0] for ln in lines[1:-1]] == ["0", "1", "0", "1"]
    assert lines[-1] == "End of Xyce(TM) Parameter Sweep"


SAMPLING = """RC Monte Carlo
.PARAM rval=1k cval=1n
V1 in 0 PULSE(0 1 1n)
R1 in out {rval}
C1 out 0 {cval}
.TRAN 10p 2u 0 25n
.SAMPLING param=rval,cval type=normal,uniform means=1k std_deviations=100
+ lower_bounds=0.5n upper_bounds=1.5n
.OPTIONS SAMPLES NUMSAMPLES=400 SEED=7
.MEASURE TRAN vmax MAX V(out)
.END
"""


def test_sampling_spec_and_lhs_marginals():
    base = S.parse(SAMPLING)
    assert base.sampling["PARAM"] == ["RVAL", "CVAL"] and base.sampling["NUMSAMPLES"] == 400
    pts = S.sample_points(base.sampling)
    r = np.array([p["RVAL"] for p in pts])
    c = np.array([p["CVAL"] for p in pts])
    assert abs(r.mean() - 1e3) < 10 and abs(r.std() - 100) < 10
    assert c.min() >= 0.5e-9 and c.max() <= 1.5e-9
    # Latin hypercube: exactly one sample in each of the 400 strata of C
    strata = np.floor((c - 0.5e-9) / 1e-9 * 400).astype(int)
    assert sorted(strata) == list(range(400))
    decks = S.parse_sampling(SAMPLING)
    assert len(decks) == 400 and decks[3].netlist.res[0][2] == pytest.approx(pts[3]["RVAL"])
    assert S.sample_points(base.sampling) == pts  # seeded


def test_sample_moments():
    st = S.sample_moments([1.0, 2.0, 3.0, 4.0])
    assert st["mean"] == 2.5 and st["variance"] == 1.25 and st["min"] == 1.0 and st["max"] == 4.0
    assert st["skew"] == pytest.approx(0.0) and st["kurtosis"] == pytest.approx(1.64)
    assert S.sample_moments([2.0, 2.0])["skew"] == 0.0  # 0/0 reads 0


class _FakeCircuit:
    """Stand-in for the GPU transient: circuit c's probe j reads
    100 (j + 1) + 10 c + sample index at t = 1 ns x sample index."""

    def __init__(self, nl, device=0, arrays=None):
        self.nl = nl

    def transient(self, tran, probes=(), cap=0):
        nc = len(self.nl.offsets) - 1
        per = [0] * nc
        for u in probes:
            per[int(np.searchsorted(self.nl.offsets, u, side="right") - 1)] += 1
        pmax = max(1, max(per))
        counts = np.full(nc, 4, np.int32)
        times = np.zeros((nc, cap))
        values = np.zeros((nc, cap, pmax))
        for c in range(nc):
            times[c, :4] = np.arange(4) * 1e-9
            for j in range(per[c]):
                values[c, :4, j] = 100.0 * (j + 1) + 10.0 * c + np.arange(4)
        return counts, times, values, {"status": 0, "rejected": 0}

    def close(self):
        pass


def test_run_and_main_single_deck(monkeypatch, tmp_path):
    import xyce_gb300
    monkeypatch.setattr(xyce_gb300, "Circuit", _FakeCircuit)
    d = S.parse(RC)
    res = S.run(d, cap=16)
    # probes in first-use order: V(OUT) -> out; V(IN,OUT) -> in; I(V1) -> branch
    np.testing.assert_array_equal(res.columns["V(OUT)"], [100, 101, 102, 103])
    np.testing.assert_array_equal(res.columns["V(IN,OUT)"], [100, 100, 100, 100])  # in - out
    np.testing.assert_array_equal(res.columns["I(V1)"], [300, 301, 302, 303])
    assert res.measures["VMAX"] == 103.0
    path = tmp_path / "rc.cir"
    path.write_text(RC)
    assert S.main([str(path)]) == 0
    names, vals = S.read_prn(str(path) + ".prn")
    assert names == ["Index", "TIME", "V(OUT)", "V(IN,OUT)", "I(V1)"] and vals.shape == (4, 5)
    assert (tmp_path / "rc.cir.mt0").read_text().startswith("VMAX = 1.030000e+02")


def test_main_sweep_and_sampling_outputs(monkeypatch, tmp_path):
    import xyce_gb300
    monkeypatch.setattr(xyce_gb300, "Circuit", _FakeCircuit)
    p = tmp_path / "sw.cir"
    p.write_text(SWEEP)
    assert S.main([str(p)]) == 0
    lines = (tmp_path / "sw.cir.prn").read_text().splitlines()
    assert lines[-1] == "End of Xyce(TM) Parameter Sweep" and len(lines) == 1 + 3 * 4 + 1
    assert [(tmp_path / f"sw.cir.mt{k}").read_text() for k in range(3)] == [
        "VMAX = 1.030000e+02\n", "VMAX = 1.130000e+02\n", "VMAX = 1.230000e+02\n"]
    q = tmp_path / "mc.cir"
    q.write_text(SAMPLING.replace("NUMSAMPLES=400", "NUMSAMPLES=5"))
    assert S.main([str(q)]) == 0
    ms = (tmp_path / "mc.cir.ms0").read_text()
    assert ms.startswith("VMAX: mean = 1.230000e+02")  # circuits 0..4 -> max 103..143


@pytest.mark.parametrize("expr,val", [("2*1k", 2000.0), ("sqrt(4)+1", 3.0), ("2^3", 8.0), ("2**3", 8.0),
                                      ("-(1.5MEG/3)", -5e5), ("max(1,2.5)+min(3,-1)", 1.5), ("10n*1e9", 10.0),
                                      ("exp(0)*log(1)+abs(-2)", 2.0)])
def test_expression_values(expr, val):
    assert S.eval_expr(expr, {}) == pytest.approx(val, rel=1e-14)


def test_expression_errors():
    for bad in ("1/0", "__import__('os')", "x.y", "a if 1 else 2"):
        with pytest.raises(ValueError):
            S.eval_expr(bad, {"A": 1.0})
    with pytest.raises(ValueError):
        S.parse("t\n.PARAM a={b+1} b={a*2}\nR1 x 0 {a}\n.TRAN 1n 1u\n.END\n")  # a cycle
    with pytest.raises(ValueError):
        S.parse("t\nR1 x 0 {nosuch*2}\n.TRAN 1n 1u\n.END\n")


DECK_EXPR = """expressions
.PARAM r2={2*r1} r1=1k amp='r1/1k*0.5' cv={ 1p * (1 + 1) }
V1 in 0 SIN(0 {amp} 1MEG)
R1 in out {r2 + 500}
C1 out 0 {cv}
D1 out 0 dm
.MODEL dm D (IS={1e-15*10} N={sqrt(1.21)})
.TRAN 1n 1u
.END
"""


def test_param_expressions_in_elements_and_models():
    d = S.parse(DECK_EXPR)
    nl = d.netlist
    assert d.params["R1"] == 1000.0 and d.params["R2"] == 2000.0 and d.params["AMP"] == 0.5
    assert nl.res[0][2] == 2500.0 and nl.cap[0][2] == pytest.approx(2e-12, rel=1e-15)
    assert nl.vsrc[0][4][1] == 0.5
    f = N.DIODE_FIELDS.index
    assert nl.diode[0][3][f("IS")] == pytest.approx(1e-14) and nl.diode[0][3][f("N")] == pytest.approx(1.1)
    # a sweep point fixes r1, and r2 follows it
    d2 = S.parse(DECK_EXPR, {"r1": 5e3})
    assert d2.params["R2"] == 1e4 and d2.netlist.res[0][2] == 1.05e4


def test_include(tmp_path):
    sub = tmp_path / "lib"
    sub.mkdir()
    (sub / "models.inc").write_text(".MODEL dm D (IS=2e-14)\n.INC 'more.inc'\n")
    (sub / "more.inc").write_text("R9 out 0 3k\n")
    text = "inc\n.INCLUDE \"lib/models.inc\"\nV1 in 0 1\nR1 in out 1k\nD1 out 0 dm\n.TRAN 1n 1u\n.END\n"
    d = S.parse(text, base_dir=str(tmp_path))
    f = N.DIODE_FIELDS.index
    assert d.netlist.diode[0][3][f("IS")] == 2e-14 and sorted(r[2] for r in d.netlist.res) == [1000.0, 3000.0]
    with pytest.raises(ValueError):
        S.parse("inc\n.INCLUDE nosuch.inc\n.TRAN 1n 1u\n.END\n", base_dir=str(tmp_path))


def test_expression_print_variables():
    d = S.parse("t\nV1 a 0 1\nR1 a b 1k\nR2 b 0 1k\n.PRINT TRAN {V(a)-V(b)} {sqrt(abs(V(b)))*2}\n"
                ".MEASURE TRAN m MAX {V(a,b)*1k}\n.TRAN 1n 1u\n.END\n")
    assert d.prints == ["{V(A)-V(B)}", "{SQRT(ABS(V(B)))*2}"] and d.measures[0].var == "{V(A,B)*1K}"
    names = d.netlist.names
    va, vb = np.array([1.0, 2.0]), np.array([0.25, 1.0])
    vals = {names["A"]: va, names["B"]: vb}
    for var, want in ((d.prints[0], va - vb), (d.prints[1], np.sqrt(vb) * 2), (d.measures[0].var, (va - vb) * 1e3)):
        us, f = S._var_probes(d, var)
        assert set(us) == {names[k] for k in ("A", "B") if names[k] in us}
        np.testing.assert_allclose(f(vals), want, rtol=1e-15)
    with pytest.raises(ValueError):
        S._var_probes(d, "{V(A)+NOSUCH}")


@pytest.mark.parametrize("line,name,vals", [
    (".STEP DEC RV 1k 100k 2", "RV", [1e3, 1e3 * 10 ** 0.5, 1e4, 1e4 * 10 ** 0.5, 1e5]),
    (".STEP OCT RV 1 8 1", "RV", [1.0, 2.0, 4.0, 8.0]),
    (".STEP LIN RV 1 3 1", "RV", [1.0, 2.0, 3.0]),
    (".STEP DEC RV 100 1 3", "RV", [100.0]),
])
def test_step_sweep_kinds(line, name, vals):
    n, v = S._step(S._tokens(line)[1:])
    assert n == name
    np.testing.assert_allclose(v, vals, rtol=1e-12)


@pytest.mark.parametrize("tran,expect", [(".TRAN 1n 1u", 5e-9), (".TRAN 1n 1u 0 2n", 2e-9), (".TRAN 1n 1u 0 9n", 5e-9)])
def test_timeint_delmax(tran, expect):
    d = S.parse(f"t\nV1 a 0 1\nR1 a 0 1k\n{tran}\n.OPTIONS TIMEINT DELMAX=5n\n.END\n")
    assert d.netlist.tran.hmax == pytest.approx(expect)
