"""Timing .MEASUREs of the SPICE reader (TRIG/TARG, WHEN, FIND ... WHEN / AT)
on piecewise-linear waveforms whose breakpoints are sample points, so the
linear interpolation the reference uses (N_IO_MeasureRiseFallDelay.C,
N_IO_MeasureFindWhen.C, N_IO_MeasureWhenAT.C) is exact: a triangle of
period 4 crosses 0.5 rising at 0.5 and 4.5 and falling at 1.5 and 5.5."""
import numpy as np
import pytest

from xyce_gb300 import spice as S

T = np.arange(0.0, 8.0 + 1e-12, 0.25)


def tri(t):
    """Triangle wave: 0 at 0, 1 at 1, 0 at 2, -1 at 3, period 4."""
    p = np.mod(t, 4.0)
    return np.where(p <= 1, p, np.where(p <= 3, 2 - p, p - 4))


COLS = {"V(A)": tri(T), "V(B)": tri(T - 0.25)}


def meas(line):
    d = S.parse(f"m\nV1 a 0 1\nR1 a b 1k\nR2 b 0 1k\n.TRAN 1n 10n\n{line}\n.END\n")
    return S.evaluate_measure(d.measures[0], T, COLS)


@pytest.mark.parametrize("clause,expect", [
    ("", 0.5), ("RISE=2", 4.5), ("FALL=1", 1.5), ("CROSS=3", 4.5), ("RISE=LAST", 4.5),
    ("FALL=LAST", 5.5), ("CROSS=LAST", 5.5), ("TD=2", 4.5), ("FALL=1 TD=2", 5.5), ("RISE=3", float("nan")),
])
def test_when(clause, expect):
    got = meas(f".MEASURE TRAN t1 WHEN V(a)=0.5 {clause}")
    if np.isnan(expect):
        assert np.isnan(got)
    else:
        assert got == pytest.approx(expect, abs=1e-12)


def test_trig_targ_delay():
    # B is A delayed by 0.25: the same edges 0.25 later
    assert meas(".MEASURE TRAN tpd TRIG V(a) VAL=0.5 RISE=1 TARG V(b) VAL=0.5 RISE=1") == pytest.approx(0.25, abs=1e-12)
    assert meas(".MEASURE TRAN tpd TRIG V(a) VAL=0.5 RISE=1 TARG V(b) VAL=0.5 FALL=2") == pytest.approx(5.75 - 0.5, abs=1e-12)
    # the period from two rising edges of the same node
    assert meas(".MEASURE TRAN per TRIG V(a) VAL=0 RISE=1 TARG V(a) VAL=0 RISE=2") == pytest.approx(4.0, abs=1e-12)
    # TD skips the first edge of the trigger
    assert meas(".MEASURE TRAN d TRIG V(a) VAL=0.5 RISE=1 TD=1 TARG V(b) VAL=0.5 RISE=2") == pytest.approx(0.25, abs=1e-12)
    assert np.isnan(meas(".MEASURE TRAN d TRIG V(a) VAL=2 TARG V(b) VAL=0.5"))


def test_find():
    assert meas(".MEASURE TRAN f1 FIND V(b) WHEN V(a)=0.5 RISE=1") == pytest.approx(0.25, abs=1e-12)
    assert meas(".MEASURE TRAN f2 FIND V(b) WHEN V(a)=0.5 FALL=LAST") == pytest.approx(tri(5.5 - 0.25), abs=1e-12)
    assert meas(".MEASURE TRAN f3 FIND V(a) AT=2.5") == pytest.approx(-0.5, abs=1e-12)
    assert np.isnan(meas(".MEASURE TRAN f4 FIND V(a) AT=20"))


def test_measure_lines_rejected():
    for bad in (".MEASURE TRAN x TRIG V(a) RISE=1 TARG V(b) VAL=1",       # no VAL
                ".MEASURE TRAN x WHEN V(a) 0.5",                           # no '='
                ".MEASURE TRAN x WHEN V(a)=0.5 RISE=1 FALL=1",             # two counts
                ".MEASURE TRAN x FIND V(a) FROM=1"):
        with pytest.raises(ValueError):
            meas(bad)


def test_measure_variables_are_probed():
    d = S.parse("m\nV1 a 0 1\nR1 a b 1k\nR2 b 0 1k\n.TRAN 1n 10n\n"
                ".MEASURE TRAN f FIND V(b) WHEN V(a)=0.5\n.END\n")
    assert d.measures[0].vars == ["V(B)", "V(A)"]


def test_deriv():
    # the triangle's slope: +1 on (0,1) and (3,5), -1 on (1,3)
    assert meas(".MEASURE TRAN d1 DERIV V(a) AT=0.6") == pytest.approx(1.0, abs=1e-12)
    assert meas(".MEASURE TRAN d2 DERIVATIVE V(a) AT=2.0") == pytest.approx(-1.0, abs=1e-12)
    assert meas(".MEASURE TRAN d3 DERIV V(b) WHEN V(a)=0.5 FALL=1") == pytest.approx(-1.0, abs=1e-12)
    assert np.isnan(meas(".MEASURE TRAN d4 DERIV V(a) AT=20"))


def test_freq_and_duty():
    """A square wave of period 1 (on for the first half of each period)
    sampled every 0.01: inside FROM=0.25 TO=9.75 it falls 10 times and rises
    9 times in 9.5 time units, so FREQ = 0.5 * 19 / 9.5 = 1; it is on half
    the time."""
    t = np.round(np.arange(0.0, 10.0 + 1e-9, 0.01), 10)
    sq = np.where(np.mod(t, 1.0) < 0.5, 1.0, 0.0)
    d = S.parse("m\nV1 a 0 1\nR1 a 0 1k\n.TRAN 1n 10n\n"
                ".MEASURE TRAN f FREQ V(a) ON=0.8 OFF=0.2 FROM=0.25 TO=9.75\n"
                ".MEASURE TRAN dc DUTY V(a) ON=0.8 OFF=0.2 FROM=0.25 TO=9.75\n.END\n")
    cols = {"V(A)": sq}
    assert S.evaluate_measure(d.measures[0], t, cols) == pytest.approx(1.0, rel=1e-12)
    assert S.evaluate_measure(d.measures[1], t, cols) == pytest.approx(0.5, abs=0.02)


def test_on_and_off_time():
    """The same square wave: each on phase lasts 0.5 (the intervals of 0.01
    that end at an on sample), and the wave enters it once per period inside
    the window; the off phases likewise."""
    t = np.round(np.arange(0.0, 10.0 + 1e-9, 0.01), 10)
    sq = np.where(np.mod(t, 1.0) < 0.5, 1.0, 0.0)
    d = S.parse("m\nV1 a 0 1\nR1 a 0 1k\n.TRAN 1n 10n\n"
                ".MEASURE TRAN ton ON_TIME V(a) ON=0.8 OFF=0.2 FROM=0.25 TO=9.75\n"
                ".MEASURE TRAN toff OFF_TIME V(a) ON=0.8 OFF=0.2 FROM=0.25 TO=9.75\n.END\n")
    cols = {"V(A)": sq}
    ton = S.evaluate_measure(d.measures[0], t, cols)
    toff = S.evaluate_measure(d.measures[1], t, cols)
    assert ton == pytest.approx(0.5, abs=0.03) and toff == pytest.approx(0.5, abs=0.03)
