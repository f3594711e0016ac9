"""Physical invariants of every nonlinear device's load, checked on the
oracle with the device alone in a netlist (so F, Q and the Jacobians hold
its stamps only).  They hold for the reference's models by construction and
do not depend on how this build restates them:
  * Kirchhoff: the terminal currents (F) and terminal charges (Q) sum to
    zero (BSIM4's charge model is charge-conserving: the source charge is
    minus the sum of the others, N_DEV_MOSFET_B4p82.C);
  * conservation under perturbation: every column of dFdx and dQdx sums to
    zero;
  * only voltage differences matter: every row of dFdx and dQdx sums to
    zero.
The GPU stamps equal the oracle's to 1e-12 (tests/test_gpu_parity.py), so
the invariants carry over to the kernels."""
import numpy as np
import pytest
import scipy.sparse as sp

from xyce_gb300 import netlist as N

REL = 1e-9


def _settled_load(o, x):
    """A load at x whose junction history is x itself (no limiting)."""
    z = np.zeros(max(1, o.nsta))
    base = o.load(x, sta_curr=z, sto_curr=np.zeros(max(1, o.nsto)), newton_iter=0)
    sta, sto = base["sta_next"], base["sto_next"]
    for _ in range(200):
        nxt = o.load(x, sta_curr=sta, sto_curr=sto, sto_prev=sto, newton_iter=1)
        if np.array_equal(nxt["sto_next"], sto):
            return nxt
        sta, sto = nxt["sta_next"], nxt["sto_next"]
    raise AssertionError("history did not settle")


def _check(oracle_mod, nl, seed, lo, hi):
    o = oracle_mod.Oracle(nl)
    rng = np.random.default_rng(seed)
    for _ in range(4):
        x = rng.uniform(lo, hi, o.n)
        ld = _settled_load(o, x)
        for vec in ("F", "Q"):
            v = ld[vec]
            assert abs(v.sum()) <= REL * np.abs(v).max() + 1e-30, (nl.label, vec, v.sum(), np.abs(v).max())
        for mat in ("dFdx", "dQdx"):
            J = sp.csr_matrix((ld[mat], o.col_idx, o.row_ptr), shape=(o.n, o.n)).toarray()
            scale = np.abs(J).max() + 1e-300
            assert np.abs(J.sum(axis=0)).max() <= REL * scale, (nl.label, mat, "columns")
            assert np.abs(J.sum(axis=1)).max() <= REL * scale, (nl.label, mat, "rows")


def _alone(label, add):
    nl = N.Netlist(label=label)
    nodes = [nl.node(f"t{k}") for k in range(4)]
    add(nl, nodes)
    nl.tran = N.Tran(tstop=1e-9)
    return nl


@pytest.mark.parametrize("card", ["nmos", "pmos"])
def test_bsim4_conserves(oracle_mod, card):
    c = N.B4_NMOS if card == "nmos" else N.B4_PMOS
    nl = _alone(f"b4_{card}", lambda nl, t: nl.M4(t[0], t[1], t[2], t[3], **c))
    _check(oracle_mod, nl, 1, -0.3, 1.2)


@pytest.mark.parametrize("series", [False, True])
def test_mosfet1_conserves(oracle_mod, series):
    card = dict(N.NMOS_CARD, TOX=4e-9, CGSO=2e-10, CGDO=2e-10, CGBO=1e-10, CJ=1e-3, CJSW=2e-10, AD=1e-12,
                AS=1e-12, PD=4e-6, PS=4e-6, GAMMA=0.4, LAMBDA=0.05, PHI=0.7)
    if series:
        card.update(RD=300.0, RSH=20.0, NRS=2.0, M=2.0)
    nl = _alone("mos1", lambda nl, t: nl.M1(t[0], t[1], t[2], t[3], **card))
    _check(oracle_mod, nl, 2, -0.5, 2.0)


@pytest.mark.parametrize("k", range(3))
def test_diode_conserves(oracle_mod, k):
    card = N.SIDEWALL_DIODES[k]
    nl = _alone(f"diode{k}", lambda nl, t: nl.D(t[0], t[1], **card))
    _check(oracle_mod, nl, 3, -5.0, 1.0)


@pytest.mark.parametrize("model", ["b4_nmos", "b4_pmos", "mos1"])
def test_source_drain_symmetry(oracle_mod, model):
    """A MOSFET with symmetric geometry is symmetric in drain and source:
    swapping the two terminal voltages swaps their currents and charges and
    leaves the gate's and the bulk's unchanged (the reverse mode of the
    reference's models, e.g. N_DEV_MOSFET_B4p82.C's mode = -1 branch).
    MOSFET-1's Meyer charges are incremental (the stored charge plus
    C * the change of voltage since the stored state), so they depend on
    the history and only its currents are compared."""
    if model == "mos1":
        card = dict(N.NMOS_CARD, TOX=4e-9, CGSO=2e-10, CGDO=2e-10, CJ=1e-3, CJSW=2e-10, AD=1e-12, AS=1e-12,
                    PD=4e-6, PS=4e-6, GAMMA=0.4, LAMBDA=0.05, PHI=0.7)
        nl = _alone("mos1", lambda nl, t: nl.M1(t[0], t[1], t[2], t[3], **card))
    else:
        c = dict(N.B4_NMOS if model == "b4_nmos" else N.B4_PMOS)
        c.update(AS=2e-14, AD=2e-14, PS=6e-7, PD=6e-7)
        nl = _alone(model, lambda nl, t: nl.M4(t[0], t[1], t[2], t[3], **c))
    o = oracle_mod.Oracle(nl)
    d, g, s, b = (nl.names[f"t{k}"] for k in range(4))
    rng = np.random.default_rng(5)
    sign = -1.0 if model == "b4_pmos" else 1.0
    for _ in range(4):
        x = sign * rng.uniform(-0.2, 1.2, o.n)
        y = x.copy()
        y[d], y[s] = x[s], x[d]
        a, r = _settled_load(o, x), _settled_load(o, y)
        for vec in (("F",) if model == "mos1" else ("F", "Q")):
            va, vr = a[vec], r[vec]
            tol = REL * np.abs(va).max() + 1e-30
            assert abs(vr[d] - va[s]) <= tol and abs(vr[s] - va[d]) <= tol, (model, vec)
            assert abs(vr[g] - va[g]) <= tol and abs(vr[b] - va[b]) <= tol, (model, vec)


def test_bsim4_textbook_behaviour(oracle_mod):
    """The 45 nm-like NMOS card shows the behaviours every MOSFET model has:
    an exponential subthreshold region no steeper than the thermal limit
    (kT/q ln 10 = 59.6 mV/decade at 300 K), drain-induced barrier lowering
    (more subthreshold current at high Vds), the body effect (less current
    with reverse body bias) and saturation (output conductance far below
    the linear region's).  The body effect is checked on a 1 um channel:
    with the card's default short-channel parameters the 45 nm device's
    current rises with reverse body bias (the depletion width, and with it
    the short-channel threshold roll-off and ETAB's DIBL, grow with it)."""
    nl = _alone("b4_textbook", lambda nl, t: nl.M4(t[0], t[1], t[2], t[3], **N.B4_NMOS))
    o = oracle_mod.Oracle(nl)
    d, g, s, b = (nl.names[f"t{k}"] for k in range(4))

    def ids(vg, vd, vb=0.0):
        x = np.zeros(o.n)
        x[d], x[g], x[b] = vd, vg, vb
        return _settled_load(o, x)["F"][d]

    sub = np.array([ids(vg, 1.0) for vg in (0.0, 0.05, 0.10, 0.15)])
    assert np.all(sub > 0)
    swing = 0.05 / np.diff(np.log10(sub))  # volts per decade
    vt = 1.3806226e-23 * 300.15 / 1.6021918e-19
    assert np.all(swing > vt * np.log(10) * 0.999) and np.all(swing < 0.15), swing
    assert np.max(swing) / np.min(swing) < 1.2, swing  # exponential: a steady slope
    assert ids(0.1, 1.0) > 2.0 * ids(0.1, 0.05)  # DIBL
    long_ch = _alone("b4_long", lambda nl, t: nl.M4(t[0], t[1], t[2], t[3], **dict(N.B4_NMOS, L=1e-6, W=2e-6)))
    ol = oracle_mod.Oracle(long_ch)

    def ids_long(vg, vd, vb=0.0):
        x = np.zeros(ol.n)
        x[d], x[g], x[b] = vd, vg, vb
        return _settled_load(ol, x)["F"][d]
    assert ids_long(0.6, 1.0, -0.5) < ids_long(0.6, 1.0, -0.2) < ids_long(0.6, 1.0)  # body effect
    # saturation: the output conductance is well below the linear region's,
    # by a large factor on the long channel (short channels keep a sizeable
    # one from channel-length modulation and DIBL)
    for f, bound in ((ids_long, 0.2), (ids, 0.5)):
        g_lin = (f(1.0, 0.06) - f(1.0, 0.04)) / 0.02
        g_sat = (f(1.0, 1.0) - f(1.0, 0.9)) / 0.1
        assert 0 < g_sat < bound * g_lin, (g_sat, g_lin)
