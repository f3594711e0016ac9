"""CPU tests of the oracle (the checker of the GPU path).

Pins, in the absence of the reference's own regression waveforms (they live in
the separate Xyce_Regression repository, not in the reference tree):
  * known answers of the reference's unit-test netlists
    (test/CircuitPKG/TestNetlist1.cir: V(1) = 5; TestNetlist2.cir: V(1) = sin(2 pi t),
    V(2) = V(1)*100/150),
  * an analytic RC step response,
  * finite-difference Jacobians of every device load (the reference's TESTJAC
    check, src/DeviceModelPKG/Core/N_DEV_NumericalJacobian.C:154),
  * the sparse LU against Kundert Sparse compiled from the reference's sources
    (golden fixture tests/golden/ksparse_solves.npz) and against scipy.
"""
import os
import sys

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

from xyce_gb300 import netlist as N

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ksparse_solves.npz")


def test_testnetlist1_dc_value(oracle_mod):
    nl = N.test_netlist1()
    t, v, st = oracle_mod.Oracle(nl).transient(probes=[nl.names["1"]])
    assert st["status"] == 0 and st["t_final"] == pytest.approx(1.0)
    np.testing.assert_array_equal(v[:, 0], 5.0)


def test_testnetlist2_analytic(oracle_mod):
    nl = N.test_netlist2()
    t, v, st = oracle_mod.Oracle(nl).transient(probes=[nl.names["1"], nl.names["2"]])
    assert st["status"] == 0
    np.testing.assert_allclose(v[:, 0], np.sin(2 * np.pi * t), atol=1e-12)
    np.testing.assert_allclose(v[:, 1], np.sin(2 * np.pi * t) * 100 / 150, atol=1e-12)


def test_rc_step_within_reltol(oracle_mod):
    nl = N.rc_step(r=1e3, c=1e-9, v=1.0, tstop=5e-6)
    t, v, st = oracle_mod.Oracle(nl).transient(probes=[nl.names["out"]])
    ref = 1.0 - np.exp(-np.maximum(t - 1e-12, 0.0) / 1e-6)
    # TIMEINT RELTOL 1e-3 on a 1 V signal: the LTE control keeps the error near it
    assert np.max(np.abs(v[:, 0] - ref)) < 1e-3


def _fd_check(oracle_mod, nl, rng, dcop, shift=0.0):
    o = oracle_mod.Oracle(nl)
    _, x0, _ = o.dcop()
    x = x0 + shift + 0.05 * rng.standard_normal(o.n)
    z = np.zeros(max(1, o.nsta))
    base = o.load(x, dcop=dcop, sta_curr=z, sto_curr=np.zeros(max(1, o.nsto)), newton_iter=0)
    # history equal to the point itself: no limiting, and the back-averaged
    # Meyer charge has its capacitance as exact derivative
    sta_c, sto_c = base["sta_next"], base["sto_next"]
    # from a zero history the junction limiting may have moved the stored
    # voltages (a diode in breakdown); reload until the history is the point
    for _ in range(200):
        nxt = o.load(x, dcop=dcop, sta_curr=sta_c, sto_curr=sto_c, sto_prev=sto_c, newton_iter=1)
        if np.array_equal(nxt["sto_next"], sto_c):
            break
        sta_c, sto_c = nxt["sta_next"], nxt["sto_next"]
    else:
        raise AssertionError("junction history did not settle")
    ref = o.load(x, dcop=dcop, sta_curr=sta_c, sto_curr=sto_c, sto_prev=sto_c, newton_iter=1)
    J = {k: sp.csr_matrix((ref[k], o.col_idx, o.row_ptr), shape=(o.n, o.n)).toarray()
         for k in ("dFdx", "dQdx")}
    for j in range(o.n):
        h = 1e-7 * (1.0 + abs(x[j]))
        xp, xm = x.copy(), x.copy()
        xp[j] += h
        xm[j] -= h
        lp = o.load(xp, dcop=dcop, sta_curr=sta_c, sto_curr=sto_c, sto_prev=sto_c, newton_iter=1)
        lm = o.load(xm, dcop=dcop, sta_curr=sta_c, sto_curr=sto_c, sto_prev=sto_c, newton_iter=1)
        for vec, mat in (("F", "dFdx"), ("Q", "dQdx")):
            fd = (lp[vec] - lm[vec]) / (2 * h)
            an = J[mat][:, j]
            scale = np.max(np.abs(J[mat])) + 1e-300
            np.testing.assert_allclose(fd, an, rtol=1e-4, atol=1e-5 * scale,
                                       err_msg=f"{nl.label} {mat}[:, {j}]")


@pytest.mark.parametrize("maker", [lambda: N.diode_ladder(8, seed=3),
                                   lambda: N.diode_ladder(9, seed=3, sidewall=True),
                                   lambda: N.ring_oscillator(5),
                                   lambda: N.ring_oscillator(5, caps=True),
                                   lambda: N.ring_oscillator(5, series=True),
                                   lambda: N.rlc_ladder(6, seed=2),
                                   lambda: N.ring_oscillator(5, caps=True, series=True),
                                   lambda: N.bsim4_inverter_chain(2),
                                   lambda: N.bsim4_logic_dag(60, 4, seed=2, tstop=0.3e-9),
                                   lambda: N.at_temperature(N.ring_oscillator(5, caps=True), 100.0, 40.0),
                                   lambda: N.at_temperature(N.diode_ladder(9, seed=3, sidewall=True), -20.0, 50.0,
                                                            IKF=5e-3, TIKF=0.01, TBV1=1e-3, TBV2=1e-6,
                                                            TRS1=2e-3, TRS2=1e-5)])
def test_finite_difference_jacobian(oracle_mod, maker):
    rng = np.random.default_rng(7)
    _fd_check(oracle_mod, maker(), rng, dcop=False)


@pytest.mark.parametrize("shift", [1.6, -4.2])
def test_finite_difference_jacobian_sidewall_regimes(oracle_mod, shift):
    """The sidewall ladder's operating point is reverse-biased (-1 V); shifted
    points put the junctions forward, above the sidewall depletion threshold
    (+0.6 V), and in breakdown for the BV = 4 V card (-5.2 V)."""
    rng = np.random.default_rng(11)
    _fd_check(oracle_mod, N.diode_ladder(9, seed=3, sidewall=True), rng, dcop=False, shift=shift)


def test_lu_matches_ksparse_golden(oracle_mod):
    """The oracle's LU reproduces the reference solver's own solutions."""
    sys.path.insert(0, os.path.dirname(__file__))
    from golden.make_golden import circuits
    g = np.load(GOLDEN)
    specs = {name: nl for name, nl, _ in circuits()}
    for name in g["names"]:
        rp, ci, vals, b, xk = (g[f"{name}.{k}"] for k in ("row_ptr", "col_idx", "vals", "b", "x_ksparse"))
        o = oracle_mod.Oracle(specs[str(name)])
        np.testing.assert_array_equal(o.row_ptr, rp)
        np.testing.assert_array_equal(o.col_idx, ci)
        x = o.lu_solve(vals, b)
        np.testing.assert_allclose(x, xk, rtol=1e-9, atol=1e-12 * np.max(np.abs(xk)), err_msg=str(name))


def test_oracle_lu_matches_scipy_and_ksparse(oracle_mod):
    rng = np.random.default_rng(5)
    for nl, h in [(N.ring_oscillator(31), 1e-12), (N.diode_ladder(40, seed=2), 1e-9),
                  (N.ring_oscillator(21, caps=True), 1e-12), (N.power_grid(10, 10), 1e-12)]:
        o = oracle_mod.Oracle(nl)
        _, x0, _ = o.dcop()
        ld = o.load(x0 + 0.01 * rng.standard_normal(o.n))
        for vals in (ld["dFdx"] + ld["dQdx"] / h, ld["dFdx"]):
            b = rng.standard_normal(o.n)
            A = sp.csr_matrix((vals, o.col_idx, o.row_ptr), shape=(o.n, o.n))
            x = o.lu_solve(vals, b)
            assert np.linalg.norm(A @ x - b) <= 1e-10 * np.linalg.norm(b)
        if os.path.exists(oracle_mod.KSPARSE_PATH):
            vals = ld["dFdx"] + ld["dQdx"] / h
            b = rng.standard_normal(o.n)
            xk = oracle_mod.ksparse_solve(o.row_ptr, o.col_idx, vals, b)
            np.testing.assert_allclose(o.lu_solve(vals, b), xk, rtol=1e-8,
                                       atol=1e-12 * np.max(np.abs(xk)))


def test_ring_dc_operating_point_symmetric(oracle_mod):
    """An odd ring has one DC solution: every stage at the inverter's switching
    point, where the NMOS and PMOS saturation currents are equal."""
    nl = N.ring_oscillator(11)
    st, x, it = oracle_mod.Oracle(nl).dcop()
    assert st > 0
    v = x[[nl.names[f"n{i + 1}"] for i in range(11)]]
    bn = 120e-6 * 2 / 0.18
    bp = 40e-6 * 4 / 0.18
    vm = (1.3 * np.sqrt(bp) + 0.5 * np.sqrt(bn)) / (np.sqrt(bn) + np.sqrt(bp))
    np.testing.assert_allclose(v, vm, atol=1e-6)


def test_ring_oscillates(oracle_mod):
    nl = N.ring_oscillator(21)
    nl.tran.tstop = 5e-9
    t, v, st = oracle_mod.Oracle(nl).transient(probes=[nl.names["n5"]])
    assert st["status"] == 0
    assert v[:, 0].max() > 1.7 and v[:, 0].min() < 0.1


def test_diode_iv_point(oracle_mod):
    """Diode from a 1 V source through 1 kohm: Id = IS (exp(Vd/Vt) - 1), KVL."""
    nl = N.Netlist(label="diode_iv")
    a, k = nl.node("a"), nl.node("k")
    nl.V(a, -1, N.WAVE_DC, [1.0])
    nl.R(a, k, 1e3)
    nl.D(k, -1, IS=1e-14, N=1.0)
    st, x, it = oracle_mod.Oracle(nl).dcop()
    vd = x[k]
    vt = 1.3806226e-23 * 300.15 / 1.6021918e-19
    i_r = (1.0 - vd) / 1e3
    i_d = 1e-14 * np.expm1(vd / vt) + 1e-12 * vd
    # the operating-point Newton stops at RHSTOL = 1e-6 A (N_NLS_Manager.C:1033)
    assert abs(i_r - i_d) < 1e-6
    assert 0.55 < vd < 0.75


@pytest.mark.parametrize("ns", [1.3, None])
def test_diode_sidewall_iv_point(oracle_mod, ns):
    """Sidewall current at DC (N_DEV_Diode.C:1226-1260): with NS given it adds
    JSW*PJ*(exp(Vd/(NS Vt)) - 1); without NS, JSW*PJ joins IS*AREA in the
    bottom characteristic."""
    nl = N.Netlist(label="diode_sw_iv")
    a, k = nl.node("a"), nl.node("k")
    nl.V(a, -1, N.WAVE_DC, [1.0])
    nl.R(a, k, 1e3)
    card = dict(IS=1e-14, N=1.0, JSW=4e-14, PJ=2.5, CJSW=1e-13)
    if ns is not None:
        card["NS"] = ns
    nl.D(k, -1, **card)
    st, x, it = oracle_mod.Oracle(nl).dcop()
    vd = x[k]
    vt = 1.3806226e-23 * 300.15 / 1.6021918e-19
    isw = 4e-14 * 2.5
    if ns is None:
        i_d = (1e-14 + isw) * np.expm1(vd / vt)
    else:
        i_d = 1e-14 * np.expm1(vd / vt) + isw * np.expm1(vd / (ns * vt))
    assert abs((1.0 - vd) / 1e3 - (i_d + 1e-12 * vd)) < 1e-6
    assert 0.45 < vd < 0.75


KB, QE, TREF = 1.3806226e-23, 1.6021918e-19, 300.15


def test_rl_step_response(oracle_mod):
    """Inductor (N_DEV_Inductor.C): a 1 V step through R into L gives
    i(t) = (V/R)(1 - exp(-t R/L)); at DC the inductor is a short."""
    nl = N.Netlist(label="rl")
    a, k = nl.node("a"), nl.node("k")
    nl.V(a, -1, N.WAVE_PULSE, [0.0, 1.0, 0.0, 1e-12, 1e-12, 1.0, 2.0])
    nl.R(a, k, 100.0)
    br = nl.L(k, -1, 1e-6)
    nl.tran = N.Tran(tstop=50e-9, hmax=0.2e-9, reltol=1e-4)
    t, v, st = oracle_mod.Oracle(nl).transient(probes=[br, k])
    assert st["status"] == 0
    tau = 1e-6 / 100.0
    ref = 0.01 * (1.0 - np.exp(-np.maximum(t - 1e-12, 0.0) / tau))
    assert np.max(np.abs(v[:, 0] - ref)) < 2e-3 * 0.01
    # the inductor's voltage is L di/dt = V exp(-t/tau)
    late = t > 5e-9
    np.testing.assert_allclose(v[late, 1], np.exp(-(t[late] - 1e-12) / tau), rtol=0, atol=5e-3)


def test_diode_temperature_dc_point(oracle_mod):
    """Diode at 75 C with TNOM 27 C (updateTemperature, N_DEV_Diode.C:1430-1470):
    IS(T) = IS exp((T/TNOM - 1) EG/(N vt) + XTI/N ln(T/TNOM)), vt = kT/q;
    RS(T) = RS (1 + dT (TRS1 + TRS2 dT))."""
    nl = N.Netlist(label="diode_75C")
    a, k = nl.node("a"), nl.node("k")
    nl.V(a, -1, N.WAVE_DC, [1.0])
    nl.R(a, k, 1e3)
    nl.D(k, -1, IS=1e-14, N=1.2, EG=1.11, XTI=3.0, RS=20.0, TRS1=5e-3, TRS2=1e-5,
         TEMP=75.0 + N.CTOK, TNOM=27.0 + N.CTOK)
    st, x, it = oracle_mod.Oracle(nl).dcop()
    T, TN = 75.0 + N.CTOK, 27.0 + N.CTOK
    vt = KB * T / QE
    is_t = 1e-14 * np.exp((T / TN - 1.0) * 1.11 / (1.2 * vt) + 3.0 / 1.2 * np.log(T / TN))
    rs_t = 20.0 * (1 + (T - TN) * (5e-3 + 1e-5 * (T - TN)))
    pri = nl.diode[0][2]
    vd = x[pri]
    i_r = (1.0 - x[k]) / 1e3
    assert abs(i_r - (x[k] - vd) / rs_t) < 1e-9
    assert abs(i_r - (is_t * np.expm1(vd / (1.2 * vt)) + 1e-12 * vd)) < 1e-6
    assert 0.3 < vd < 0.7


def test_mosfet1_temperature_saturation_current(oracle_mod):
    """NMOS (GAMMA = 0, LAMBDA = 0) in saturation at 100 C with TNOM 27 C
    (Instance::updateTemperature, N_DEV_MOSFET1.C:3525-3560): beta scales by
    (T/TNOM)^-1.5 and VTO moves by (egfet(TNOM) - egfet(T))/2 + (tPhi - PHI)/2.
    The reverse-biased drain junction adds (IS(T)/vt + gmin) * Vdb, with
    IS(T) = IS exp(-egfet(T)/vt + egfet(TNOM)/vtnom) (the linear reverse
    junction of the reference's MOSFET-1)."""
    T, TN, vto, phi, kp = 100.0 + N.CTOK, 27.0 + N.CTOK, 0.5, 0.6, 120e-6
    nl = N.Netlist(label="nmos_100C")
    vdd, gate = nl.node("vdd"), nl.node("g")
    br = nl.V(vdd, -1, N.WAVE_DC, [1.8])
    nl.V(gate, -1, N.WAVE_DC, [1.2])
    nl.M1(vdd, gate, -1, -1, TYPE=1.0, VTO=vto, KP=kp, PHI=phi, W=2e-6, L=0.18e-6, TEMP=T, TNOM=TN)
    st, x, it = oracle_mod.Oracle(nl).dcop()
    egfet = lambda t: 1.16 - 7.02e-4 * t * t / (t + 1108)

    def pbfact(t):
        vt = KB * t / QE
        arg = -egfet(t) / (2 * KB * t) + 1.1150877 / (KB * (TREF + TREF))
        return -2 * vt * (1.5 * np.log(t / TREF) + QE * arg)
    phio = (phi - pbfact(TN)) / (TN / TREF)
    tphi = T / TREF * phio + pbfact(T)
    tvto = vto + 0.5 * (egfet(TN) - egfet(T)) + 0.5 * (tphi - phi)
    beta = kp / (T / TN) ** 1.5 * 2e-6 / 0.18e-6
    vt, vtnom = KB * T / QE, KB * TN / QE
    is_t = 1e-14 * np.exp(-egfet(T) / vt + egfet(TN) / vtnom)
    i_d = beta / 2 * (1.2 - tvto) ** 2 + (is_t / vt + 1e-12) * 1.8
    assert abs(abs(x[br]) - i_d) < 1e-9 * i_d
    assert abs(tvto - vto) > 0.05  # the shift is not negligible at 100 C


def test_mosfet1_series_resistance_dc_point(oracle_mod):
    """NMOS in saturation with RS in the source and RD in the drain
    (N_DEV_MOSFET1.C:410-450, 2212-2240): Id = beta/2 (Vg - Id RS - VTO)^2,
    the drain' sits Id * RD below the supply, the source' Id * RS above ground."""
    nl = N.Netlist(label="nmos_rs")
    vdd, gate = nl.node("vdd"), nl.node("g")
    nl.V(vdd, -1, N.WAVE_DC, [1.8])
    nl.V(gate, -1, N.WAVE_DC, [1.2])
    nl.M1(vdd, gate, -1, -1, TYPE=1.0, VTO=0.5, KP=120e-6, W=2e-6, L=0.18e-6, RD=2000.0, RS=500.0)
    d, g, s, b, row, dp, sp = nl.mos1[0]
    assert dp != d and sp != s and sp >= 0
    st, x, it = oracle_mod.Oracle(nl).dcop()
    beta = 120e-6 * 2e-6 / 0.18e-6
    # beta/2 (v - RS Id)^2 = Id with v = Vg - VTO: the smaller root
    v, rs = 1.2 - 0.5, 500.0
    a = beta / 2 * rs * rs
    bq = -(beta * rs * v + 1.0)
    cq = beta / 2 * v * v
    i_d = (-bq - np.sqrt(bq * bq - 4 * a * cq)) / (2 * a)
    assert abs(x[sp] - i_d * rs) < 1e-6 and abs(1.8 - x[dp] - i_d * 2000.0) < 1e-6
    # RSH with squares gives the same point as the equal RD / RS
    nl2 = N.Netlist(label="nmos_rsh")
    vdd, gate = nl2.node("vdd"), nl2.node("g")
    nl2.V(vdd, -1, N.WAVE_DC, [1.8])
    nl2.V(gate, -1, N.WAVE_DC, [1.2])
    nl2.M1(vdd, gate, -1, -1, TYPE=1.0, VTO=0.5, KP=120e-6, W=2e-6, L=0.18e-6, RSH=100.0, NRD=20.0,
           NRS=5.0)
    st2, x2, _ = oracle_mod.Oracle(nl2).dcop()
    assert abs(x2[nl2.mos1[0][6]] - x[sp]) < 1e-9 and abs(x2[nl2.mos1[0][5]] - x[dp]) < 1e-9


def test_mosfet1_series_nodes_are_checked(oracle_mod):
    nl = N.ring_oscillator(3, series=True)
    d, g, s, b, row, dp, sp = nl.mos1[0]
    nl.mos1[0] = (d, g, s, b, row, d, sp)  # RD given but no drain' node
    with pytest.raises(ValueError):
        oracle_mod.Oracle(nl)


def test_bsim4_iv_known_behaviour(oracle_mod):
    """BSIM4 (level 54) drain current of the 45 nm-like cards: off current
    far below on current, monotone in Vgs, sign set by TYPE, zero at Vds = 0."""
    for typ in (1.0, -1.0):
        nl = N.Netlist(label="b4_iv")
        d, g = nl.node("d"), nl.node("g")
        nl.V(d, -1, N.WAVE_DC, [typ])
        nl.V(g, -1, N.WAVE_DC, [typ])
        nl.M4(d, g, -1, -1, **(N.B4_NMOS if typ > 0 else N.B4_PMOS))
        nl.tran = N.Tran(tstop=1e-9)
        o = oracle_mod.Oracle(nl)
        z = np.zeros(o.nsto)
        ids = []
        for vg in np.linspace(0.0, 1.0, 11):
            x = np.zeros(o.n)
            x[d], x[g] = typ * 1.0, typ * vg
            ids.append(typ * o.load(x, newton_iter=1, sto_curr=z, sto_prev=z)["F"][d])
        ids = np.array(ids)
        assert np.all(np.diff(ids) > 0), ids
        assert ids[0] < 1e-9 and ids[-1] > 5e-5 and ids[-1] / ids[0] > 1e5, ids
        x = np.zeros(o.n)
        x[g] = typ * 1.0
        assert abs(o.load(x, newton_iter=1, sto_curr=z, sto_prev=z)["F"][d]) < 1e-15


def test_bsim4_chain_switches(oracle_mod):
    """Three BSIM4 inverters follow their PULSE input with alternating polarity."""
    nl = N.bsim4_inverter_chain(3)
    pr = [nl.names[k] for k in ("in", "n1", "n2", "n3")]
    t, v, st = oracle_mod.Oracle(nl).transient(probes=pr)
    assert st["status"] == 0
    k = np.searchsorted(t, 0.3e-9)  # input high since ~70 ps
    assert v[k, 0] > 0.99 and v[k, 1] < 0.05 and v[k, 2] > 0.95 and v[k, 3] < 0.05
    k = np.searchsorted(t, 0.65e-9)  # input low again since ~390 ps
    assert v[k, 0] < 0.01 and v[k, 1] > 0.95 and v[k, 3] > 0.95


# ---- Gear12 (BDF1/2), .OPTIONS TIMEINT METHOD=GEAR ---------------------------

def _gear(nl):
    nl.tran.method = 8
    return nl


def test_gear_testnetlists_exact(oracle_mod):
    """Source-driven nodes are exact under any integrator."""
    nl = _gear(N.test_netlist2())
    t, v, st = oracle_mod.Oracle(nl).transient(probes=[nl.names["1"], nl.names["2"]])
    assert st["status"] == 0 and st["t_final"] == pytest.approx(1.0)
    np.testing.assert_allclose(v[:, 0], np.sin(2 * np.pi * t), atol=1e-12)
    np.testing.assert_allclose(v[:, 1], np.sin(2 * np.pi * t) * 100 / 150, atol=1e-12)


def test_gear_rc_step_within_reltol(oracle_mod):
    nl = _gear(N.rc_step(r=1e3, c=1e-9, v=1.0, tstop=5e-6))
    t, v, st = oracle_mod.Oracle(nl).transient(probes=[nl.names["out"]])
    assert st["status"] == 0
    ref = 1.0 - np.exp(-np.maximum(t - 1e-12, 0.0) / 1e-6)
    assert np.max(np.abs(v[:, 0] - ref)) < 1e-3


def test_gear_rc_converges_at_second_order(oracle_mod):
    """Steps held at HMAX (tolerances too loose to bind): halving the step
    divides the error by ~4 for both second-order methods, Gear's error
    constant being the larger (BDF2 2/9 against the trapezoid's 1/12)."""
    errs = {}
    for method in (7, 8):
        for hm in (20e-9, 10e-9):
            nl = N.rc_step(r=1e3, c=1e-9, v=1.0, tstop=3e-6)
            nl.tran.method, nl.tran.reltol, nl.tran.abstol, nl.tran.hmax = method, 1.0, 1.0, hm
            t, v, st = oracle_mod.Oracle(nl).transient(probes=[nl.names["out"]])
            assert st["status"] == 0
            late = t > 1e-6
            ref = 1.0 - np.exp(-(t[late] - 1e-12) / 1e-6)
            errs[method, hm] = np.max(np.abs(v[late, 0] - ref))
    for method in (7, 8):
        assert 3.0 < errs[method, 20e-9] / errs[method, 10e-9] < 5.0
    assert 2.0 < errs[8, 10e-9] / errs[7, 10e-9] < 6.0


def test_gear_first_order_is_backward_euler(oracle_mod):
    """MAXORD=1: Gear12 and OneStep both reduce to backward Euler with the
    same coefficients; their waveforms agree to rounding on a linear circuit
    (the step-size controllers see different error constants, so compare at
    a fixed step: HMAX well below every step the error control would take)."""
    out = []
    for method in (7, 8):
        nl = N.rc_step(r=1e3, c=1e-9, v=1.0, tstop=1e-6)
        nl.tran.method = method
        nl.tran.max_order = 1
        nl.tran.hmax = 1e-9
        nl.tran.reltol = 1.0
        t, v, st = oracle_mod.Oracle(nl).transient(probes=[nl.names["out"]])
        out.append((t, v[:, 0]))
    (t7, v7), (t8, v8) = out
    n = min(len(t7), len(t8))
    same = np.flatnonzero(np.abs(t7[:n] - t8[:n]) < 1e-18)
    assert len(same) > 100
    np.testing.assert_allclose(v8[same], v7[same], rtol=1e-9, atol=1e-12)


def test_gear_ring_oscillates(oracle_mod):
    nl = _gear(N.ring_oscillator(21, caps=True))
    t, v, st = oracle_mod.Oracle(nl).transient(probes=[nl.names["n1"]])
    assert st["status"] == 0
    late = v[t > 5e-9, 0]
    assert late.max() > 1.5 and late.min() < 0.3


# ---- failure paths (injected on the host: no GPU fault) ----------------------

def test_nan_parameter_fails_operating_point_with_nan_code(oracle_mod):
    """A NaN element value makes the residual NaN: DampedNewton's nanFail
    (-6, N_NLS_DampedNewton.C:1207-1253) ends the operating point, reported
    as -100 + code."""
    nl = N.rc_step()
    a, b, _ = nl.res[0]
    nl.res[0] = (a, b, float("nan"))
    t, v, st = oracle_mod.Oracle(nl).transient(probes=[nl.names["out"]])
    assert st["status"] == -106 and st["accepted"] == 0


def test_one_newton_step_limit_fails_the_ring(oracle_mod):
    """NONLIN-TRAN MAXSTEP=1 on a switching ring: Newton fails on the
    switching steps, each failure cuts the step by 8 and after 15
    consecutive failures the transient stops (status -1)."""
    nl = N.ring_oscillator(21, caps=True)
    nl.tran.nl_maxstep = 1
    t, v, st = oracle_mod.Oracle(nl).transient(probes=[nl.names["n1"]])
    assert st["status"] == -1
    assert st["newton_fail"] > 0 and st["rejected"] >= st["newton_fail"]
    assert st["t_final"] < nl.tran.tstop


def test_linear_circuit_converges_in_one_newton_step(oracle_mod):
    nl = N.rc_step()
    nl.tran.nl_maxstep = 1
    t, v, st = oracle_mod.Oracle(nl).transient(probes=[nl.names["out"]])
    assert st["status"] == 0 and st["newton_fail"] == 0


@pytest.mark.parametrize("method", [7, 8], ids=["onestep", "gear"])
@pytest.mark.parametrize("maker,probes", [
    (lambda: N.ring_oscillator(21, caps=True), ["n1", "n11"]),
    (lambda: N.diode_ladder(50, seed=5), ["n1", "n25", "n50"]),
], ids=["ring21", "ladder50"])
def test_replay_reproduces_a_free_run(oracle_mod, maker, probes, method):
    """Replaying a run's own accepted times and integration orders gives the
    same points and values: replay changes which steps are taken, not how a
    step is computed.  (A replayed step's size is recomputed as the
    difference of two recorded times, which may differ from the free run's
    step in the last bit, hence the round-off tolerance.)"""
    nl = maker()
    nl.tran.method = method
    pr = [nl.names[p] for p in probes]
    o = oracle_mod.Oracle(nl)
    t, v, st = o.transient(probes=pr)
    orders = o.recorded_orders(len(t))
    assert st["status"] == 0 and len(orders) == len(t) and orders[0] == 0
    assert set(orders[1:].tolist()) <= {1, 2} and 2 in orders[1:]
    tr, vr, sr = o.replay(t, orders, probes=pr)
    assert sr["status"] == 0 and sr["rejected"] == 0
    assert len(tr) == len(t)
    np.testing.assert_array_equal(tr, t)
    np.testing.assert_array_equal(o.recorded_orders(len(tr)), orders)
    np.testing.assert_allclose(vr, v, rtol=0, atol=1e-9 * np.max(np.abs(v)))


def test_replay_rejects_bad_sequences(oracle_mod):
    o = oracle_mod.Oracle(N.rc_step())
    with pytest.raises(ValueError):
        o.replay([0.0, 1e-9, 1e-9], [0, 1, 1])   # times must increase
    with pytest.raises(ValueError):
        o.replay([0.0, 1e-9, 2e-9], [0, 1, 3])   # orders 1 or 2


def test_standalone_newton_matches_operating_point(oracle_mod):
    """orc_newton with the operating-point rules from x = 0 (initJct on the
    first iteration) converges where the operating point does, to the same
    solution; a one-step limit fails with DampedNewton's -1."""
    nl = N.diode_ladder(30, seed=3)
    o = oracle_mod.Oracle(nl)
    st0, x0, _ = o.dcop()
    st, it, x, _, _ = o.newton(np.zeros(o.n), flags=3, reltol=1e-3, abstol=1e-12, deltaxtol=1.0,
                               rhstol=1e-6, maxstep=200)
    assert st0 > 0 and st > 0 and it >= 2
    np.testing.assert_allclose(x, x0, rtol=1e-9, atol=1e-12)
    st, it, _, _, _ = o.newton(np.zeros(o.n), flags=3, maxstep=1)
    assert st == -1 and it == 1
