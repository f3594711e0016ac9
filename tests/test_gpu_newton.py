"""xg_newton_solve — DampedNewton on the device for a caller that keeps its own
time integrator — against the oracle's DampedNewton (orc_newton) on the same
coefficients, histories and initial guess.

Tolerances: the DampedNewton status codes and iteration counts agree
exactly; the returned iterates agree within NEWTON_RTOL * max|x| +
NEWTON_ATOL (the same iterations in another summation order and with CUDA's
exp; each iterate then differs from the oracle's by round-off times the
conditioning of the Jacobian).
"""
import numpy as np
import pytest

from xyce_gb300 import netlist as N

pytestmark = pytest.mark.gpu

NEWTON_RTOL, NEWTON_ATOL = 1e-9, 1e-12
DC = dict(reltol=1e-3, abstol=1e-12, deltaxtol=1.0, rhstol=1e-6, maxstep=200)  # N_NLS_Manager.C:1030-1052


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _dev(torch, a):
    return torch.as_tensor(np.ascontiguousarray(a, np.float64), device="cuda:0")


def _solve_both(xg, oracle_mod, torch, nl, x0, x_curr=None, sta_c=None, sto_c=None, qhist0=None, **kw):
    c = xg.Circuit(nl)
    o = oracle_mod.Oracle(nl)
    z = lambda k: np.zeros(max(1, k))
    sta_c = z(o.nsta) if sta_c is None else sta_c
    sto_c = z(o.nsto) if sto_c is None else sto_c
    x = _dev(torch, x0)
    stan, ston = _dev(torch, z(o.nsta)), _dev(torch, z(o.nsto))
    st, it = c.newton_solve(x, _dev(torch, sta_c), _dev(torch, sto_c), stan, ston,
                            x_curr=None if x_curr is None else _dev(torch, x_curr),
                            qhist0=None if qhist0 is None else _dev(torch, qhist0), **kw)
    torch.cuda.synchronize()
    xg_x = x.cpu().numpy()
    c.close()
    ost, oit, ox, osta, osto = o.newton(x0, x_curr=x_curr, sta_curr=sta_c, sto_curr=sto_c, qhist0=qhist0, **kw)
    return (st, it, xg_x), (ost, oit, ox)


def _assert_same(gpu, ref, circuit=0):
    st, it, x = gpu
    ost, oit, ox = ref
    assert (int(st[circuit]), int(it[circuit])) == (ost, oit)
    np.testing.assert_allclose(x, ox, rtol=0, atol=NEWTON_RTOL * np.max(np.abs(ox)) + NEWTON_ATOL)


def test_operating_point_solve_matches_oracle(xg, oracle_mod, torch_cuda):
    """Operating-point rules from x = 0 with initJct: a diode-RC ladder."""
    nl = N.diode_ladder(200, seed=2)
    x0 = np.zeros(nl.n)
    gpu, ref = _solve_both(xg, oracle_mod, torch_cuda, nl, x0, flags=xg.FLAG_DCOP | xg.FLAG_INITJCT, **DC)
    assert ref[0] > 0
    _assert_same(gpu, ref)


def test_operating_point_through_a_near_singular_start(xg, oracle_mod, torch_cuda):
    """A ring with series drain/source resistances at junction initialisation:
    every MOSFET is cut off, so each output node and its two drain' nodes
    reach ground only through gmin-sized conductances (the first Jacobian
    has condition number ~1e12).  The analysis of that matrix exempts those
    columns from the full pivot threshold; on the second iteration the
    devices conduct and the frozen order's pivot there collapses, which must
    still re-pivot (the bounded exemption) rather than be accepted.  Status
    and iteration count equal the oracle's; the converged iterate agrees
    within the conditioning of the first solve (1e-6)."""
    nl = N.ring_oscillator(11, series=True)
    x0 = np.zeros(nl.n)
    gpu, ref = _solve_both(xg, oracle_mod, torch_cuda, nl, x0, flags=xg.FLAG_DCOP | xg.FLAG_INITJCT, **DC)
    assert ref[0] > 0
    st, it, x = gpu
    assert (int(st[0]), int(it[0])) == (ref[0], ref[1])
    np.testing.assert_allclose(x, ref[2], rtol=0, atol=1e-6 * np.max(np.abs(ref[2])))
    c = xg.Circuit(nl)
    xd, itd = c.dcop()
    c.close()
    ost, ox, oit = oracle_mod.Oracle(nl).dcop()
    assert ost > 0 and itd == oit
    np.testing.assert_allclose(xd, ox, rtol=0, atol=1e-6 * np.max(np.abs(ox)))


@pytest.mark.parametrize("maker,caps", [(lambda: N.ring_oscillator(101), False),
                                        (lambda: N.ring_oscillator(21, caps=True), True),
                                        (lambda: N.bsim4_inverter_chain(3), True)],
                         ids=["ring101", "ring21_caps", "b4_chain3"])
def test_backward_euler_step_matches_oracle(xg, oracle_mod, torch_cuda, maker, caps):
    """One backward-Euler step from the operating point, in the OneStep form
    (qscale = 1/h, fscale = 1, qhist0 = Q at the operating point), at a time
    inside the ring's current kick, with the accepted state and store."""
    nl = maker()
    o = oracle_mod.Oracle(nl)
    st0, x_op, _ = o.dcop()
    assert st0 > 0
    ld = o.load(x_op, time=0.0, newton_iter=0, dcop=True)  # the operating point's own state, unlimited
    h, t = 2e-12, 0.3e-9
    gpu, ref = _solve_both(xg, oracle_mod, torch_cuda, nl, x_op, x_curr=x_op, sta_c=ld["sta_next"],
                           sto_c=ld["sto_next"], qhist0=ld["Q"], time=t, qscale=1.0 / h, fscale=1.0,
                           reltol=1e-6, abstol=1e-9)
    assert ref[0] > 0 and ref[1] >= 1
    _assert_same(gpu, ref)


def test_failure_codes_match_oracle(xg, oracle_mod, torch_cuda):
    """A one-iteration limit on the operating point of a ring: DampedNewton's
    -1 (too many steps) on both, after one iteration."""
    nl = N.ring_oscillator(21)
    x0 = np.zeros(nl.n)
    gpu, ref = _solve_both(xg, oracle_mod, torch_cuda, nl, x0, flags=xg.FLAG_DCOP | xg.FLAG_INITJCT,
                           **dict(DC, maxstep=1))
    assert ref[0] == -1 and int(gpu[0][0]) == -1 and int(gpu[1][0]) == ref[1] == 1


def test_batched_circuits_each_match_their_own_solve(xg, oracle_mod, torch_cuda):
    """Three uneven Monte-Carlo rings in one context: each circuit gets its
    own status and iteration count, equal to the oracle's solve of that ring
    alone."""
    torch = torch_cuda
    b = N.monte_carlo_rings(3, 11, 31, seed=8)
    c = xg.Circuit(b)
    nsta, nsto = c.nsta, c.nsto
    x = torch.zeros(b.n, dtype=torch.float64, device="cuda:0")
    z = lambda k: torch.zeros(max(1, k), dtype=torch.float64, device="cuda:0")
    st, it = c.newton_solve(x, z(nsta), z(nsto), z(nsta), z(nsto), flags=xg.FLAG_DCOP | xg.FLAG_INITJCT, **DC)
    torch.cuda.synchronize()
    xs = x.cpu().numpy()
    c.close()
    for k in range(3):
        single = N.extract_circuit(b, k)
        o = oracle_mod.Oracle(single)
        ost, oit, ox, _, _ = o.newton(np.zeros(single.n), flags=3, **DC)
        assert (int(st[k]), int(it[k])) == (ost, oit), k
        seg = xs[b.offsets[k]:b.offsets[k + 1]]
        np.testing.assert_allclose(seg, ox, rtol=0, atol=NEWTON_RTOL * np.max(np.abs(ox)) + NEWTON_ATOL)


def test_update_state_load_type(xg, torch_cuda):
    """updateState with loadType LINEAR evaluates no device (the reference's
    DeviceMaster::updateState skips nonlinear devices for it); NONLINEAR and
    ALL give the same iterate."""
    torch = torch_cuda
    nl = N.ring_oscillator(11)
    c = xg.Circuit(nl)
    x = torch.full((c.n,), 0.9, dtype=torch.float64, device="cuda:0")
    z = lambda k: torch.zeros(max(1, k), dtype=torch.float64, device="cuda:0")
    sta_c, sto_c = z(c.nsta), z(c.nsto)
    outs = {}
    for lt in (xg.LOAD_LINEAR, xg.LOAD_NONLINEAR, xg.LOAD_ALL):
        stan, ston = torch.full_like(sta_c, -7.0), torch.full_like(sto_c, -7.0)
        c.update_state(x, sta_c, sto_c, stan, ston, newton_iter=0, load_type=lt)
        torch.cuda.synchronize()
        outs[lt] = ston.cpu().numpy()
    assert np.all(outs[xg.LOAD_LINEAR] == -7.0)
    assert not np.any(outs[xg.LOAD_ALL] == -7.0)
    np.testing.assert_array_equal(outs[xg.LOAD_NONLINEAR], outs[xg.LOAD_ALL])
    with pytest.raises(xg.XgError):
        c.update_state(x, sta_c, sto_c, sta_c, sto_c, load_type=5)
    c.close()
