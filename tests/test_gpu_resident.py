"""The circuit-resident tick (XG_FORM_RESIDENT: one CTA runs every stage of
every tick of a circuit) against the tick graph (XG_FORM_TICK_GRAPH: 16
kernels per tick over the whole batch).  Each item of every stage is
computed the same way in both, so the runs are equal bit for bit: the same
accepted and rejected steps, Newton iterations, recorded times and values —
across pauses between windows too."""
import numpy as np
import pytest

from xyce_gb300 import netlist as N

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _windows(xg, nl, probes, form, windows, steps):
    c = xg.Circuit(nl)
    c.tran_set_form(form)
    c.tran_start(probes=probes, cap=windows * steps + 64)
    for _ in range(windows):
        c.tran_advance(steps)
    counts, t, v, st = c.tran_results()
    c.tran_end()
    c.close()
    return counts, t, v, st


def _same(a, b):
    ca, ta, va, sa = a
    cb, tb, vb, sb = b
    assert sa["status"] == 0 and sb["status"] == 0
    for k in ("accepted", "rejected", "newton_iters", "newton_fail", "lte_fail", "dcop_iters", "n_analyze"):
        assert sa[k] == sb[k], (k, sa[k], sb[k])
    np.testing.assert_array_equal(ca, cb)
    for i in range(len(ca)):
        m = int(ca[i])
        np.testing.assert_array_equal(ta[i, :m], tb[i, :m], err_msg=f"times of circuit {i}")
        np.testing.assert_array_equal(va[i, :m], vb[i, :m], err_msg=f"values of circuit {i}")


@pytest.mark.parametrize("windows,steps", [(1, 40), (4, 25)])
def test_resident_ticks_equal_tick_graph_on_ring_batch(xg, torch_cuda, windows, steps):
    nl = N.monte_carlo_rings(96, 11, 301, seed=13)
    probes = [nl.names[f"c{i}.n1"] for i in range(0, 96, 5)] + [nl.names["c95.n3"]]
    g = _windows(xg, nl, probes, xg.FORM_TICK_GRAPH, windows, steps)
    r = _windows(xg, nl, probes, xg.FORM_RESIDENT, windows, steps)
    assert g[3]["form"] == xg.FORM_TICK_GRAPH and r[3]["form"] == xg.FORM_RESIDENT
    assert r[3]["circuit_ticks"] > 0
    _same(g, r)


def test_resident_ticks_equal_tick_graph_with_diodes(xg, torch_cuda):
    """A batch mixing diode-RC ladders (diodes, a SIN source) and rings."""
    parts = [N.diode_ladder(8 + (k % 5), seed=k) for k in range(40)] + \
            [N.extract_circuit(N.monte_carlo_rings(30, 11, 41, seed=3), k) for k in range(30)]
    nl = N.batch(parts, label="mixed")
    nl.tran = N.Tran(tstop=0.3e-6, hmax=5e-9)
    probes = [nl.names[f"{k}:n1"] for k in range(0, 40, 7)]
    g = _windows(xg, nl, probes, xg.FORM_TICK_GRAPH, 2, 30)
    r = _windows(xg, nl, probes, xg.FORM_RESIDENT, 2, 30)
    assert r[3]["form"] == xg.FORM_RESIDENT
    _same(g, r)


def test_resident_form_refused_where_it_does_not_apply(xg, torch_cuda):
    """One circuit is not a batch: asking for the resident form is
    XG_ERR_UNSUPPORTED, and AUTO falls back to the tick graph."""
    nl = N.ring_oscillator(21)
    c = xg.Circuit(nl)
    c.tran_set_form(xg.FORM_RESIDENT)
    with pytest.raises(xg.XgError) as e:
        c.tran_start(probes=[nl.names["n1"]], cap=16)
    assert e.value.code == -4
    c.tran_set_form(xg.FORM_AUTO)
    nl.tran.tstop = 0.2e-9
    counts, t, v, st = c.transient(probes=[nl.names["n1"]], cap=4096)
    assert st["status"] == 0 and st["form"] == xg.FORM_TICK_GRAPH
    c.close()


def test_auto_times_the_options_and_keeps_the_bits(xg, torch_cuda):
    """XG_FORM_AUTO on a batch that admits the resident form: the first
    advances time the tick graph and resident CTA sizes (128 and 256
    threads, then on in the direction that got faster), switching between
    them mid-run, and the run still equals the tick graph's bit for bit; the
    stats name the option kept and each timed option's time."""
    nl = N.monte_carlo_rings(96, 11, 301, seed=13)
    probes = [nl.names[f"c{i}.n1"] for i in range(0, 96, 5)]
    g = _windows(xg, nl, probes, xg.FORM_TICK_GRAPH, 7, 20)
    a = _windows(xg, nl, probes, xg.FORM_AUTO, 7, 20)
    _same(g, a)
    st = a[3]
    us = st["option_us_per_iter"]
    timed = [k for k in range(6) if us[k] > 0]
    assert 5 in timed and 2 in timed and 3 in timed, us
    assert len(timed) in (3, 4, 5), us
    best = min(timed, key=lambda k: us[k])
    assert st["option"] == best
    assert st["form"] == (xg.FORM_TICK_GRAPH if best == 5 else xg.FORM_RESIDENT)
    # the forced resident form times CTA sizes only
    r = _windows(xg, nl, probes, xg.FORM_RESIDENT, 6, 20)
    assert 0 <= r[3]["option"] <= 4 and r[3]["option_us_per_iter"][5] == 0
    print("us per circuit Newton iteration:", us, "kept", st["option"])
