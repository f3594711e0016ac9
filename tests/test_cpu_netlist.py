"""Seeded generators produce the workloads' shapes and value ranges."""
import numpy as np

from xyce_gb300 import netlist as N


def test_diode_ladder_shape():
    nl = N.diode_ladder(1000, seed=1)
    assert nl.n == 1000 + 1000 + 1  # nodes, diode internal nodes (RS=10), source branch
    assert len(nl.res) == 999 and len(nl.cap) == 1000 and len(nl.diode) == 1000
    r = np.array([x[2] for x in nl.res])
    c = np.array([x[2] for x in nl.cap])
    assert r.min() >= 500 and r.max() <= 2000 and c.min() >= 0.1e-12 and c.max() <= 1e-12
    assert nl.tran.hmax == 10e-9 and nl.tran.abstol == 1e-12


def test_ring_sizes():
    for st in (101, 10001):
        nl = N.ring_oscillator(st)
        assert len(nl.mos1) == 2 * st and nl.n == st + 2
        assert nl.tran.tstop == 20e-9 and nl.tran.hmax == 5e-12


def test_power_grid_shape():
    nl = N.power_grid(20, n_sinks=50, seed=3)
    assert len(nl.res) == 2 * 20 * 19 + 4 and len(nl.cap) == 400 and len(nl.isrc) == 50
    assert len(nl.vsrc) == 4


def test_monte_carlo_uneven_odd_sizes():
    nl = N.monte_carlo_rings(64, 11, 301, seed=4)
    assert nl.n_circuits == 64
    sizes = np.diff(nl.offsets) - 2  # stage nodes = unknowns minus vdd node and branch
    assert np.all(sizes % 2 == 1) and sizes.min() >= 11 and sizes.max() <= 301
    vto_n = np.array([m[4][1] for m in nl.mos1 if m[4][0] > 0])
    assert abs(vto_n.mean() - 0.5) < 0.01 and 0.02 < vto_n.std() < 0.04


def test_generators_are_seeded():
    a = N.monte_carlo_rings(8, seed=4).arrays()
    b = N.monte_carlo_rings(8, seed=4).arrays()
    np.testing.assert_array_equal(a["mos1"][6], b["mos1"][6])
