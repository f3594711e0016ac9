"""Netlist decks through the SPICE-subset reader on the GPU path: parity
with the oracle on the same parsed circuit, and the .prn / .mt0 outputs."""
import numpy as np
import pytest

from xyce_gb300 import spice as S

from test_cpu_spice import INV_RING, RC

pytestmark = pytest.mark.gpu

WAVE_RTOL, WAVE_ATOL = 1e-6, 1e-9


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_deck_ring_matches_oracle(xg, oracle_mod, torch_cuda):
    d = S.parse(INV_RING)
    res = S.run(d)
    nl = d.netlist
    to, vo, so = oracle_mod.Oracle(nl).transient(probes=[nl.names["N1"]])
    assert so["status"] == 0 and res.stats["status"] == 0
    assert res.stats["accepted"] == so["accepted"] and len(res.times) == len(to)
    g = np.interp(to, res.times, res.columns["V(N1)"])
    assert np.max(np.abs(g - vo[:, 0])) <= WAVE_RTOL * np.max(np.abs(vo)) + WAVE_ATOL


def test_deck_rc_outputs(xg, torch_cuda, tmp_path):
    path = tmp_path / "rc.cir"
    path.write_text(RC)
    assert S.main([str(path)]) == 0
    names, vals = S.read_prn(str(path) + ".prn")
    assert names == ["Index", "TIME", "V(OUT)", "V(IN,OUT)", "I(V1)"]
    t, vout, vio, i1 = vals[:, 1], vals[:, 2], vals[:, 3], vals[:, 4]
    np.testing.assert_array_equal(vals[:, 0], np.arange(len(t)))
    assert t[0] == 0.0 and t[-1] == pytest.approx(5e-6)
    # KCL at the driven node: the source current is the resistor current
    np.testing.assert_allclose(i1, -vio / 1e3, rtol=1e-8, atol=1e-15)
    # first-order step response after the 1 ns edge (10 ps rise)
    tau = 1e3 * 1e-9
    late = t > 50e-9
    ref = 1.0 - np.exp(-(t[late] - 1e-9 - 5e-12) / tau)
    assert np.max(np.abs(vout[late] - ref)) < 2e-3
    mt = dict(ln.split(" = ") for ln in open(str(path) + ".mt0").read().splitlines())
    assert float(mt["VMAX"]) == pytest.approx(vout.max(), rel=1e-6)
    sel = (t >= 1e-6) & (t <= 4e-6)
    ts, vs = t[sel], vout[sel]
    integ = np.sum(0.5 * np.diff(ts) * (vs[1:] + vs[:-1]))
    assert float(mt["VAVG"]) == pytest.approx(integ / (ts[-1] - ts[0]), rel=1e-6)
