"""Re-pivoting one circuit, not the batch.  A frozen pivot that fails the
acceptance threshold parks its circuit's Newton iteration; the host
re-analyses that circuit alone from the parked Jacobian while every other
circuit keeps its pivot rows, factors and results.  A strict threshold
(xg_lu_set_pivot_tolerance) forces many breakdowns; each ring of the batch
must still equal, bit for bit, the same ring run alone with the same
threshold — in both advancing forms."""
import numpy as np
import pytest

from xyce_gb300 import netlist as N

pytestmark = pytest.mark.gpu

PIVOT_TOL = 0.9


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _run(xg, nl, probes, form):
    c = xg.Circuit(nl)
    c.lu_set_pivot_tolerance(PIVOT_TOL)
    c.tran_set_form(form)
    counts, t, v, st = c.transient(probes=probes, cap=50000)
    c.close()
    assert st["status"] == 0, st
    return counts, t, v, st


@pytest.mark.parametrize("form", ["tick_graph", "resident"])
def test_breakdown_repivots_only_its_circuit(xg, torch_cuda, form):
    b = N.monte_carlo_rings(64, 11, 61, seed=17)
    b.tran.tstop = 0.6e-9
    picks = list(range(0, 64, 9))
    probes = [b.names[f"c{k}.n1"] for k in picks]
    fcode = xg.FORM_TICK_GRAPH if form == "tick_graph" else xg.FORM_RESIDENT
    counts, t, v, st = _run(xg, b, probes, fcode)
    assert st["n_analyze"] > 1, "the threshold forced no breakdown"
    assert st["form"] == fcode
    for j, k in enumerate(picks):
        single = N.extract_circuit(b, k)
        c1, t1, v1, s1 = _run(xg, single, [single.names[f"c{k}.n1"]], xg.FORM_AUTO)
        m = int(counts[k])
        assert m == int(c1[0]), (k, m, int(c1[0]))
        np.testing.assert_array_equal(t[k, :m], t1[0, :m], err_msg=f"times of ring {k}")
        np.testing.assert_array_equal(v[k, :m, 0], v1[0, :m, 0], err_msg=f"values of ring {k}")
    print(form, "analyses:", st["n_analyze"])
