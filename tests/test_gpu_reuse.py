"""Factor reuse (xg_lu_set_reuse): a circuit without nonlinear devices whose
Jacobian coefficients did not change since its last factorization skips the
refactorization.  Its Jacobian is then the same bit for bit, so runs with and
without reuse are identical — step counts, times and values — while the
reusing run counts the skipped factorizations."""
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


def _run(xg, nl, probes, reuse, form=None):
    c = xg.Circuit(nl)
    c.lu_set_reuse(reuse)
    if form is not None:
        c.tran_set_form(form)
    counts, t, v, st = c.transient(probes=probes, cap=100000)
    c.close()
    return counts, t, v, st


@pytest.mark.parametrize("name", ["grid", "rc_batch_with_rings"])
def test_reuse_gives_identical_runs(xg, torch_cuda, name):
    if name == "grid":
        nl = N.power_grid(24, 30, seed=4)
        nl.tran.tstop = 0.3e-9
        probes = [nl.names["center"]]
    else:
        parts = [N.rc_step(r=1e3 * (1 + k % 7), c=1e-12 * (1 + k % 3), tstop=20e-9) for k in range(70)]
        parts += [N.extract_circuit(N.monte_carlo_rings(6, 11, 31, seed=5), k) for k in range(6)]
        nl = N.batch(parts, label="rc_rings")
        nl.tran = N.Tran(tstop=2e-9, hmax=5e-12)
        probes = [nl.names[f"{k}:out"] for k in range(0, 70, 9)] + [nl.names["72:c2.n1"]]
    a = _run(xg, nl, probes, False)
    b = _run(xg, nl, probes, True)
    assert a[3]["status"] == 0 and b[3]["status"] == 0
    for k in ("accepted", "rejected", "newton_iters"):
        assert a[3][k] == b[3][k], k
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_array_equal(a[2], b[2])
    assert a[3]["factor_skips"] == 0 and b[3]["factor_skips"] > 0
    print(name, "skipped", b[3]["factor_skips"], "of", b[3]["newton_iters"], "factorizations")
