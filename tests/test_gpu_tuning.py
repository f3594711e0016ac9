"""Launch-shape tuner of the LU sweeps (xg_lu_set_tuning): every shape it
tries computes the same bits, so a run with the timed choice equals a run
with the closed-form choice exactly — the same accepted steps, Newton
iterations and waveforms, bit for bit — and a second context with the same
analysis takes the choice from the cache."""
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


_CASES = {
    "mc64": (lambda: N.monte_carlo_rings(64, seed=11), lambda nl: [nl.names[f"c{i}.n1"] for i in (0, 31, 63)],
             0.5e-9),
    # enough groups for single-thread factor columns, and packs of supply
    # columns that mix circuits
    "mc1024": (lambda: N.monte_carlo_rings(1024, seed=11),
               lambda nl: [nl.names[f"c{i}.n1"] for i in range(0, 1024, 97)], 0.3e-9),
    "ring101": (lambda: N.ring_oscillator(101), lambda nl: [nl.names["n1"], nl.names["n50"]], 2e-9),
    "grid40": (lambda: N.power_grid(40, 50, seed=2), lambda nl: [nl.names["center"]], 0.2e-9),
    "b4dag3000": (lambda: N.bsim4_logic_dag(3000, 16, seed=9, tstop=1e-9), lambda nl: [nl.names["g40"]], 0.3e-9),
}


def _run(xg, nl, probes, mode):
    c = xg.Circuit(nl)
    c.lu_set_tuning(mode)
    c.tran_start(probes=probes, cap=200000)
    c.tran_advance(0)
    counts, t, v, st = c.tran_results()
    tuning = c.lu_tuning()
    c.tran_end()
    c.close()
    return counts, t, v, st, tuning


@pytest.mark.parametrize("name", sorted(_CASES))
def test_timed_launch_shapes_give_identical_runs(xg, torch_cuda, name):
    make, probes_of, tstop = _CASES[name]
    nl = make()
    nl.tran.tstop = tstop
    probes = probes_of(nl)
    c0, t0, v0, s0, tm = _run(xg, nl, probes, xg.TUNE_MODEL)
    c1, t1, v1, s1, tt = _run(xg, nl, probes, xg.TUNE_TIMED)
    assert s0["status"] == 0 and s1["status"] == 0
    for k in ("accepted", "rejected", "newton_iters", "n_analyze"):
        assert s0[k] == s1[k], (k, s0[k], s1[k])
    np.testing.assert_array_equal(c0, c1)
    np.testing.assert_array_equal(t0, t1)
    np.testing.assert_array_equal(v0, v1)
    assert tm["mode"] == xg.TUNE_MODEL and tt["mode"] == xg.TUNE_TIMED
    for key in ("factor_threads", "lsolve_threads", "usolve_threads"):
        assert tt[key] in (64, 128, 256, 512)
    # the timed choice is never slower than the model's in the trials
    assert tt["factor_us"] <= tt["model_factor_us"] or tt["from_cache"]
    assert tt["solve_us"] <= tt["model_solve_us"] or tt["from_cache"]
    print(name, {k: tt[k] for k in tt})


def test_tuning_is_cached_per_analysis(xg, torch_cuda):
    """A second context with the same circuit reuses the timed choice."""
    torch = torch_cuda
    nl = N.monte_carlo_rings(16, seed=12)
    import oracle
    o = oracle.Oracle(nl)
    _, x0, _ = o.dcop()
    ld = o.load(x0)
    vals = torch.as_tensor(ld["dFdx"] + ld["dQdx"] / 1e-12, device="cuda:0")
    picks = []
    for _ in range(2):
        c = xg.Circuit(nl)
        c.lu_analyze(vals)
        picks.append(c.lu_tuning())
        c.close()
    assert picks[0]["from_cache"] == 0 and picks[1]["from_cache"] == 1
    for k in ("factor_threads", "factor_meta", "lsolve_threads", "usolve_threads"):
        assert picks[0][k] == picks[1][k]


_SHAPE_CASES = {
    "mc1024": (lambda: N.monte_carlo_rings(1024, seed=11), lambda nl: [nl.names[f"c{i}.n1"] for i in range(0, 1024, 97)],
               0.2e-9),
    "b4dag3000": (lambda: N.bsim4_logic_dag(3000, 16, seed=9, tstop=1e-9), lambda nl: [nl.names["g40"]], 0.2e-9),
    "grid40": (lambda: N.power_grid(40, 50, seed=2), lambda nl: [nl.names["center"]], 0.1e-9),
}


@pytest.mark.parametrize("name", sorted(_SHAPE_CASES))
def test_every_launch_shape_gives_identical_runs(xg, torch_cuda, name):
    """Each candidate shape the tuner may pick, pinned with xg_lu_set_shapes
    (the factorization at every CTA size with and without its metadata
    staged, then each solve at every CTA size), runs the transient to the
    same bits as the closed-form shapes."""
    make, probes_of, tstop = _SHAPE_CASES[name]
    nl = make()
    nl.tran.tstop = tstop
    probes = probes_of(nl)
    ref = _run(xg, nl, probes, xg.TUNE_MODEL)
    shapes = [(s, m, 0, 0) for s in (64, 128, 256, 512) for m in (0, 1)]
    shapes += [(0, -1, s, 0) for s in (64, 128, 256, 512)] + [(0, -1, 0, s) for s in (64, 128, 256, 512)]
    for sh in shapes:
        c = xg.Circuit(nl)
        c.lu_set_shapes(*sh)
        c.tran_start(probes=probes, cap=200000)
        c.tran_advance(0)
        counts, t, v, st = c.tran_results()
        tun = c.lu_tuning()
        c.tran_end()
        c.close()
        assert tun["mode"] == xg.TUNE_FIXED
        assert st["status"] == 0, (sh, st["status"])
        for k in ("accepted", "rejected", "newton_iters", "n_analyze"):
            assert st[k] == ref[3][k], (sh, k, st[k], ref[3][k])
        np.testing.assert_array_equal(counts, ref[0], err_msg=str(sh))
        np.testing.assert_array_equal(t, ref[1], err_msg=str(sh))
        np.testing.assert_array_equal(v, ref[2], err_msg=str(sh))
