"""Waveform parity on the benchmark configurations, at identical time points.

Two correct integrators whose round-off differs (CUDA's exp against glibc's,
another LU elimination order) can, when run freely, accept different step
sequences: a step whose error estimate lies within round-off of the
acceptance threshold goes one way in one run and the other way in the other.
So every GPU run here is compared with the oracle REPLAYING the GPU's
accepted step sequence — its times and integration orders, recorded by
xg_tran_orders — which makes the oracle compute the same steps (histories,
coefficients, predictors, breakpoints and Newton solves as in a free run).

Pointwise criterion:  |v_gpu - v_oracle| <= WAVE_RTOL * max|v_oracle| + WAVE_ATOL
with WAVE_RTOL = 1e-6 (the reltol of the target forms) and WAVE_ATOL = 1e-9 V.

Round-off floor.  A ring oscillator kicked out of its metastable operating
point amplifies round-off: every inverter starts at high gain.  The oracle
replaying the same accepted steps with every time point moved by one unit
in the last place — a perturbation of the size of the GPU's own round-off
(CUDA's exp, another summation order) — agrees with the unperturbed replay
pointwise only for the first ~100 ps and then differs by up to 0.07 V over
2 ns: a sub-picosecond shift of the switching instants.  (The LU elimination
order is not such a perturbation here: on these rings every order gives the
same bits to 1e-22.)  Where the configuration is such a ring, that
difference is the reference's own round-off floor.  The GPU must then meet
the pointwise criterion on every point up to the first one where the floor
exceeds FLOOR_NEGLIGIBLE * max|v| (the floor is negligible there, so the
comparison is exact), and on the whole run stay within max(pointwise
tolerance, FLOOR_FACTOR * the largest floor).  Driven, stable circuits (the
diode ladder, the grid, the logic DAG) and the first 200 steps of the long
ring do not amplify round-off and meet the pointwise criterion everywhere.

Newton runs at RELTOL 1e-6 / ABSTOL 1e-9 so that a Newton solve that takes
one iteration more in one run than in the other still lands within the
tolerance; the TIMEINT options are each configuration's own, except the
Monte-Carlo rings, which also run TIMEINT RELTOL 1e-6.  The oracle's free
run is compared too: its accepted-step count must agree with the GPU's
within FREE_COUNT_TOL (a ring's free runs whose round-off differs follow
trajectories a few picoseconds apart and take a few percent more or fewer
steps).

Configurations (full size unless stated): the 1,000-node diode-RC ladder
(5 us); 32 rings drawn from the 4,096-ring Monte-Carlo batch of the bench,
run as one batch (2 ns); the 10,001-stage ring (first 200 steps); a 200 x
200 power grid with 320 sinks (first 40 steps); a 5,000-transistor BSIM4
logic DAG (first 100 steps).
"""
import numpy as np
import pytest

from xyce_gb300 import netlist as N

pytestmark = pytest.mark.gpu

WAVE_RTOL, WAVE_ATOL = 1e-6, 1e-9
FREE_COUNT_TOL = 0.05
FLOOR_NEGLIGIBLE = 1e-9
FLOOR_FACTOR = 30.0
MIN_EXACT_POINTS = 500


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _tight_newton(tran):
    tran.nl_reltol, tran.nl_abstol = 1e-6, 1e-9
    return tran


def _gpu_run(xg, nl, probes, cap):
    """Transient on the GPU; per circuit: (times, orders, values) of its points."""
    c = xg.Circuit(nl)
    c.tran_start(probes=probes, cap=cap)
    c.tran_advance(0)
    counts, t, v, st = c.tran_results()
    orders = c.tran_orders()
    c.tran_end()
    c.close()
    assert st["status"] == 0, st
    out = []
    for k in range(len(counts)):
        m = int(counts[k])
        assert m < cap, "recording buffer too small"
        out.append((t[k, :m].copy(), orders[k, :m].copy(), v[k, :m].copy()))
    return out, st


def _replayed(name, t_gpu, res):
    t_o, v_o, st_o = res
    assert st_o["status"] == 0, (name, st_o)
    assert len(t_o) == len(t_gpu), (name, len(t_o), len(t_gpu))
    np.testing.assert_array_equal(t_o, t_gpu)
    return v_o


def _check(name, t_gpu, v_gpu, ref, alt=None):
    """ref: the oracle's replay; alt: the same replay with every time moved
    by one ulp (None for circuits that do not amplify round-off).  Returns
    the largest |dv|, the number of exactly compared points and the floor."""
    v_ref = _replayed(name, t_gpu, ref)
    vmax = float(np.max(np.abs(v_ref)))
    tol = WAVE_RTOL * vmax + WAVE_ATOL
    err = np.max(np.abs(v_gpu[:, : v_ref.shape[1]] - v_ref), axis=1)
    if alt is None:
        assert float(err.max()) <= tol, (name, float(err.max()), tol)
        return float(err.max()), len(err), 0.0
    t_alt, v_alt, st_alt = alt
    assert st_alt["status"] == 0 and len(t_alt) == len(t_gpu), (name, "floor replay", st_alt)
    floor = np.max(np.abs(v_alt - v_ref), axis=1)
    above = np.nonzero(floor > FLOOR_NEGLIGIBLE * vmax)[0]
    exact = int(above[0]) if len(above) else len(floor)
    assert exact >= min(MIN_EXACT_POINTS, len(floor)), (name, exact)
    worst_exact = float(err[:exact].max())
    assert worst_exact <= tol, (name, "exact window", exact, worst_exact, tol)
    bound = max(tol, FLOOR_FACTOR * float(floor.max()))
    assert float(err.max()) <= bound, (name, float(err.max()), float(floor.max()))
    return float(err.max()), exact, float(floor.max())


def test_monte_carlo_batch_rings_match_oracle_replay(xg, oracle_mod, torch_cuda):
    """32 rings of the bench's 4,096-ring batch, run as one batch on the GPU
    (each circuit keeps its own step control) at TIMEINT and Newton RELTOL
    1e-6; every ring is replayed alone by the oracle, as recorded and (the
    round-off floor) with its times moved by one ulp."""
    full = N.monte_carlo_rings(4096)
    picks = [int(i * 4096 / 32) + (i % 7) for i in range(32)]
    rings = [N.extract_circuit(full, ci) for ci in picks]
    b = N.batch(rings, label="mc32")
    b.tran = _tight_newton(N.Tran(tstop=2e-9, hmax=5e-12, reltol=1e-6, abstol=1e-9))
    local_probes = []
    probes = []
    for k, (ci, r) in enumerate(zip(picks, rings)):
        stages = len(r.mos1) // 2
        names = [f"c{ci}.n1", f"c{ci}.n{stages // 2 + 1}"]
        local_probes.append([r.names[nm] for nm in names])
        probes += [b.names[f"{k}:{nm}"] for nm in names]
    runs, st = _gpu_run(xg, b, probes, cap=150000)
    tasks = []
    for k, r in enumerate(rings):
        r.tran = b.tran
        t, o, _ = runs[k]
        tasks += [(r, local_probes[k], t, o, None), (r, local_probes[k], t, o, "ulp"),
                  (r, local_probes[k], None, None, None)]
    res = oracle_mod.run_many(tasks)
    worst, exact_min, count_dev = 0.0, None, []
    for k in range(len(rings)):
        t, o, v = runs[k]
        assert set(np.unique(o[1:]).tolist()) <= {1, 2}
        e, exact, _ = _check(f"ring {picks[k]}", t, v, res[3 * k], res[3 * k + 1])
        worst = max(worst, e)
        exact_min = exact if exact_min is None else min(exact_min, exact)
        count_dev.append(abs(len(res[3 * k + 2][0]) - len(t)) / len(t))
    assert max(count_dev) <= FREE_COUNT_TOL, count_dev
    print(f"mc32: {st['accepted']} accepted steps, >= {exact_min} points per ring compared exactly, "
          f"max |dv| vs replayed oracle {worst:.3e}")


_CONFIGS = {
    # name: (netlist maker, probe names, max accepted steps (0: to tstop), oracle elimination
    #        order, round-off-floor replay (None: the circuit does not amplify round-off))
    "c1_diode_ladder_1000": (lambda: N.diode_ladder(1000, seed=1), ["n1", "n500", "n1000"], 0, "md", None),
    "c2_ring_10001": (lambda: N.ring_oscillator(10001), ["n1", "n5000", "n10001"], 200, None, "ulp"),
    "c3_power_grid_200": (lambda: N.power_grid(200, 320, seed=3), ["center"], 40, "md", None),
    "c5_bsim4_dag_5000": (lambda: N.bsim4_logic_dag(5000, 16, seed=7, tstop=2e-9), ["g10", "g200", "g600"],
                          100, "md", None),
}


@pytest.mark.parametrize("name", sorted(_CONFIGS))
def test_benchmark_config_matches_oracle_replay(xg, oracle_mod, torch_cuda, name):
    maker, pnames, max_steps, order, alt_order = _CONFIGS[name]
    nl = maker()
    _tight_newton(nl.tran)
    nl.tran.max_steps = max_steps
    probes = [nl.names[p] for p in pnames]
    runs, st = _gpu_run(xg, nl, probes, cap=(max_steps + 16) if max_steps else 200000)
    t, o, v = runs[0]
    tasks = [(nl, probes, t, o, order), (nl, probes, None, None, order)]
    if alt_order:
        tasks.append((nl, probes, t, o, alt_order))
    res = oracle_mod.run_many(tasks)
    err, exact, floor = _check(name, t, v, res[0], res[2] if alt_order else None)
    free = res[1]
    assert free[2]["status"] == 0
    assert abs(len(free[0]) - len(t)) <= FREE_COUNT_TOL * len(t), (len(free[0]), len(t))
    print(f"{name}: {len(t) - 1} accepted steps, {exact} compared exactly, max |dv| vs replayed oracle "
          f"{err:.3e} (round-off floor {floor:.3e})")
