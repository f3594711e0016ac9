"""bench.py helpers that need no GPU: clock-sample parsing, peaks, the
one-line JSON contract's static parts."""
import importlib.util
import json
import os

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_clock_summary_median_max_and_reasons(bench, tmp_path):
    p = tmp_path / "clk.csv"
    p.write_text("0, 2070, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active\n"
                 "0, 1980, 2070, 1300.0, 0x4, Not Active, Not Active, Not Active, Active\n"
                 "0, 2070, 2070, 950.0, 0x0, Not Active, Not Active, Not Active, Not Active\n"
                 "1, 500, 2070, 100.0, 0x0, Active, Not Active, Not Active, Not Active\n"
                 "0, [N/A], 2070, 0, 0x0, Not Active, Not Active, Not Active, Not Active\n")
    c = bench._clock_summary(str(p), 0)
    assert c == {"sm_mhz": 2070.0, "sm_max_mhz": 2070.0, "reasons": ["sw_power_cap"]}
    c1 = bench._clock_summary(str(p), 1)
    assert c1["reasons"] == ["hw_slowdown"]


def test_clock_summary_without_samples(bench, tmp_path):
    assert bench._clock_summary(str(tmp_path / "none.csv"), 0)["reasons"] == ["unsampled"]


def test_peaks_read_measured_file_or_fall_back(bench):
    value, kind = bench._peaks()
    assert value > 1000.0 and kind in ("measured", "fallback")
    if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")):
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            assert value == pytest.approx(float(json.load(f)["hbm_gbs"]))


def test_workload_descriptions(bench):
    nl, probes, desc = bench._workload("mc", rings=8)
    assert desc["circuits"] == 8 and desc["workload"] == "monte_carlo_rings_8"
    assert len(probes) == 4 and nl.n_circuits == 8


def test_error_vs_fp64_on_an_oracle_sequence(bench):
    """The bench's error check, fed sequences the oracle itself produced for
    a batch of two diode-RC ladders (driven, stable circuits: a replay whose
    step sizes differ in the last bit stays within round-off): the replay
    reproduces them, and the summary fields add up."""
    import oracle
    from xyce_gb300 import netlist as N
    nl = N.batch([N.diode_ladder(40, seed=2), N.diode_ladder(30, seed=3)])
    nl.tran.tstop = 0.5e-6
    sample = [(0, nl.names["0:n1"]), (0, nl.names["0:n40"]), (1, nl.names["1:n15"])]
    seqs = {}
    for ci in (0, 1):
        sub = N.extract_circuit(nl, ci)
        prs = [pr for c, pr in sample if c == ci]
        o = oracle.Oracle(sub)
        t, v, st = o.transient(probes=[pr - nl.offsets[ci] for pr in prs])
        od = o.recorded_orders(len(t))
        for j, pr in enumerate(prs):
            seqs[(ci, pr)] = (t, od, v[:, j])
    err = bench._error_vs_fp64(nl, sample, seqs, "mc")
    assert "error" not in err, err
    assert err["circuits"] == 2
    assert err["points"] == len(seqs[sample[0]][0]) + len(seqs[sample[2]][0])
    assert err["max_abs_v"] < 1e-9 and err["max_abs_v_exact_window"] <= err["max_abs_v"]


def test_cpu_ring_sample_times_only_the_later_steps(bench):
    """The CPU arm's ring task runs a ring from its operating point and times
    only the accepted steps after the first n_warm (the steps the GPU arm
    times): it returns that many steps and a positive time."""
    from xyce_gb300 import netlist as N
    bench._BATCH = N.monte_carlo_rings(4, 11, 21, seed=7)
    steps, secs = bench._cpu_ring_task((1, 20, 30))
    assert steps == 30 and secs > 0.0
    # no timed steps when the ring stops within the warm-up
    nl = bench._BATCH
    nl.tran.tstop = 1e-12
    steps0, secs0 = bench._cpu_ring_task((1, 20, 30))
    assert steps0 == 0 and secs0 == 0.0
