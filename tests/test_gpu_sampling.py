""".SAMPLING on the GPU: a deck's Latin-hypercube samples
(src/AnalysisPKG/N_ANP_Sampling.C) run as the circuits of one batch, each
with its own step control, against the oracle run on each sample alone.

The circuit is driven and stable (an RC low-pass with a clamping diode,
SIN input), so round-off is not amplified: every sampled circuit's
waveform matches the oracle replaying its accepted steps pointwise within
WAVE_RTOL * max|v| + WAVE_ATOL, and each sample's .MEASURE matches the
value computed from the oracle's replay within the same tolerance."""
import numpy as np
import pytest

from xyce_gb300 import netlist as N
from xyce_gb300 import spice as S

pytestmark = pytest.mark.gpu

WAVE_RTOL, WAVE_ATOL = 1e-6, 1e-9
N_SAMPLES = 64
CHECKED = 8

DECK = f"""Clamped RC Monte Carlo
.PARAM rval=1k cval=1n
V1 in 0 SIN(0 2 1MEG)
R1 in out {{rval}}
C1 out 0 {{cval}}
D1 out 0 dclamp
.MODEL dclamp D(IS=1e-14 N=1 RS=10 CJO=1p)
.TRAN 1n 3u 0 10n
.OPTIONS NONLIN-TRAN RELTOL=1e-6 ABSTOL=1e-9
.SAMPLING param=rval,cval type=normal,uniform means=1k std_deviations=100
+ lower_bounds=0.5n upper_bounds=1.5n
.OPTIONS SAMPLES NUMSAMPLES={N_SAMPLES} SEED=11
.PRINT TRAN V(out)
.MEASURE TRAN vmax MAX V(out)
.END
"""


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def test_sampling_deck_matches_oracle_per_sample(xg, oracle_mod, torch_cuda):
    decks = S.parse_sampling(DECK)
    assert len(decks) == N_SAMPLES
    # the reader's own batched run: one Result (columns, measures) per sample
    results = S.run_sweep(decks)
    assert all(r.stats["status"] == 0 for r in results)
    # the same batch through the C-ABI, with the accepted-step sequences
    nl = N.batch([d.netlist for d in decks], label="sampling")
    probes = [nl.names[f"{k}:OUT"] for k in range(N_SAMPLES)]
    c = xg.Circuit(nl)
    c.tran_start(probes=probes, cap=20000)
    c.tran_advance(0)
    counts, t, v, st = c.tran_results()
    orders = c.tran_orders()
    c.tran_end()
    c.close()
    assert st["status"] == 0
    picks = [int(i * N_SAMPLES / CHECKED) for i in range(CHECKED)]
    tasks = []
    for k in picks:
        m = int(counts[k])
        # the reader's run and this one are the same computation
        np.testing.assert_array_equal(results[k].times, t[k, :m])
        np.testing.assert_array_equal(results[k].columns["V(OUT)"], v[k, :m, 0])
        sub = decks[k].netlist
        tasks.append((sub, [sub.names["OUT"]], t[k, :m].copy(), orders[k, :m].copy(), None))
    res = oracle_mod.run_many(tasks)
    for k, (to, vo, so) in zip(picks, res):
        m = int(counts[k])
        assert so["status"] == 0 and len(to) == m
        tol = WAVE_RTOL * float(np.max(np.abs(vo))) + WAVE_ATOL
        err = float(np.max(np.abs(v[k, :m, 0] - vo[:, 0])))
        assert err <= tol, (k, err, tol)
        vmax_oracle = float(np.max(vo[:, 0]))
        assert abs(results[k].measures["VMAX"] - vmax_oracle) <= tol, (k, results[k].measures["VMAX"], vmax_oracle)
    mom = S.sample_moments([r.measures["VMAX"] for r in results])
    assert 0.5 < mom["mean"] < 2.0 and mom["variance"] > 0


ES_DECK = f"""Clamped RC embedded sampling
.PARAM rval=1k cval=1n
V1 in 0 SIN(0 2 1MEG)
R1 in out {{rval}}
C1 out 0 {{cval}}
D1 out 0 dclamp
.MODEL dclamp D(IS=1e-14 N=1 RS=10 CJO=1p)
.TRAN 1n 3u 0 10n
.OPTIONS NONLIN-TRAN RELTOL=1e-6 ABSTOL=1e-9
.EMBEDDEDSAMPLING param=rval,cval type=normal,uniform means=1k std_deviations=100
+ lower_bounds=0.5n upper_bounds=1.5n
.OPTIONS EMBEDDEDSAMPLES NUMSAMPLES=32 SEED=11 OUTPUTS={{V(OUT)}},{{V(IN,OUT)}}
.END
"""


def test_embedded_sampling_block_system_matches_oracle(xg, oracle_mod, torch_cuda):
    """.EMBEDDEDSAMPLING: the 32 samples as ONE circuit (one block system,
    one step control) on the GPU, against the oracle running the same
    union netlist: the same accepted and rejected steps, and every sample's
    outputs within WAVE_RTOL * max|v| + WAVE_ATOL at the oracle's time points."""
    decks = S.parse_embedded(ES_DECK)
    ens = S.run_embedded(decks)

    def oracle_run(nl, probes, cap):
        return oracle_mod.Oracle(nl).transient(probes=probes)
    ref = S.run_embedded(decks, transient=oracle_run)
    assert ens.stats["status"] == 0 and ref.stats["status"] == 0
    assert (ens.stats["accepted"], ens.stats["rejected"]) == (ref.stats["accepted"], ref.stats["rejected"])
    assert len(ens.times) == len(ref.times)
    for var in ("V(OUT)", "V(IN,OUT)"):
        g, r = ens.samples[var], ref.samples[var]
        tol = WAVE_RTOL * np.max(np.abs(r)) + WAVE_ATOL
        gi = np.stack([np.interp(ref.times, ens.times, g[k]) for k in range(g.shape[0])])
        assert np.max(np.abs(gi - r)) <= tol, (var, float(np.max(np.abs(gi - r))), tol)
        np.testing.assert_allclose(ens.moments(var)["stddev"], ref.moments(var)["stddev"], rtol=0,
                                   atol=2 * tol)
