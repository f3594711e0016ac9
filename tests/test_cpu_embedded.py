""".EMBEDDEDSAMPLING in the SPICE reader, checked on the CPU with the oracle
as the transient runner: the samples form ONE circuit (one block system with
one step control, src/AnalysisPKG/N_ANP_EmbeddedSampling.C), so every sample
has the same time points; a single sample reproduces the plain deck; the
ensemble file has the reference's layout (hackEnsembleOutput,
N_ANP_EmbeddedSampling.C:1377-1560) and holds the per-point moments."""
import numpy as np
import pytest

from xyce_gb300 import netlist as N
from xyce_gb300 import spice as S

DECK = """Clamped RC embedded sampling
.PARAM rval=1k cval=1n
V1 in 0 SIN(0 2 1MEG)
R1 in out {{rval}}
C1 out 0 {{cval}}
D1 out 0 dclamp
.MODEL dclamp D(IS=1e-14 N=1 RS=10 CJO=1p)
.TRAN 1n 1u 0 10n
.EMBEDDEDSAMPLING param=rval,cval type=normal,uniform means=1k std_deviations=100
+ lower_bounds=0.5n upper_bounds=1.5n
.OPTIONS EMBEDDEDSAMPLES NUMSAMPLES={n} SEED=5 OUTPUTS={{V(OUT)}},{{V(IN,OUT)}} {extra}
.END
"""


def _oracle_runner(oracle_mod):
    def run(nl, probes, cap):
        assert len(set(probes)) == len(probes)  # the C-ABI takes each unknown once
        t, v, st = oracle_mod.Oracle(nl).transient(probes=probes)
        return t, v, st
    return run


def test_embedded_options_parse():
    d = S.parse(DECK.format(n=6, extra="OUTPUT_ALL_SAMPLES=1 OUTPUTFORMAT=TECPLOT SAMPLE_TYPE=MC"))
    e = d.embedded
    assert e["PARAM"] == ["RVAL", "CVAL"] and e["TYPE"] == ["NORMAL", "UNIFORM"]
    assert e["NUMSAMPLES"] == 6 and e["SEED"] == 5 and e["SAMPLE_TYPE"] == "MC"
    assert e["OUTPUTS"] == ["V(OUT)", "V(IN,OUT)"] and e["OUTPUT_ALL_SAMPLES"] and e["OUTPUTFORMAT"] == "TECPLOT"
    with pytest.raises(ValueError):
        S.parse(DECK.format(n=6, extra="PROJECTION_PCE=1"))
    with pytest.raises(ValueError):
        S.parse(DECK.format(n=0, extra=""))


def test_samples_form_one_circuit():
    decks = S.parse_embedded(DECK.format(n=5, extra=""))
    assert len(decks) == 5
    nl, bases = S.ensemble_netlist(decks)
    assert nl.offsets == [0, nl.n] and nl.n_circuits == 1
    assert bases == [k * decks[0].netlist.n for k in range(5)]
    r = [d.netlist.res[0][2] for d in decks]
    assert len(set(r)) == 5  # every sample has its own resistor


def test_one_sample_is_the_plain_deck(oracle_mod):
    decks = S.parse_embedded(DECK.format(n=1, extra=""))
    ens = S.run_embedded(decks, transient=_oracle_runner(oracle_mod))
    nl = decks[0].netlist
    t, v, st = oracle_mod.Oracle(nl).transient(probes=[nl.names["OUT"]])
    np.testing.assert_array_equal(ens.times, t)
    np.testing.assert_array_equal(ens.samples["V(OUT)"][0], v[:, 0])


def test_ensemble_moments_and_file(oracle_mod, tmp_path):
    text = DECK.format(n=8, extra="OUTPUT_ALL_SAMPLES=1")
    decks = S.parse_embedded(text)
    ens = S.run_embedded(decks, transient=_oracle_runner(oracle_mod))
    assert ens.stats["status"] == 0
    vout = ens.samples["V(OUT)"]
    assert vout.shape == (8, len(ens.times))
    # the samples differ (R and C are sampled) on the shared time points
    assert np.max(np.std(vout, axis=0)) > 1e-3
    m = ens.moments("V(IN,OUT)")
    np.testing.assert_allclose(m["mean"], ens.samples["V(IN,OUT)"].mean(axis=0), rtol=1e-14, atol=0)
    np.testing.assert_allclose(m["stddev"], ens.samples["V(IN,OUT)"].std(axis=0), rtol=1e-12, atol=1e-18)
    path = str(tmp_path / "es.cir")
    out = S.write_ensemble(path, decks[0], ens)
    assert out == path + "_ensemble.prn"
    lines = open(out).read().splitlines()
    assert lines[0] == 'TITLE = "embedded sampling output"\tVARIABLES= '
    assert lines[1] == '\t" TIME "' and lines[2] == '\t" V(OUT)_mean"' and lines[8] == '\t" V(OUT)_variance"'
    assert lines[9] == '\t" V(OUT)_0"'
    z = lines.index('ZONE F=POINT  T="Xyce data"')
    rows = [list(map(float, ln.split("\t"))) for ln in lines[z + 1:]]
    assert len(rows) == len(ens.times)
    k = len(rows) // 2
    mo = ens.moments("V(OUT)")
    mean, sd = mo["mean"][k], mo["stddev"][k]
    np.testing.assert_allclose(rows[k][:8], [ens.times[k], mean, mean + sd, mean - sd, mean + 2 * sd,
                                             mean - 2 * sd, sd, mo["variance"][k]], rtol=1e-6, atol=1e-15)
    np.testing.assert_allclose(rows[k][8:16], vout[:, k], rtol=1e-6, atol=1e-15)
