"""The host LU analysis (xyce_gb300/csrc/xg_symbolic.cpp) on the CPU, through
tests/lu_analysis_probe.cpp: the factors in the analysed order reconstruct
the permuted matrix; the analysis of a matrix whose static pivots are
cancelled by elimination (a ring with series drain/source resistance at its
operating point) falls back to threshold partial pivoting and leaves no
column below the device's pivot threshold; an order frozen on one matrix is
tested, as the device does, on the next one; the factor and L-solve
schedules (hubs, dependency-closed groups, the top) respect every
dependency."""
import os
import shutil
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

from xyce_gb300 import netlist as N

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
RUNTIME_PIVOT_TOL = 1e-2  # kRuntimePivotTol, xyce_gb300/csrc/xg_internal.h


def _cuda_include():
    for base in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if base and os.path.exists(os.path.join(base, "include", "cuda_runtime.h")):
            return os.path.join(base, "include")
    return None


@pytest.fixture(scope="module")
def probe(tmp_path_factory):
    inc = _cuda_include()
    if shutil.which("g++") is None or inc is None:
        pytest.skip("g++ or the CUDA headers are missing")
    exe = str(tmp_path_factory.mktemp("probe") / "lu_analysis_probe")
    subprocess.run(["g++", "-O2", "-std=c++17", "-w", f"-I{inc}", "-o", exe,
                    os.path.join(HERE, "lu_analysis_probe.cpp"),
                    os.path.join(ROOT, "xyce_gb300", "csrc", "xg_symbolic.cpp"), "-lpthread"],
                   check=True, capture_output=True)
    return exe


def _run(probe, tmp_path, rp, ci, va, vb=None):
    vb = va if vb is None else vb
    path = str(tmp_path / "m.bin")
    with open(path, "wb") as f:
        np.array([len(rp) - 1, len(ci)], np.int32).tofile(f)
        np.asarray(rp, np.int32).tofile(f)
        np.asarray(ci, np.int32).tofile(f)
        np.asarray(va, np.float64).tofile(f)
        np.asarray(vb, np.float64).tofile(f)
    out = subprocess.run([probe, path], check=True, capture_output=True, text=True).stdout.split()
    rc, exempt = int(out[0]), int(out[1])
    # every analysis' factor and L-solve schedules respect the dependencies
    assert rc != 0 or (out[5], out[6]) == ("1", "1"), out
    _run.layout = (int(out[7]), int(out[8]))  # factor hubs, factor top items
    return rc, exempt, float(out[2]), float(out[3]), float(out[4])


def _jacobians(oracle_mod, nl):
    """The operating point's junction-initialisation Jacobian and its
    converged one (dFdx), on the oracle's CSR pattern."""
    o = oracle_mod.Oracle(nl)
    init = o.load(np.zeros(o.n), dcop=True, newton_iter=0, init_jct=True)["dFdx"]
    st, x, it = o.dcop()
    assert st > 0
    conv = o.load(x, dcop=True, newton_iter=1)["dFdx"]
    tran = conv + o.load(x, dcop=True, newton_iter=1)["dQdx"] / 5e-12
    return o, init, conv, tran


def test_cancelled_static_pivots_fall_back_to_partial_pivoting(probe, oracle_mod, tmp_path):
    o, init, conv, _ = _jacobians(oracle_mod, N.ring_oscillator(11, series=True))
    # the order analysed at junction initialisation fails on the converged
    # matrix (the device flags that and re-analyses) ...
    rc, ex, ra, rb, err = _run(probe, tmp_path, o.row_ptr, o.col_idx, init, conv)
    assert rc == 0 and ra >= RUNTIME_PIVOT_TOL and rb < 1e-6
    # ... and the re-analysis of the converged matrix pivots it cleanly
    rc, ex, ra, rb, err = _run(probe, tmp_path, o.row_ptr, o.col_idx, conv)
    assert rc == 0 and ex == 0 and ra >= RUNTIME_PIVOT_TOL and err < 1e-12


def test_fallback_keeps_the_order_it_pivoted_in(probe, oracle_mod, tmp_path):
    """An RLC ladder's operating point (inductors are shorts: a branch row
    with no diagonal): the static pivots leave columns below the threshold;
    the fallback's rows, kept together with the order they were chosen in,
    reproduce threshold partial pivoting, so no column stays exempt."""
    o, init, conv, tran = _jacobians(oracle_mod, N.rlc_ladder(20, seed=1))
    rc, ex, ra, rb, err = _run(probe, tmp_path, o.row_ptr, o.col_idx, conv)
    assert rc == 0 and ex == 0 and ra >= 0.1 and err < 1e-12


@pytest.mark.parametrize("maker", [lambda: N.ring_oscillator(31), lambda: N.ring_oscillator(21, caps=True),
                                   lambda: N.diode_ladder(40, seed=2), lambda: N.power_grid(8, 12, seed=3),
                                   lambda: N.bsim4_logic_dag(120, 6, seed=3, tstop=0.5e-9),
                                   lambda: N.ring_oscillator(11, caps=True, series=True)],
                         ids=["ring31", "ring21_caps", "diode40", "grid8x12", "b4dag120", "ring11_caps_rs"])
def test_analysed_factors_reconstruct_the_matrix(probe, oracle_mod, tmp_path, maker):
    o, init, conv, tran = _jacobians(oracle_mod, maker())
    for vals in (init, conv, tran):
        rc, ex, ra, rb, err = _run(probe, tmp_path, o.row_ptr, o.col_idx, vals)
        assert rc == 0 and ex == 0 and ra >= RUNTIME_PIVOT_TOL and err < 1e-12


@pytest.mark.parametrize("maker", [lambda: N.power_grid(30, 30, seed=4), lambda: N.diode_ladder(300, seed=1)],
                         ids=["grid30", "diode300"])
def test_schedules_with_a_top(probe, oracle_mod, tmp_path, maker):
    """Circuits larger than one dependency-closed group (512 items): the
    columns that depend on several groups form the top (30 items on a
    30 x 30 grid, 2 on a 300-node diode ladder).  The schedules still
    respect every dependency (checked inside _run)."""
    o, init, conv, tran = _jacobians(oracle_mod, maker())
    rc, ex, ra, rb, err = _run(probe, tmp_path, o.row_ptr, o.col_idx, tran)
    hubs, top = _run.layout
    assert rc == 0 and err < 1e-12 and top > 0, _run.layout


@pytest.mark.parametrize("seed", range(6))
def test_random_permuted_matrices(probe, tmp_path, seed):
    """Random sparse matrices whose large entries sit on a random row
    permutation (the row matching has to find it), plus small off-diagonal
    couplings."""
    rng = np.random.default_rng(seed)
    n = 60
    perm = rng.permutation(n)
    big = sp.csr_matrix((rng.uniform(1.0, 2.0, n) * rng.choice([-1, 1], n), (perm, np.arange(n))), shape=(n, n))
    small = sp.random(n, n, density=0.05, random_state=np.random.RandomState(seed), format="csr") * 0.05
    A = (big + small).tocsr()
    A.sort_indices()
    rc, ex, ra, rb, err = _run(probe, tmp_path, A.indptr, A.indices, A.data)
    assert rc == 0 and err < 1e-12
    assert ra >= RUNTIME_PIVOT_TOL or ex > 0
