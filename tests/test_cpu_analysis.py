"""Host LU analysis on CPU (xg_lu_analyze_pattern: no device): the ordering
choice per matrix family, fill against scipy's orderings, schedule shape."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

from xyce_gb300 import netlist as N


def _matrix(oracle_mod, nl):
    o = oracle_mod.Oracle(nl)
    rng = np.random.default_rng(5)
    x = rng.uniform(0.0, 1.0, o.n)
    ld = o.load(x, newton_iter=1, sto_curr=np.zeros(max(1, o.nsto)), sto_prev=np.zeros(max(1, o.nsto)))
    vals = ld["dFdx"] + ld["dQdx"] / 1e-12
    return np.asarray(o.row_ptr, np.int32), np.asarray(o.col_idx, np.int32), np.asarray(vals)


@pytest.fixture(scope="module")
def dag(oracle_mod):
    return _matrix(oracle_mod, N.bsim4_logic_dag(3000, 16, seed=9, tstop=1e-9))


def test_logic_dag_takes_minimum_degree(xg, dag):
    auto = xg.analyze_pattern(*dag)
    nd = xg.analyze_pattern(*dag, ordering=xg.ORDER_ND)
    md = xg.analyze_pattern(*dag, ordering=xg.ORDER_MIN_DEGREE)
    assert auto["ordering"] == "min_degree" and auto["nnz_lu"] == md["nnz_lu"]
    assert md["nnz_lu"] * 3 < nd["nnz_lu"]


def test_minimum_degree_fill_near_scipy_mmd(xg, dag):
    """The restated approximate minimum degree fills about as little as
    SuperLU's multiple minimum degree on A + A^T."""
    rp, ci, v = dag
    n = len(rp) - 1
    A = sp.csr_matrix((v, ci, rp), shape=(n, n)).tocsc()
    lu = spl.splu(A, permc_spec="MMD_AT_PLUS_A", diag_pivot_thresh=0.001,
                  options=dict(SymmetricMode=True))
    ref = lu.L.nnz + lu.U.nnz
    md = xg.analyze_pattern(rp, ci, v, ordering=xg.ORDER_MIN_DEGREE)
    assert md["nnz_lu"] < 2.0 * ref


def test_grid_keeps_nested_dissection(xg, oracle_mod):
    m = _matrix(oracle_mod, N.power_grid(40, 50, seed=2))
    a = xg.analyze_pattern(*m)
    assert a["ordering"] == "nested_dissection"
    assert a["n_top"] >= 64  # the upper separators


def test_ring_batch_groups(xg, oracle_mod):
    """Every ring of a batch factors in its own dependency-closed group,
    with nested dissection (short chains); no top."""
    m = _matrix(oracle_mod, N.monte_carlo_rings(16))
    a = xg.analyze_pattern(*m)
    assert a["ordering"] == "nested_dissection"
    assert a["n_top"] == 0 and a["n_groups"] >= 16


def test_analyze_pattern_rejects_bad_input(xg):
    with pytest.raises(xg.XgError):
        xg.analyze_pattern(np.array([0, 1, 2]), np.array([0, 5]), np.ones(2))  # column out of range


def test_analysis_is_deterministic(xg, oracle_mod):
    """The host analysis orders components on several threads; its result
    does not depend on their timing."""
    m = _matrix(oracle_mod, N.monte_carlo_rings(24))
    runs = [xg.analyze_pattern(*m) for _ in range(3)]
    assert runs[0] == runs[1] == runs[2]
    forced = [xg.analyze_pattern(*m, ordering=o) for o in (xg.ORDER_ND, xg.ORDER_MIN_DEGREE)]
    assert {f["ordering"] for f in forced} == {"nested_dissection", "min_degree"}
