"""Factor reuse with iterative refinement (the reference's LINSOL TYPE=IR,
src/LinearAlgebraServicesPKG/N_LAS_IRSolver.C:428-560) in the oracle.

The first Newton iteration of every solve factors; later iterations solve
with the factors they find, accept at a relative residual of IR_SOLVER_TOL,
refine below IR_MIN_TOL and otherwise refactor.  These tests check that the
transient is the same computation with either linear solver (same accepted
points and Newton iterations, waveforms within the refinement's residual),
that the counters add up, and that the refactor fallback reproduces the
refactor-every-iteration run bit for bit.

Also the elimination order of the oracle's LU: KLU factors each block in
the minimum-degree order its symbolic analysis fixed; the oracle does the
same when asked (use_minimum_degree), with the same answers.
"""
import numpy as np
import pytest

from xyce_gb300 import netlist as N


def _run(oracle_mod, nl, kind, **kw):
    o = oracle_mod.Oracle(nl)
    o.set_linear_solver(kind, **kw)
    o.lu_counts(reset=True)
    probes = list(range(min(o.n, 12)))
    t, v, st = o.transient(probes=probes)
    assert st["status"] == 0
    return t, v, st, o.lu_counts()


def _ring():
    nl = N.ring_oscillator(101)
    nl.tran.tstop = 4e-9
    return nl


@pytest.mark.parametrize("make", [_ring, lambda: N.bsim4_inverter_chain(5)], ids=["mos1_ring", "bsim4_chain"])
def test_reuse_same_transient(oracle_mod, make):
    nl = make()
    t0, v0, s0, c0 = _run(oracle_mod, nl, "klu")
    t1, v1, s1, c1 = _run(oracle_mod, nl, "ir")
    # the same accepted points and Newton iterations ...
    assert len(t0) == len(t1) and s0["newton_iters"] == s1["newton_iters"]
    assert np.max(np.abs(t0 - t1)) <= 1e-9 * nl.tran.tstop  # step sizes see the roundoff
    # ... and waveforms within what a 1e-9 relative residual moves them
    scale = max(1.0, float(np.max(np.abs(v0))))
    assert np.max(np.abs(v0 - v1)) <= 1e-9 * scale
    # every Newton iteration solved once: fresh factors, reused factors as
    # they were, or reused factors after refinement
    assert c0["reuse"] == c0["refined"] == c0["fallback"] == 0
    assert c1["factor"] + c1["reuse"] + c1["refined"] == c0["factor"]
    # reuse saved factorizations; the refined solves took at most 10 steps
    assert c1["factor"] < c0["factor"]
    assert c1["refined"] > 0 and c1["refine_steps"] <= 10 * (c1["refined"] + c1["fallback"])
    assert c1["refine_steps"] >= c1["refined"]


def test_linear_circuit_reuses_without_refinement(oracle_mod):
    """A linear circuit's Jacobian does not change within a Newton solve:
    the second iteration (when there is one) reuses the factors as they are."""
    nl = N.power_grid(12, 10, seed=2)
    nl.tran.tstop = 0.2e-9
    t0, v0, s0, c0 = _run(oracle_mod, nl, "klu")
    t1, v1, s1, c1 = _run(oracle_mod, nl, "ir")
    assert len(t0) == len(t1)
    assert c1["reuse"] > 0 and c1["refined"] == 0 and c1["fallback"] == 0
    assert c1["factor"] + c1["reuse"] == c0["factor"]
    assert np.max(np.abs(v0 - v1)) <= 1e-12 * max(1.0, float(np.max(np.abs(v0))))


def test_fallback_matches_refactoring_bit_for_bit(oracle_mod):
    """With tolerances no reused solve can meet, every reused solve falls
    back to a refactorization: the run is the refactor-every-iteration run."""
    nl = _ring()
    t0, v0, s0, c0 = _run(oracle_mod, nl, "klu")
    t1, v1, s1, c1 = _run(oracle_mod, nl, "ir", ir_tol=1e-300, ir_min_tol=1e-300)
    assert np.array_equal(t0, t1) and np.array_equal(v0, v1)
    assert c1["reuse"] == c1["refined"] == c1["refine_steps"] == 0
    assert c1["factor"] == c0["factor"] and c1["fallback"] > 0


def test_refinement_disabled_below_min_tol(oracle_mod):
    """IR_MIN_TOL below every stale residual: no refinement, only fallbacks
    (and reuse where the stale factors already meet IR_SOLVER_TOL)."""
    nl = _ring()
    _, _, _, c = _run(oracle_mod, nl, "ir", ir_min_tol=1e-300)
    assert c["refined"] == 0 and c["refine_steps"] == 0 and c["fallback"] > 0


def test_linear_solver_options_checked(oracle_mod):
    o = oracle_mod.Oracle(N.rc_step())
    with pytest.raises(KeyError):
        o.set_linear_solver("gmres")
    with pytest.raises(ValueError):
        o.set_linear_solver("ir", ir_tol=0.0)
    with pytest.raises(ValueError):
        o.set_linear_solver("ir", ir_min_tol=-1.0)


# ---- elimination order (KLU's symbolic ordering) ---------------------------

def test_min_degree_order_same_transient(oracle_mod):
    """Factoring P A P^T in a minimum-degree order changes only the roundoff:
    the same accepted points and Newton iterations as the natural order."""
    nl = N.bsim4_logic_dag(600, 8, seed=3, tstop=0.3e-9)
    runs = []
    for md in (False, True):
        o = oracle_mod.Oracle(nl)
        if md:
            o.use_minimum_degree()
        t, v, st = o.transient(probes=list(range(10)))
        assert st["status"] == 0
        runs.append((t, v, st))
    (t0, v0, s0), (t1, v1, s1) = runs
    assert len(t0) == len(t1) and s0["newton_iters"] == s1["newton_iters"]
    assert np.max(np.abs(t0 - t1)) <= 1e-9 * nl.tran.tstop
    assert np.max(np.abs(v0 - v1)) <= 1e-10


def test_min_degree_order_solves(oracle_mod):
    """The ordered LU solves the same systems (scipy's solve checks the
    answer), and the order is a permutation of the unknowns."""
    nl = N.power_grid(20, 10, seed=1)
    o = oracle_mod.Oracle(nl)
    perm = oracle_mod.min_degree_order(o.row_ptr, o.col_idx)
    assert sorted(perm.tolist()) == list(range(o.n))
    rng = np.random.default_rng(2)
    vals = rng.uniform(-1, 1, o.nnz)
    diag = np.array([p for i in range(o.n) for p in range(o.row_ptr[i], o.row_ptr[i + 1])
                     if o.col_idx[p] == i])
    vals[diag] += 8.0
    b = rng.uniform(-1, 1, o.n)
    x0 = o.lu_solve(vals, b)
    o.set_order(perm)
    x1 = o.lu_solve(vals, b)
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    A = sp.csr_matrix((vals, o.col_idx, o.row_ptr), shape=(o.n, o.n))
    ref = spl.spsolve(A.tocsc(), b)
    assert np.allclose(x0, ref, rtol=1e-11, atol=1e-12) and np.allclose(x1, ref, rtol=1e-11, atol=1e-12)
    o.set_order(None)  # back to the natural order
    assert np.array_equal(o.lu_solve(vals, b), x0)


def test_set_order_rejects_non_permutations(oracle_mod):
    o = oracle_mod.Oracle(N.rc_step())
    with pytest.raises(ValueError):
        o.set_order(np.zeros(o.n, np.int32))  # repeated unknown
    with pytest.raises(ValueError):
        o.set_order(np.arange(o.n + 1))  # wrong length
    with pytest.raises(ValueError):
        o.set_order(np.arange(o.n)[::-1] + 1)  # out of range
