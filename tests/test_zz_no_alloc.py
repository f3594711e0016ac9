"""xg_lu_solve_noalloc: the allocation-free triangular solve.

Some callers cannot call cudaMalloc (their device memory is owned by another
allocator, or their loop must not block on the CUDA allocator).  For them
the solve keeps its scratch vector in a static device array instead of
allocated memory.  These tests call it through the C-ABI and check it
against xg_lu_solve, the entry point it is a variant of, on two calls in a
row (the scratch keeps the previous call's contents: nothing may leak from
one call into the next), and check that oversized systems are rejected.

This file is collected last so that a run stopping at the first failure has
already run every other test.
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spl

from xyce_gb300 import netlist as N

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # same kernels, different scratch: agreement to round-off


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _t(torch, a):
    return torch.as_tensor(np.ascontiguousarray(a, np.float64), device="cuda:0")


_CASES = {
    # a ring: the whole system factors in dependency-closed groups
    "ring101": dict(make=lambda: N.ring_oscillator(101), sched=None),
    # a grid whose upper separators form a large top, with the tops of the
    # factorization and of both solves forced to one launch per level
    # (k_toplv_*, k_lsolve_level, k_usolve_level read and write the scratch)
    "grid40_levels": dict(make=lambda: N.power_grid(40, 50, seed=2), sched=(-1, 2, 2)),
}


@pytest.mark.parametrize("prec", ["fp64", "fp32_ir"])
@pytest.mark.parametrize("case", sorted(_CASES))
def test_noalloc_solve_matches_allocated_solve(xg, oracle_mod, torch_cuda, case, prec):
    """Two calls in a row, each against xg_lu_solve on the same factors, in
    FP64 and in the FP32-factor + FP64-refinement form (whose refinement
    solves also run on the static scratch)."""
    torch = torch_cuda
    spec = _CASES[case]
    nl = spec["make"]()
    c = xg.Circuit(nl)
    if spec["sched"]:
        c.lu_set_schedule(*spec["sched"])
    if prec == "fp32_ir":
        c.lu_set_precision(xg.PREC_FP32_IR, 2)
    o = oracle_mod.Oracle(nl)
    rng = np.random.default_rng(17)
    if case == "ring101":
        _, x0, _ = o.dcop()
        ld = o.load(x0)
    else:
        ld = o.load(rng.uniform(0.0, 1.0, o.n), newton_iter=1)
    vals = ld["dFdx"] + ld["dQdx"] / 1e-12
    v = _t(torch, vals)
    c.lu_analyze(v)
    c.lu_factor(v)
    if spec["sched"]:
        info = c.lu_info()
        assert info["factor_top"] == "levels" and info["solve_top"] == "levels", info
    A = sp.csr_matrix((vals, o.col_idx, o.row_ptr), shape=(o.n, o.n))
    for call in range(2):
        b = _t(torch, rng.standard_normal(o.n) * (10.0 ** call))
        x_ref = torch.zeros_like(b)
        x_na = torch.full_like(b, np.nan)
        c.lu_solve(b, x_ref)
        c.lu_solve_noalloc(b, x_na)
        torch.cuda.synchronize()
        xr, xn = x_ref.cpu().numpy(), x_na.cpu().numpy()
        np.testing.assert_allclose(xn, xr, rtol=RTOL, atol=RTOL * np.max(np.abs(xr)))
        xs = spl.spsolve(A.tocsc(), b.cpu().numpy())
        np.testing.assert_allclose(xn, xs, rtol=1e-9, atol=1e-12 * np.max(np.abs(xs)))
    c.close()


def test_noalloc_rejects_oversized_system(xg, torch_cuda):
    torch = torch_cuda
    n = 262144 + 8  # XG_NOALLOC_MAX_N + 8 unknowns
    nl = N.Netlist(label="long_chain")
    nodes = [nl.node() for _ in range(n)]
    nl.R(nodes[0], -1, 1.0)
    for i in range(n - 1):
        nl.R(nodes[i], nodes[i + 1], 1.0)
    c = xg.Circuit(nl)
    b = torch.zeros(c.n, dtype=torch.float64, device="cuda:0")
    x = torch.zeros_like(b)
    with pytest.raises(xg.XgError) as e:
        c.lu_solve_noalloc(b, x)
    assert e.value.code == -1 and "scratch limit" in str(e.value)
    c.close()
