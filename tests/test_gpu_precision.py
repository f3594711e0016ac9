"""Precision form: FP32 LU factors with FP64 iterative refinement.

The factors are computed and stored in FP32; every solve is refined against
the FP64 matrix (r = b - A x in FP64, x += (LU)^-1 r), the scheme of Xyce's
IRSolver (src/LinearAlgebraServicesPKG/N_LAS_IRSolver.C:482-540) with a
fresh FP32 factorization in place of a stale FP64 one.

Tolerances (written here, used below):
  * linear solves: after REFINE steps, relative error <= 1e-9 against Kundert
    Sparse compiled from the reference (golden fixture) — the FP64 path's
    bar; with no refinement the FP32 solve alone must be visibly worse
    (error > 1e-12), which shows the refinement is doing the work;
  * waveforms: the precision form against the FP64 oracle at the oracle's
    accepted time points, |dv| <= 1e-6 * max|v| + 1e-9 (reltol 1e-6) on
    circuits run with TIMEINT / Newton reltol 1e-6, abstol 1e-9.
"""
import os
import sys

import numpy as np
import pytest

from xyce_gb300 import netlist as N

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ksparse_solves.npz")
REFINE = 3
WAVE_RTOL, WAVE_ATOL = 1e-6, 1e-9


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _t(torch, a):
    return torch.as_tensor(np.ascontiguousarray(a, np.float64), device="cuda:0")


def _solve(xg, torch, nl, vals, b, prec, refine):
    c = xg.Circuit(nl)
    c.lu_set_precision(prec, refine)
    v, bb = _t(torch, vals), _t(torch, b)
    x = torch.zeros_like(bb)
    c.lu_analyze(v)
    c.lu_factor(v)
    c.lu_solve(bb, x)
    torch.cuda.synchronize()
    out = x.cpu().numpy()
    c.close()
    return out


def test_fp32_refined_solve_matches_ksparse_golden(xg, torch_cuda):
    sys.path.insert(0, os.path.dirname(__file__))
    from golden.make_golden import circuits
    g = np.load(GOLDEN)
    specs = {name: nl for name, nl, _ in circuits()}
    for name in g["names"]:
        vals, b, xk = (g[f"{name}.{k}"] for k in ("vals", "b", "x_ksparse"))
        nl = specs[str(name)]
        x = _solve(xg, torch_cuda, nl, vals, b, xg.PREC_FP32_IR, REFINE)
        scale = np.max(np.abs(xk))
        err = np.max(np.abs(x - xk)) / scale
        assert err <= 1e-9, (str(name), err)


def test_refinement_is_what_recovers_fp64_accuracy(xg, torch_cuda):
    sys.path.insert(0, os.path.dirname(__file__))
    from golden.make_golden import circuits
    g = np.load(GOLDEN)
    specs = {name: nl for name, nl, _ in circuits()}
    name = "power_grid_12"
    vals, b, xk = (g[f"{name}.{k}"] for k in ("vals", "b", "x_ksparse"))
    scale = np.max(np.abs(xk))
    e0 = np.max(np.abs(_solve(xg, torch_cuda, specs[name], vals, b, xg.PREC_FP32_IR, 0) - xk)) / scale
    e3 = np.max(np.abs(_solve(xg, torch_cuda, specs[name], vals, b, xg.PREC_FP32_IR, REFINE) - xk)) / scale
    assert e0 > 1e-12, e0          # FP32 factors alone: single-precision accuracy
    assert e3 <= 1e-9 and e3 < e0 * 1e-2, (e0, e3)


def _tight(nl, tstop):
    nl.tran.tstop = tstop
    nl.tran.reltol, nl.tran.abstol = 1e-6, 1e-9
    nl.tran.nl_reltol, nl.tran.nl_abstol = 1e-6, 1e-9
    return nl


@pytest.mark.parametrize("name,maker,probes", [
    ("power_grid_20", lambda: _tight(N.power_grid(20, 40, seed=7), 0.2e-9), [0, "center", 399]),
    ("ring_21", lambda: _tight(N.ring_oscillator(21), 2e-9), ["n1", "n11"]),
    ("mc_rings_3", lambda: _tight(N.monte_carlo_rings(3, 11, 21, seed=2), 1e-9), ["c0.n1", "c2.n1"]),
])
def test_precision_form_waveforms_match_fp64_oracle(xg, oracle_mod, torch_cuda, name, maker, probes):
    nl = maker()
    pr = [nl.names[p] if isinstance(p, str) else p for p in probes]
    c = xg.Circuit(nl)
    c.lu_set_precision(xg.PREC_FP32_IR, 2)
    counts, t, v, st = c.transient(probes=pr, cap=400000)
    assert st["status"] == 0
    for ci in range(nl.n_circuits):
        mine = [j for j, p in enumerate(pr) if nl.circuit_of(p) == ci]
        if not mine:
            continue
        k = int(counts[ci])
        sub = N.extract_circuit(nl, ci)
        to, vo, so = oracle_mod.Oracle(sub).transient(probes=[pr[j] - nl.offsets[ci] for j in mine])
        assert so["status"] == 0
        g = np.stack([np.interp(to, t[ci, :k], v[ci, :k, q]) for q in range(len(mine))], axis=1)
        err = np.max(np.abs(g - vo))
        tol = WAVE_RTOL * np.max(np.abs(vo)) + WAVE_ATOL
        print(f"{name} circuit {ci}: max |dv| vs FP64 oracle = {err:.3e} (tol {tol:.3e})")
        assert err <= tol, (name, ci, err, tol)
