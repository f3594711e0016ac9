"""Generates tests/golden/ksparse_solves.npz: sparse systems drawn from the
synthetic circuits, solved by Kundert Sparse 1.3 compiled from the reference's
own sources (src/LinearAlgebraServicesPKG/ksparse, via oracle/Makefile `ref`)
with the reference's default thresholds (Epetra_CrsKundertSparse.h:130-132).

Run here, where the reference tree is present:  python tests/golden/make_golden.py
The fixture lets the GPU-box tests (no reference tree there) compare the GPU
LU against the reference solver's own outputs.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from xyce_gb300 import netlist as N  # noqa: E402


def circuits():
    """(name, netlist, step) of every system in the fixture."""
    return [("testnetlist2", N.test_netlist2(), 1e-6),
            ("diode_ladder_60", N.diode_ladder(60, seed=11), 1e-9),
            ("ring_51", N.ring_oscillator(51), 1e-12),
            ("ring_21_caps", N.ring_oscillator(21, caps=True), 2e-12),
            ("power_grid_12", N.power_grid(12, 20, seed=5), 1e-12),
            ("mc_rings_4", N.monte_carlo_rings(4, 11, 31, seed=9), 1e-12)]


def cases():
    out = []
    rng = np.random.default_rng(2024)
    for name, nl, h in circuits():
        o = oracle.Oracle(nl)
        st, x0, _ = o.dcop()
        x = x0 + 0.01 * rng.standard_normal(o.n)
        ld = o.load(x, time=1e-9, sto_curr=np.zeros(max(1, o.nsto)))
        vals = ld["dFdx"] + ld["dQdx"] / h
        b = rng.standard_normal(o.n)
        xk = oracle.ksparse_solve(o.row_ptr, o.col_idx, vals, b)
        out.append((name, o.row_ptr.copy(), o.col_idx.copy(), vals, b, xk))
    return out


def main():
    arrays = {}
    names = []
    for name, rp, ci, vals, b, xk in cases():
        names.append(name)
        arrays[f"{name}.row_ptr"] = rp
        arrays[f"{name}.col_idx"] = ci
        arrays[f"{name}.vals"] = vals
        arrays[f"{name}.b"] = b
        arrays[f"{name}.x_ksparse"] = xk
    arrays["names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "ksparse_solves.npz"), **arrays)
    print("wrote", len(names), "systems")


if __name__ == "__main__":
    main()
