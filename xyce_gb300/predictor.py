"""Learned Newton predictor: training data, training and evaluation.

The network and its kernels live in the library (xg_mlp.cu, C-ABI
xg_mlp_* / xg_set_predictor).  This module builds the training set from
plain (polynomial-predictor) runs recorded on the GPU and trains the network
there with the library's own forward/backward kernels.

Training set (one row per node unknown and accepted step n+1 with four
accepted solutions before it, as the device applies the network), with the
node's recent motion s = |d1| + |d2| + |d3| + 1e-9 V (d1 = x_n - x_{n-1},
d2 = x_{n-1} - x_{n-2}, d3 = x_{n-2} - x_{n-3}):
  features  d1 / s, d2 / s, d3 / s, x_n, log(h_{n+1} / h_n)
  target    (x_{n+1} - polynomial predictor of step n+1) / s
The device starts Newton from the polynomial predictor plus s times the
network's output; nodes with s < 1e-5 V keep the polynomial guess and are
left out of the training set.
The recorded sequence of a circuit starts with its operating point (index 0)
followed by the accepted transient points, so step index m >= 5 qualifies.
"""
from __future__ import annotations

import numpy as np

from . import MLP_NNORM, MLP_NPARAM, PRED_LEARNED, PRED_POLY, Circuit

N_IN, N_HID = 5, 64
SCALE_FLOOR = 1e-9  # V, as kMlpScaleFloor in the library
ACTIVE = 1e-5       # V, as kMlpActive: nodes moving less are not corrected


def node_unknowns(nl) -> np.ndarray:
    """Unknowns that are node voltages (voltage-source branch currents excluded)."""
    branch = {v[2] for v in nl.vsrc}
    return np.array([u for u in range(nl.n) if u not in branch], np.int32)


def record(nl, cap=20000, tran=None):
    """Plain run recording every node voltage and its predictor at each
    accepted point: returns (counts, times, values, predictors, probes, stats)."""
    probes = node_unknowns(nl)
    c = Circuit(nl)
    try:
        c.set_predictor(PRED_POLY)
        c.tran_start(tran, probes=probes, cap=cap)
        c.tran_advance(0)
        counts, t, v, st = c.tran_results()
        p = c.tran_predictors()
        c.tran_end()
    finally:
        c.close()
    return counts, t, v, p, probes, st


def dataset(counts, t, v, p, pcount):
    """Features X (rows x 5) and targets Y from recorded runs; pcount[c] is
    the number of probes recorded for circuit c."""
    xs, ys = [], []
    for c in range(len(counts)):
        k, q = int(counts[c]), int(pcount[c])
        if k < 6 or q == 0:
            continue
        tt, vv, pp = t[c, :k], v[c, :k, :q], p[c, :k, :q]
        for m in range(5, k):
            h1, h0 = tt[m] - tt[m - 1], tt[m - 1] - tt[m - 2]
            if h1 <= 0 or h0 <= 0:
                continue
            d1, d2, d3 = vv[m - 1] - vv[m - 2], vv[m - 2] - vv[m - 3], vv[m - 3] - vv[m - 4]
            sc = np.abs(d1) + np.abs(d2) + np.abs(d3) + SCALE_FLOOR
            act = sc >= ACTIVE
            if not act.any():
                continue
            f = np.empty((int(act.sum()), N_IN))
            f[:, 0], f[:, 1], f[:, 2] = d1[act] / sc[act], d2[act] / sc[act], d3[act] / sc[act]
            f[:, 3] = vv[m - 1][act]
            f[:, 4] = np.log(h1 / h0)
            xs.append(f)
            ys.append((vv[m][act] - pp[m][act]) / sc[act])
    return np.concatenate(xs), np.concatenate(ys)


def normalization(X, Y):
    """in_shift, in_scale, out_shift, out_scale (standardization)."""
    mu, sd = X.mean(0), X.std(0)
    sd[sd == 0] = 1.0
    ymu, ysd = float(Y.mean()), float(Y.std()) or 1.0
    return np.concatenate([mu, 1.0 / sd, [ymu, ysd]]).astype(np.float32)


def init_theta(seed=0) -> np.ndarray:
    """Glorot-uniform weights, zero biases; the output layer starts at zero so
    the untrained network returns the polynomial predictor unchanged."""
    rng = np.random.default_rng(seed)
    th = np.zeros(MLP_NPARAM, np.float32)
    a1 = np.sqrt(6.0 / (N_IN + N_HID))
    th[0:N_IN * N_HID] = rng.uniform(-a1, a1, N_IN * N_HID)
    o = N_IN * N_HID + N_HID
    a2 = np.sqrt(6.0 / (2 * N_HID))
    th[o:o + N_HID * N_HID] = rng.uniform(-a2, a2, N_HID * N_HID)
    return th


def train(circ: Circuit, X, Y, iters=400, lr=3e-3, seed=0, batch=None):
    """Standardize, upload and train on the GPU (Adam, full batch or a
    random subset of `batch` rows); returns (theta, norm, loss history)."""
    import torch
    norm = normalization(X, Y)
    Xs = ((X - norm[:N_IN]) * norm[N_IN:2 * N_IN]).astype(np.float32)
    Ys = ((Y - norm[2 * N_IN]) / norm[2 * N_IN + 1]).astype(np.float32)
    if batch is not None and batch < len(Ys):
        idx = np.random.default_rng(seed).choice(len(Ys), batch, replace=False)
        Xs, Ys = Xs[idx], Ys[idx]
    dev = "cuda:%d" % torch.cuda.current_device()
    Xd = torch.as_tensor(np.ascontiguousarray(Xs), device=dev)
    Yd = torch.as_tensor(np.ascontiguousarray(Ys), device=dev)
    circ.mlp_set(init_theta(seed), norm)
    hist = circ.mlp_train(Xd, Yd, iters, lr)
    theta, norm = circ.mlp_get()
    return theta, norm, hist


def run(nl, theta=None, norm=None, probes=(), cap=0):
    """Transient with the learned predictor (when theta is given) or the
    polynomial one; returns (counts, times, values, stats, predictor stats)."""
    c = Circuit(nl)
    try:
        if theta is not None:
            c.mlp_set(theta, norm)
            c.set_predictor(PRED_LEARNED)
        c.tran_start(probes=probes, cap=cap)
        c.tran_advance(0)
        counts, t, v, st = c.tran_results()
        ps = c.predictor_stats()
        c.tran_end()
    finally:
        c.close()
    return counts, t, v, st, ps
