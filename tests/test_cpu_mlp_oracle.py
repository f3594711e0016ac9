"""The MLP oracle's backward pass against finite differences (BF16 rounding
switched off so the loss is smooth): pins the restated gradients that the
GPU training kernels are checked against."""
import numpy as np

import oracle.mlp as M


def test_oracle_mlp_gradient_matches_finite_differences(monkeypatch):
    monkeypatch.setattr(M, "bf16", lambda a: np.asarray(a, np.float64))
    rng = np.random.default_rng(3)
    theta = rng.normal(0, 0.3, M.N_PARAM)
    X = rng.normal(0, 1, (40, M.N_IN))
    Y = rng.normal(0, 1, 40)
    _, g = M.loss_and_grad(theta, X, Y)
    idx = np.concatenate([rng.choice(M.N_PARAM, 60, replace=False), [M.OFF_B3]])
    for i in idx:
        h = 1e-6
        tp, tm = theta.copy(), theta.copy()
        tp[i] += h
        tm[i] -= h
        fd = (M.loss_and_grad(tp, X, Y)[0] - M.loss_and_grad(tm, X, Y)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 1e-30], np.float32)
    r = M.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -6 and r[3] == -2.5
