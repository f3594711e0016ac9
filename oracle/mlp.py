"""CPU restatement of the learned predictor's network, forward and backward.

TEST INFRASTRUCTURE ONLY: the checker for the GPU MLP kernels of xyce_gb300
(xg_mlp.cu).  The network has no counterpart in the reference (it hooks the
predictor of WorkingIntegrationMethod::obtainPredictor,
src/TimeIntegrationPKG/N_TIA_WorkingIntegrationMethod.C:176).  Arithmetic is
FP64; the operands the GPU feeds to its BF16 tensor-core products are rounded
to BF16 at the same points (features and W1 for layer 1, tanh(Z1) and W2 for
layer 2, dZ2 and W2 for dH1 = dZ2 W2^T), so the GPU gradients can be checked
to FP32 accumulation accuracy.
"""
from __future__ import annotations

import numpy as np

N_IN, N_HID = 5, 64
OFF_W1 = 0
OFF_B1 = OFF_W1 + N_IN * N_HID
OFF_W2 = OFF_B1 + N_HID
OFF_B2 = OFF_W2 + N_HID * N_HID
OFF_W3 = OFF_B2 + N_HID
OFF_B3 = OFF_W3 + N_HID
N_PARAM = OFF_B3 + 1


def bf16(a):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.asarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(theta):
    t = np.asarray(theta, np.float64)
    W1 = t[OFF_W1:OFF_B1].reshape(N_IN, N_HID)
    b1 = t[OFF_B1:OFF_W2]
    W2 = t[OFF_W2:OFF_B2].reshape(N_HID, N_HID)
    b2 = t[OFF_B2:OFF_W3]
    w3 = t[OFF_W3:OFF_B3]
    b3 = t[OFF_B3]
    return W1, b1, W2, b2, w3, b3


def forward(theta, X):
    W1, b1, W2, b2, w3, b3 = unpack(theta)
    h1 = np.tanh(bf16(X) @ bf16(W1) + b1)
    h2 = np.tanh(bf16(h1) @ bf16(W2) + b2)
    return h2 @ w3 + b3, (h1, h2)


def loss_and_grad(theta, X, Y):
    """L = 0.5 / N * sum (MLP(X) - Y)^2 and dL/dtheta (layout of N_PARAM)."""
    X = np.asarray(X, np.float64)
    Y = np.asarray(Y, np.float64)
    W1, b1, W2, b2, w3, b3 = unpack(theta)
    y, (h1, h2) = forward(theta, X)
    n = len(Y)
    e = y - Y
    loss = 0.5 * np.sum(e * e) / n
    dy = e / n
    dz2 = dy[:, None] * w3[None, :] * (1.0 - h2 * h2)
    dh1 = bf16(dz2) @ bf16(W2).T
    dz1 = dh1 * (1.0 - h1 * h1)
    g = np.zeros(N_PARAM)
    g[OFF_W1:OFF_B1] = (X.T @ dz1).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    g[OFF_W2:OFF_B2] = (h1.T @ dz2).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    g[OFF_W3:OFF_B3] = h2.T @ dy
    g[OFF_B3] = dy.sum()
    return loss, g
