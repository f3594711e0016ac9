"""Learned predictor: GPU kernels against the CPU oracle, training, and what
the trained network gains over the polynomial predictor.

Tolerances (written here, used below):
  * forward and gradients: the oracle (oracle/mlp.py, FP64 with the GPU's
    BF16 operand rounding) and the GPU (BF16 tensor-core products, FP32
    accumulation) agree to 2e-3 of each parameter block's largest magnitude
    (FP32 accumulation order, tanhf);
  * waveforms of the learned-predictor run against the polynomial run of the
    same circuit: both are converged to the same Newton and LTE tolerances
    (TIMEINT reltol 1e-4, abstol 1e-7), so they agree to a few times the
    tolerance, 10 * (reltol * max|v| + abstol).
"""
import numpy as np
import pytest

import oracle.mlp as M
from xyce_gb300 import netlist as N

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def _blocks():
    return [("W1", M.OFF_W1, M.OFF_B1), ("b1", M.OFF_B1, M.OFF_W2), ("W2", M.OFF_W2, M.OFF_B2),
            ("b2", M.OFF_B2, M.OFF_W3), ("w3", M.OFF_W3, M.OFF_B3), ("b3", M.OFF_B3, M.N_PARAM)]


def _small_circuit(xg):
    return xg.Circuit(N.bsim4_inverter_chain(2))


def test_mlp_forward_and_gradients_match_oracle(xg, torch_cuda):
    torch = torch_cuda
    rng = np.random.default_rng(11)
    theta = rng.normal(0, 0.25, M.N_PARAM).astype(np.float32)
    norm = np.concatenate([np.zeros(5), np.ones(5), [0.0, 1.0]]).astype(np.float32)
    X = rng.normal(0, 1, (3001, 5)).astype(np.float32)   # not a multiple of the 64-row tile
    Y = rng.normal(0, 1, 3001).astype(np.float32)
    c = _small_circuit(xg)
    c.mlp_set(theta, norm)
    Xd, Yd = torch.as_tensor(X, device="cuda:0"), torch.as_tensor(Y, device="cuda:0")
    out = torch.zeros(len(Y), dtype=torch.float32, device="cuda:0")
    c.mlp_forward(Xd, out)
    torch.cuda.synchronize()
    y_ref, _ = M.forward(theta.astype(np.float64), X)
    np.testing.assert_allclose(out.cpu().numpy(), y_ref, rtol=0, atol=2e-3 * np.max(np.abs(y_ref)))
    loss, g = c.mlp_grad(Xd, Yd)
    loss_ref, g_ref = M.loss_and_grad(theta.astype(np.float64), X, Y)
    assert abs(loss - loss_ref) <= 1e-4 * loss_ref, (loss, loss_ref)
    for name, a, b in _blocks():
        scale = np.max(np.abs(g_ref[a:b]))
        err = np.max(np.abs(g[a:b] - g_ref[a:b]))
        assert err <= 2e-3 * scale, (name, err, scale)
    c.close()


def _tight(nl):
    nl.tran.reltol, nl.tran.abstol = 1e-4, 1e-7
    return nl


def test_trained_predictor_on_unseen_circuit(xg, torch_cuda):
    """Train on the plain runs of two BSIM4 logic DAGs, apply to a third
    (different seed), and report what the network gains over the polynomial
    predictor: Newton iterations per accepted step of both runs.

    What is asserted: training lowers the loss; the trained network is used
    on the unseen circuit; the fallback rule bounds any loss of iterations to
    10 %; both runs stay within the tolerance band of each other (20 mV on
    a 1 V logic circuit with 20 ps edges: the two runs place their steps
    differently and each is converged to TIMEINT reltol 1e-4).  On this
    family the gain measured so far is negative (the next node state depends
    on neighbouring gates that a per-node history does not see); the number
    printed here is the record of it."""
    from xyce_gb300 import predictor as P
    fam = lambda seed: _tight(N.bsim4_logic_dag(800, 12, seed=seed, tstop=3e-9))
    Xs, Ys = [], []
    for seed in (21, 22):
        nl = fam(seed)
        counts, t, v, p, probes, st = P.record(nl, cap=4000)
        assert st["status"] == 0
        X, Y = P.dataset(counts, t, v, p, [len(probes)])
        Xs.append(X)
        Ys.append(Y)
    X, Y = np.concatenate(Xs), np.concatenate(Ys)
    c = _small_circuit(xg)
    theta, norm, hist = P.train(c, X, Y, iters=600, lr=3e-3, batch=200000)
    c.close()
    assert hist[-1] < hist[0], (hist[0], hist[-1])
    test = fam(23)
    probes = [test.names["g50"], test.names["g120"], test.names["g200"]]
    cp, tp, vp, sp, _ = P.run(test, probes=probes, cap=4000)
    cl, tl, vl, sl, ps = P.run(test, theta, norm, probes=probes, cap=4000)
    assert sp["status"] == 0 and sl["status"] == 0
    ipp = sp["newton_iters"] / sp["accepted"]
    ipl = sl["newton_iters"] / sl["accepted"]
    print(f"Newton iterations per step: polynomial {ipp:.3f}, learned {ipl:.3f} "
          f"(gain {100 * (ipp - ipl) / ipp:+.1f} %); learned steps {ps['learned_steps']} "
          f"({ps['learned_iters'] / max(1, ps['learned_steps']):.3f} it/step), fallback steps {ps['poly_steps']}")
    assert ps["learned_steps"] > 0
    assert ipl <= 1.10 * ipp, (ipl, ipp)
    kp, kl = int(cp[0]), int(cl[0])
    g = np.stack([np.interp(tp[0, :kp], tl[0, :kl], vl[0, :kl, j]) for j in range(3)], axis=1)
    err = np.max(np.abs(g - vp[0, :kp]))
    assert err <= 0.02, err
