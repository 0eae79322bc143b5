"""The scoring MLP's own CUDA forward/backward/Adam kernels against the float64
oracle (oracle/mlp_oracle.py) on the same bf16-rounded weights.

Tolerances: forward probabilities and the loss within 2e-5 absolute; every
gradient tensor within 1e-3 relative to its largest magnitude (fp32
accumulation in a different order and fp32 atomics, against float64)."""
import numpy as np
import pytest

from oracle import mlp_oracle

pytestmark = pytest.mark.gpu


def _data(n, F, seed):
    rng = np.random.default_rng(seed)
    X = rng.random((n, F)).astype(np.float32)
    Y = (rng.random(n) < 0.3).astype(np.float32)
    WT = rng.uniform(0.5, 2.0, n).astype(np.float32)
    return X, Y, WT


@pytest.mark.parametrize("n,seed", [(1000, 0), (37, 1), (4096, 2)])
def test_forward_backward_match_oracle(engine, n, seed):
    torch = pytest.importorskip("torch")
    from sgfim.mlp import Trainer
    tr = Trainer(engine, seed=seed)
    X, Y, WT = _data(n, tr.in_dim, seed)
    loss, g = tr.gradients(torch.from_numpy(X), torch.from_numpy(Y), torch.from_numpy(WT))
    torch.cuda.synchronize()
    w = tr.weights_bf16_as_float()
    ref_loss, ref_g = mlp_oracle.loss_and_grads(X.astype(np.float64), Y.astype(np.float64), WT, w["W1"], w["b1"],
                                                w["W2"], w["b2"], w["w3"], w["b3"][0])
    P = tr.forward(torch.from_numpy(X)).cpu().numpy()
    _, _, ref_p = mlp_oracle.forward(X, w["W1"], w["b1"], w["W2"], w["b2"], w["w3"], w["b3"][0])
    assert np.abs(P - ref_p).max() < 2e-5
    assert abs(float(loss.item()) - ref_loss) < 2e-5
    for k in ("W1", "b1", "W2", "b2", "w3", "b3"):
        got = g[k].cpu().numpy().astype(np.float64).reshape(ref_g[k].shape)
        scale = max(np.abs(ref_g[k]).max(), 1e-12)
        assert np.abs(got - ref_g[k]).max() / scale < 1e-3, k


def test_oracle_gradients_by_finite_differences():
    rng = np.random.default_rng(5)
    F, H, n = 8, 32, 50
    X = rng.random((n, F))
    Y = (rng.random(n) < 0.4).astype(float)
    W = dict(W1=rng.normal(0, .5, (H, F)), b1=rng.normal(0, .1, H), W2=rng.normal(0, .3, (H, H)),
             b2=rng.normal(0, .1, H), w3=rng.normal(0, .3, H), b3=np.array([0.1]))
    _, g = mlp_oracle.loss_and_grads(X, Y, None, W["W1"], W["b1"], W["W2"], W["b2"], W["w3"], W["b3"][0])
    eps = 1e-6
    for k in W:
        flat = W[k].reshape(-1)
        for i in rng.choice(flat.size, min(5, flat.size), replace=False):
            old = flat[i]
            flat[i] = old + eps
            lp, _ = mlp_oracle.loss_and_grads(X, Y, None, W["W1"], W["b1"], W["W2"], W["b2"], W["w3"], W["b3"][0])
            flat[i] = old - eps
            lm, _ = mlp_oracle.loss_and_grads(X, Y, None, W["W1"], W["b1"], W["W2"], W["b2"], W["w3"], W["b3"][0])
            flat[i] = old
            assert abs((lp - lm) / (2 * eps) - g[k].reshape(-1)[i]) < 1e-6


def test_training_reduces_loss(engine):
    torch = pytest.importorskip("torch")
    from sgfim.mlp import Trainer
    rng = np.random.default_rng(9)
    n = 20000
    X = rng.random((n, 8)).astype(np.float32)
    Y = ((X[:, 0] * 2 + X[:, 3] - X[:, 5]) > 1.0).astype(np.float32)   # a learnable rule
    tr = Trainer(engine, seed=1)
    hist = tr.fit(X, Y, epochs=6, batch=2048, lr=3e-3, balance=False)
    assert hist[-1] < 0.5 * hist[0]
    P = tr.forward(torch.from_numpy(X)).cpu().numpy()
    assert ((P > 0.5) == (Y > 0.5)).mean() > 0.95
