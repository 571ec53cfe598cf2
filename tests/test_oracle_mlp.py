"""The CPU restatement of the proposal network (oracle/mlp.py), pinned before it
checks the device: its gradient equals central finite differences of its loss
(computed in float64 without the bf16 rounding, which the gradient treats as the
identity)."""
import numpy as np

from oracle import mlp


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(3)
    n = 96
    x = mlp.bf16_round(rng.normal(size=(n, mlp.N_IN)).astype(np.float32))
    y = rng.random(n) < 0.3
    p = (rng.normal(size=mlp.N_HID * mlp.N_IN + 2 * mlp.N_HID + 1) * 0.3).astype(np.float32)
    # parameters already on the bf16 grid, so the rounding is exact at p
    k = mlp.N_HID * mlp.N_IN
    p[:k] = mlp.bf16_round(p[:k])
    p[k + mlp.N_HID:k + 2 * mlp.N_HID] = mlp.bf16_round(p[k + mlp.N_HID:k + 2 * mlp.N_HID])
    loss, g = mlp.loss_and_grads(p, x, y, 2.5)

    def loss64(q):
        W1, b1, w2, b2 = [a.astype(np.float64) for a in mlp.unpack(q)]
        h = np.maximum(x.astype(np.float64) @ W1.T + b1, 0)
        z = h @ w2 + b2
        wt = np.where(y, 2.5, 1.0)
        sp = lambda t: np.maximum(t, 0) + np.log1p(np.exp(-np.abs(t)))  # noqa: E731
        return np.mean(wt * np.where(y, sp(-z), sp(z)))

    assert abs(loss - loss64(p.astype(np.float64))) < 1e-5
    eps = 1e-4
    for i in list(range(0, k, 37)) + list(range(k, len(p))):
        q1, q2 = p.astype(np.float64).copy(), p.astype(np.float64).copy()
        q1[i] += eps
        q2[i] -= eps
        fd = (loss64(q1) - loss64(q2)) / (2 * eps)
        assert abs(fd - g[i]) < 1e-4 + 1e-3 * abs(fd), (i, fd, g[i])
