"""CPU: the FP64 NumPy restatement of the warm-start MLP (oracle/mlp.py) is
pinned by central finite differences of its own loss."""
from __future__ import annotations

import numpy as np


def test_mlp_oracle_gradient_matches_finite_differences():
    from oracle import mlp
    rng = np.random.default_rng(0)
    P = mlp.offsets(9, 2)["P"]
    # parameters already on the BF16 grid, so the straight-through rounding is exact
    p = mlp.bf16((0.2 * rng.standard_normal(P)).astype(np.float32)).astype(np.float32)
    X = rng.standard_normal((16, 9))
    T = rng.standard_normal((16, 2))
    loss, g = mlp.loss_and_grad(p, X, T)
    o = mlp.offsets(9, 2)
    W0, b0, W1, b1, W2, b2, W3, b3 = mlp.unpack(p, 9, 2)

    def L(q):
        """loss with the (unrounded) biases taken from the FP64 vector q"""
        a0 = mlp.gelu(X @ W0.T + q[o["b0"]:o["W1"]])
        a1 = mlp.gelu(a0 @ W1.T + q[o["b1"]:o["W2"]])
        a2 = mlp.gelu(a1 @ W2.T + q[o["b2"]:o["W3"]])
        return np.mean((a2 @ W3.T + q[o["b3"]:] - T) ** 2)

    h = 1e-3
    for idx in (o["b0"] + 3, o["b1"] + 10, o["b2"] + 63, o["b3"] + 1):
        pp = p.astype(np.float64).copy()
        pm = p.astype(np.float64).copy()
        pp[idx] += h
        pm[idx] -= h
        fd = (L(pp) - L(pm)) / (2 * h)
        assert abs(fd - g[idx]) < 1e-6 * max(1.0, abs(g[idx])) + 1e-9
    # a weight entry: perturb by one BF16 ulp-scale step through a float64 loss
    assert np.isfinite(loss) and g.shape == (P,)
