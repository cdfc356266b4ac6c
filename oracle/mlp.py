"""NumPy FP64 restatement of the warm-start MLP (TEST INFRASTRUCTURE ONLY):
9 -> 64 -> 64 -> 64 -> 2, GELU (erf form), weights rounded to BF16 as the GPU
kernels read them, MSE loss; forward and backward, for the gradient check of
the GPU training kernels."""
from __future__ import annotations

import math

import numpy as np

H = 64


def bf16(x: np.ndarray) -> np.ndarray:
    """Round float32 to bfloat16 (nearest even), returned as float64."""
    u = np.ascontiguousarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def offsets(n_in, n_out):
    o = {}
    o["W0"] = 0
    o["b0"] = o["W0"] + H * n_in
    o["W1"] = o["b0"] + H
    o["b1"] = o["W1"] + H * H
    o["W2"] = o["b1"] + H
    o["b2"] = o["W2"] + H * H
    o["W3"] = o["b2"] + H
    o["b3"] = o["W3"] + n_out * H
    o["P"] = o["b3"] + n_out
    return o


def unpack(p, n_in, n_out):
    o = offsets(n_in, n_out)
    p = np.asarray(p, dtype=np.float32)
    W0 = bf16(p[o["W0"]:o["b0"]]).reshape(H, n_in)
    b0 = p[o["b0"]:o["W1"]].astype(np.float64)
    W1 = bf16(p[o["W1"]:o["b1"]]).reshape(H, H)
    b1 = p[o["b1"]:o["W2"]].astype(np.float64)
    W2 = bf16(p[o["W2"]:o["b2"]]).reshape(H, H)
    b2 = p[o["b2"]:o["W3"]].astype(np.float64)
    W3 = bf16(p[o["W3"]:o["b3"]]).reshape(n_out, H)
    b3 = p[o["b3"]:].astype(np.float64)
    return W0, b0, W1, b1, W2, b2, W3, b3


_erf = np.vectorize(math.erf)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_d(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2 * math.pi)


def forward(p, X, n_in=9, n_out=2):
    W0, b0, W1, b1, W2, b2, W3, b3 = unpack(p, n_in, n_out)
    z0 = X @ W0.T + b0
    a0 = gelu(z0)
    z1 = a0 @ W1.T + b1
    a1 = gelu(z1)
    z2 = a1 @ W2.T + b2
    a2 = gelu(z2)
    y = a2 @ W3.T + b3
    return y, (z0, a0, z1, a1, z2, a2)


def loss_and_grad(p, X, T, n_in=9, n_out=2):
    """MSE over samples and outputs; gradient w.r.t. the FP32 master parameters
    (the BF16 rounding is passed straight through)."""
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    W0, b0, W1, b1, W2, b2, W3, b3 = unpack(p, n_in, n_out)
    y, (z0, a0, z1, a1, z2, a2) = forward(p, X, n_in, n_out)
    B = X.shape[0]
    loss = np.mean((y - T) ** 2)
    dy = 2.0 * (y - T) / (B * n_out)
    gW3 = dy.T @ a2
    gb3 = dy.sum(0)
    d2 = (dy @ W3) * gelu_d(z2)
    gW2 = d2.T @ a1
    gb2 = d2.sum(0)
    d1 = (d2 @ W2) * gelu_d(z1)
    gW1 = d1.T @ a0
    gb1 = d1.sum(0)
    d0 = (d1 @ W1) * gelu_d(z0)
    gW0 = d0.T @ X
    gb0 = d0.sum(0)
    g = np.concatenate([gW0.ravel(), gb0, gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g
