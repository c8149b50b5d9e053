"""CPU oracle of the cost-model MLP (test infrastructure only).

float64 restatement of the network the library's kernels implement
(cuspfft_gb300/csrc/gbsp_mlp.cu): n_in -> 64 -> 64 -> 1 with ReLU, packed
parameters W1[n_in][64], b1[64], W2[64][64], b2[64], w3[64], b3; loss
mean((f(x) - t)^2); ReLU derivative 0 at 0.  The network has no
counterpart in the reference: it follows the published backpropagation
equations, and the tests use it to check the GPU gradients.
"""
from __future__ import annotations

import numpy as np

H = 64


def unpack(p: np.ndarray, n_in: int):
    p = np.asarray(p, np.float64)
    o = 0
    w1 = p[o:o + n_in * H].reshape(n_in, H); o += n_in * H
    b1 = p[o:o + H]; o += H
    w2 = p[o:o + H * H].reshape(H, H); o += H * H
    b2 = p[o:o + H]; o += H
    w3 = p[o:o + H]; o += H
    b3 = p[o]; o += 1
    assert o == p.size
    return w1, b1, w2, b2, w3, b3


def forward(p: np.ndarray, x: np.ndarray) -> np.ndarray:
    x = np.asarray(x, np.float64)
    w1, b1, w2, b2, w3, b3 = unpack(p, x.shape[1])
    h1 = np.maximum(x @ w1 + b1, 0.0)
    h2 = np.maximum(h1 @ w2 + b2, 0.0)
    return h2 @ w3 + b3


def loss_and_grad(p: np.ndarray, x: np.ndarray, t: np.ndarray) -> tuple[float, np.ndarray]:
    x = np.asarray(x, np.float64)
    t = np.asarray(t, np.float64)
    n = x.shape[0]
    w1, b1, w2, b2, w3, b3 = unpack(p, x.shape[1])
    h1 = np.maximum(x @ w1 + b1, 0.0)
    h2 = np.maximum(h1 @ w2 + b2, 0.0)
    y = h2 @ w3 + b3
    e = y - t
    dy = 2.0 * e / n
    g_w3 = h2.T @ dy
    g_b3 = dy.sum()
    d2 = np.outer(dy, w3) * (h2 > 0)
    g_w2 = h1.T @ d2
    g_b2 = d2.sum(axis=0)
    d1 = (d2 @ w2.T) * (h1 > 0)
    g_w1 = x.T @ d1
    g_b1 = d1.sum(axis=0)
    g = np.concatenate([g_w1.ravel(), g_b1, g_w2.ravel(), g_b2, g_w3, [g_b3]])
    return float(np.mean(e * e)), g


def adam(p, g, m, v, lr, b1, b2, eps, step):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = p - lr * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
    return p, m, v
