"""CPU restatement (numpy, float64) of the learned tile-cost model -- TEST INFRASTRUCTURE ONLY.

The network of the GPU scheduler (parallel-rdp_gb300/csrc/sched.cu): 16 -> 64 -> 64 -> 1 with
ReLU, parameters packed as W1[64][16], b1[64], W2[64][64], b2[64], W3[64], b3, stored in FP16
on the device.  The loss is the mean squared error.  This file gives the forward pass and the
analytic gradients the GPU kernels must reproduce (the GPU accumulates in FP32).  The model is
this build's own (the reference has none), so there is nothing to pin it to beyond calculus:
`numeric_gradients` checks `gradients` by central differences.
"""
import numpy as np

IN, H = 16, 64
W1, B1 = 0, H * IN
W2 = B1 + H
B2 = W2 + H * H
W3 = B2 + H
B3 = W3 + H
PARAMS = B3 + 1


def fp16_round(params):
    return np.asarray(params, dtype=np.float32).astype(np.float16).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[W1:B1].reshape(H, IN), p[B1:W2], p[W2:B2].reshape(H, H), p[B2:W3], p[W3:B3], p[B3])


def forward(params, x):
    w1, b1, w2, b2, w3, b3 = unpack(params)
    x = np.asarray(x, dtype=np.float64)
    h1 = np.maximum(x @ w1.T + b1, 0.0)
    h2 = np.maximum(h1 @ w2.T + b2, 0.0)
    return h2 @ w3 + b3, (x, h1, h2)


def loss(params, x, y):
    out, _ = forward(params, x)
    return float(np.mean((out - np.asarray(y, dtype=np.float64)) ** 2))


def gradients(params, x, y):
    """d loss / d params (packed like params) and the loss."""
    w1, b1, w2, b2, w3, b3 = unpack(params)
    out, (x, h1, h2) = forward(params, x)
    n = x.shape[0]
    d_out = 2.0 * (out - np.asarray(y, dtype=np.float64)) / n
    g = np.zeros(PARAMS)
    g[W3:B3] = d_out @ h2
    g[B3] = d_out.sum()
    d_h2 = np.outer(d_out, w3) * (h2 > 0)
    g[W2:B2] = (d_h2.T @ h1).ravel()
    g[B2:W3] = d_h2.sum(axis=0)
    d_h1 = (d_h2 @ w2) * (h1 > 0)
    g[W1:B1] = (d_h1.T @ x).ravel()
    g[B1:W2] = d_h1.sum(axis=0)
    return g, float(np.mean((out - y) ** 2))


def numeric_gradients(params, x, y, indices, eps=1e-6):
    p = np.asarray(params, dtype=np.float64).copy()
    out = []
    for i in indices:
        a, b = p.copy(), p.copy()
        a[i] += eps
        b[i] -= eps
        out.append((loss(a, x, y) - loss(b, x, y)) / (2 * eps))
    return np.array(out)


def init_params(seed=0):
    rng = np.random.default_rng(seed)
    p = np.zeros(PARAMS)
    p[W1:B1] = rng.uniform(-1, 1, H * IN) * np.sqrt(6 / (IN + H))
    p[W2:B2] = rng.uniform(-1, 1, H * H) * np.sqrt(6 / (2 * H))
    p[W3:B3] = rng.uniform(-1, 1, H) * np.sqrt(6 / (H + 1))
    p[B1:W2] = rng.uniform(0, 0.1, H)
    p[B2:W3] = rng.uniform(0, 0.1, H)
    return p
