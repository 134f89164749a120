"""The CPU restatement of the learned tile-cost model: its analytic gradients agree with
central differences (this pins the oracle the GPU training kernels are checked against)."""
import numpy as np

from mlp_oracle import PARAMS, IN, fp16_round, gradients, init_params, numeric_gradients


def test_gradients_match_central_differences():
    rng = np.random.default_rng(0)
    p = fp16_round(init_params(3))
    x = rng.uniform(0, 1, (24, IN))
    y = rng.uniform(0, 2, 24)
    g, _ = gradients(p, x, y)
    idx = np.concatenate([rng.integers(0, PARAMS, 200), [PARAMS - 1]])
    num = numeric_gradients(p, x, y, idx)
    np.testing.assert_allclose(g[idx], num, rtol=1e-4, atol=1e-7)


def test_gradient_descent_reduces_loss():
    rng = np.random.default_rng(1)
    p = init_params(4)
    x = rng.uniform(0, 1, (256, IN))
    y = x[:, 0] * 1.5 + 0.25 * x[:, 3]
    g, l0 = gradients(p, x, y)
    for _ in range(200):
        g, l = gradients(p, x, y)
        p = p - 0.05 * g
    assert l < 0.25 * l0
