"""The CPU oracle of the learned mode's network: its analytic gradients against finite differences."""
import numpy as np

from oracle import mlp_oracle as mo


def _loss(flat, dims, x, y, w):
    acts = mo.forward(flat, dims, x)
    return mo.gauss_loss(acts[-1], y, w)[0]


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    dims = [5, 7, 6, 3]
    n = sum(dims[k] * dims[k + 1] + dims[k + 1] for k in range(len(dims) - 1))
    flat = rng.normal(0, 0.5, n)
    x = rng.normal(size=(9, 5))
    y = rng.normal(size=(9, 2))
    w = rng.uniform(0.5, 2.0, 9)
    acts = mo.forward(flat, dims, x)
    _, dout = mo.gauss_loss(acts[-1], y, w)
    g = mo.backward(flat, dims, acts, dout)
    h = 1e-6
    fd = np.empty(n)
    for k in range(n):
        e = np.zeros(n)
        e[k] = h
        fd[k] = (_loss(flat + e, dims, x, y, w) - _loss(flat - e, dims, x, y, w)) / (2 * h)
    assert np.allclose(g, fd, rtol=1e-6, atol=1e-8)


def test_adam_first_step_moves_by_lr():
    p, g = np.array([1.0, -2.0]), np.array([0.3, -5.0])
    p1, m, v = mo.adam(p, g, np.zeros(2), np.zeros(2), 1, lr=0.01)
    assert np.allclose(p1, p - 0.01 * np.sign(g), atol=1e-7)
