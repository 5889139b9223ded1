"""The learned mode's hand-written FP32 network kernels against the CPU oracle (float64).

Tolerances are FP32 round-off for these sizes: forward 2e-5, gradients 1e-4
relative to the largest entry of each layer's gradient.
"""
import numpy as np
import pytest
import torch

from oracle import mlp_oracle as mo
from sccm_gb300.mlp import MLP

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    rng = np.random.default_rng(11)
    rows, n_in = 1000, 21                      # ragged against the 64-row tiles and 16-wide k steps
    net = MLP(n_in, width=256, depth=4, seed=3, zero_output=False)
    x = rng.normal(size=(rows, n_in)).astype(np.float32)
    y = rng.normal(size=(rows, 2)).astype(np.float32)
    w = rng.uniform(0.2, 2.0, rows).astype(np.float32)
    return net, x, y, w


def test_forward_matches_oracle(setup):
    net, x, _, _ = setup
    out = net.forward(torch.from_numpy(x).cuda()).cpu().numpy()
    ref = mo.forward(net.state(), net.dims, x)[-1]
    assert np.abs(out - ref).max() <= 2e-5 * np.abs(ref).max()


def test_loss_and_gradients_match_oracle(setup):
    net, x, y, w = setup
    dx, dy, dw = (torch.from_numpy(a).cuda() for a in (x, y, w))
    out = net.forward(dx)
    loss, dout = net.loss_grad(out, dy, dw)
    net.backward(dout)
    flat = net.state()
    acts = mo.forward(flat, net.dims, x)
    rl, rdout = mo.gauss_loss(acts[-1], y, w)
    assert abs(float(loss) - rl) <= 1e-5 * abs(rl)
    assert np.abs(dout.cpu().numpy() - rdout).max() <= 1e-4 * np.abs(rdout).max()
    g = net.grads.cpu().numpy()
    rg = mo.backward(flat, net.dims, acts, rdout)
    for k in range(len(net.dims) - 1):
        w0, b0 = net.offsets[k]
        o = net.dims[k + 1]
        for lo, hi in ((w0, b0), (b0, b0 + o)):
            sc = np.abs(rg[lo:hi]).max()
            assert np.abs(g[lo:hi] - rg[lo:hi]).max() <= 1e-4 * sc, (k, lo)


@pytest.mark.parametrize("mode", [1, 2])
def test_loss_modes_match_oracle(setup, mode):
    net, x, y, w = setup
    dx, dy, dw = (torch.from_numpy(a).cuda() for a in (x, y, w))
    out = net.forward(dx)
    loss, dout = net.loss_grad(out, dy, dw, mode=mode)
    rl, rdout = mo.gauss_loss(out.cpu().numpy().astype(np.float64), y, w, mode=mode)
    assert abs(float(loss) - rl) <= 1e-5 * abs(rl)
    assert np.abs(dout.cpu().numpy() - rdout).max() <= 1e-4 * np.abs(rdout).max()


def test_adam_step_matches_oracle(setup):
    net, x, y, w = setup
    p0, g0 = net.state().astype(np.float64), net.grads.cpu().numpy().astype(np.float64)
    m0, v0 = net.m.cpu().numpy().astype(np.float64), net.v.cpu().numpy().astype(np.float64)
    step = net.step + 1
    net.adam(lr=1e-3)
    ref, _, _ = mo.adam(p0, g0, m0, v0, step, lr=1e-3)
    assert np.abs(net.state() - ref).max() <= 1e-6


def test_training_fits_a_smooth_function():
    rng = np.random.default_rng(2)
    x = rng.uniform(-1, 1, size=(8192, 4)).astype(np.float32)
    y = np.stack([np.sin(2 * x[:, 0]) * x[:, 1], np.cos(x[:, 2] + x[:, 3])], 1).astype(np.float32)
    net = MLP(4, width=64, depth=2, seed=1, zero_output=False)
    dx, dy = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    first = float(net.train_step(dx, dy, lr=3e-3))
    for _ in range(800):
        last = float(net.train_step(dx, dy, lr=3e-3))
    out = net.forward(dx).cpu().numpy()
    assert last < first - 3.0
    assert np.sqrt(np.mean((out[:, :2] - y) ** 2)) < 0.05
