"""ORACLE — test infrastructure only (not part of the product path).

CPU (numpy, float64) restatement of the learned mode's network for checking
the hand-written GPU kernels of `include/pnamp_mlp.h`: dense layers with tanh,
the heteroscedastic Gaussian loss and its gradient, and the Adam update. The
network is not part of the reference (which evaluates every mesh point
exactly, Codes/PNAMP/PNAMP_Kernel3D.f90:178-260), so there is no reference
file to follow; the formulas are the textbook ones:
  * layer: Y = act(X W^T + b), dZ = dY * act'(Z), dW = dZ^T X, db = sum_r dZ, dX = dZ W
  * loss: mean_r w_r [ |y_r - mu_r|^2 e^{-2 s_r} / 2 + 2 s_r ], s clamped to [-12, 6]
    (mode 1: s = 0 and no gradient to s; mode 2: no gradient to mu)
  * Adam (Kingma & Ba 2015) with bias correction.
"""
from __future__ import annotations

import numpy as np


def unpack(flat, dims):
    """Flat parameter vector (per layer W [out][in] then b [out]) -> [(W, b)]."""
    out, off = [], 0
    for k in range(len(dims) - 1):
        i, o = dims[k], dims[k + 1]
        W = flat[off:off + o * i].reshape(o, i)
        off += o * i
        b = flat[off:off + o]
        off += o
        out.append((W, b))
    return out


def forward(flat, dims, x):
    """Returns the list of activations [x, h1, ..., out]."""
    acts = [np.asarray(x, dtype=np.float64)]
    layers = unpack(np.asarray(flat, dtype=np.float64), dims)
    for k, (W, b) in enumerate(layers):
        z = acts[-1] @ W.T + b
        acts.append(np.tanh(z) if k < len(layers) - 1 else z)
    return acts


def gauss_loss(out, y, w=None, mode=0):
    """mode 0: gradients to mu and s; 1: s = 0, no gradient to s; 2: gradient to s only."""
    rows = out.shape[0]
    w = np.ones(rows) if w is None else np.asarray(w, dtype=np.float64)
    s_raw = out[:, 2]
    s = np.zeros(rows) if mode == 1 else np.clip(s_raw, -12.0, 6.0)
    er, ei = y[:, 0] - out[:, 0], y[:, 1] - out[:, 1]
    iv = np.exp(-2.0 * s)
    e2 = er * er + ei * ei
    loss = np.sum(w * (0.5 * e2 * iv + 2.0 * s)) / rows
    g = w / rows
    ds = np.where((s_raw > -12.0) & (s_raw < 6.0), g * (2.0 - e2 * iv), 0.0)
    dm = 0.0 if mode == 2 else 1.0
    dout = np.stack([-g * er * iv * dm, -g * ei * iv * dm, ds * (mode != 1)], axis=1)
    return loss, dout


def backward(flat, dims, acts, dout):
    """Gradient of the loss w.r.t. the flat parameters, given the activations and d loss / d out."""
    layers = unpack(np.asarray(flat, dtype=np.float64), dims)
    grads = []
    d = dout
    for k in range(len(layers) - 1, -1, -1):
        W, _ = layers[k]
        if k < len(layers) - 1:
            d = d * (1.0 - acts[k + 1] ** 2)
        grads.append((d.T @ acts[k], d.sum(axis=0)))
        d = d @ W
    grads.reverse()
    return np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])


def adam(p, g, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v
