"""Host side of the learned mode's network: an FP32 MLP on the hand-written kernels.

The layers, loss and optimiser run only through `include/pnamp_mlp.h`
(`sccm_gb300/csrc/mlp_kernels.cu`); torch provides device memory and streams.
Architecture: inputs -> 4 hidden layers of width 256 (tanh) -> 3 outputs
(mean of the real and imaginary target, log sigma), trained with the
heteroscedastic Gaussian loss and Adam. No reference counterpart (the
reference has no learned component).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from .pnamp import load_library

MLP_EXPORTS = ("pnamp_mlp_linear_forward", "pnamp_mlp_work_floats", "pnamp_mlp_linear_backward",
               "pnamp_mlp_loss_blocks", "pnamp_mlp_gauss_loss", "pnamp_mlp_adam", "pnamp_learned_features",
               "pnamp_learned_assemble", "pnamp_learned_interp")

_bound = False


def _lib():
    global _bound
    lib = load_library()
    if not _bound:
        vp, i, f = C.c_void_p, C.c_int, C.c_float
        lib.pnamp_mlp_linear_forward.argtypes = [vp, vp, vp, vp, i, i, i, i, vp]
        lib.pnamp_mlp_work_floats.argtypes = [i, i, i]
        lib.pnamp_mlp_work_floats.restype = C.c_longlong
        lib.pnamp_mlp_linear_backward.argtypes = [vp, vp, vp, vp, vp, vp, vp, i, i, i, i, vp, vp]
        lib.pnamp_mlp_loss_blocks.argtypes = [i]
        lib.pnamp_mlp_gauss_loss.argtypes = [vp, vp, vp, i, i, vp, vp, vp]
        lib.pnamp_mlp_adam.argtypes = [vp, vp, vp, vp, C.c_longlong, f, f, f, f, i, vp]
        lib.pnamp_learned_features.argtypes = [i, i, i, vp, C.c_longlong] + [vp] * 10
        lib.pnamp_learned_assemble.argtypes = [i, i, i, vp, vp, vp, C.c_double, vp, vp, vp, vp, vp]
        lib.pnamp_learned_interp.argtypes = [i] * 8 + [vp] * 7
        _bound = True
    return lib


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(None)


def _ck(rc, where):
    if rc != 0:
        raise RuntimeError(f"{where} failed (code {rc})")


class MLP:
    """Parameters in one flat FP32 device buffer: per layer W [out][in] then b [out]."""

    def __init__(self, n_in, width=256, depth=4, n_out=3, seed=0, device="cuda", zero_output=True):
        self.dims = [n_in] + [width] * depth + [n_out]
        self.device = torch.device(device)
        sizes = [(self.dims[k + 1], self.dims[k]) for k in range(len(self.dims) - 1)]
        self.offsets = []
        off = 0
        for (o, i) in sizes:
            self.offsets.append((off, off + o * i))
            off += o * i + o
        self.n_params = off
        rng = np.random.default_rng(seed)
        flat = np.zeros(off, dtype=np.float32)
        for k, (o, i) in enumerate(sizes[:-1] if zero_output else sizes):
            w0, b0 = self.offsets[k]
            lim = np.sqrt(6.0 / (i + o))                     # Glorot uniform
            flat[w0:b0] = rng.uniform(-lim, lim, o * i).astype(np.float32)
        # zero_output: the output layer starts at zero, so an untrained network predicts 0
        # (no correction to the interpolation, sigma = 1)
        self.params = torch.from_numpy(flat).to(self.device)
        self.grads = torch.zeros_like(self.params)
        self.m = torch.zeros_like(self.params)
        self.v = torch.zeros_like(self.params)
        self.step = 0
        self._rows = -1

    def layer(self, k, t=None):
        t = self.params if t is None else t
        o, i = self.dims[k + 1], self.dims[k]
        w0, b0 = self.offsets[k]
        return t[w0:b0].view(o, i), t[b0:b0 + o]

    def state(self):
        return self.params.detach().cpu().numpy().copy()

    def load(self, flat):
        self.params.copy_(torch.as_tensor(np.asarray(flat, dtype=np.float32), device=self.device))

    # ------------------------------------------------------------------
    def _buffers(self, rows):
        if rows == self._rows:
            return
        L = len(self.dims) - 1
        self.acts = [None] + [torch.empty((rows, self.dims[k + 1]), dtype=torch.float32, device=self.device)
                              for k in range(L)]
        self.dacts = [torch.empty((rows, self.dims[k]), dtype=torch.float32, device=self.device)
                      for k in range(L + 1)]
        lib = _lib()
        wf = max(lib.pnamp_mlp_work_floats(rows, self.dims[k], self.dims[k + 1]) for k in range(L))
        self.work = torch.empty(int(wf), dtype=torch.float32, device=self.device)
        self.loss_part = torch.empty(lib.pnamp_mlp_loss_blocks(rows), dtype=torch.float32, device=self.device)
        self._rows = rows

    def forward(self, x, stream=None):
        """x: float32 [rows, n_in] on the device -> [rows, n_out] (a view of an internal buffer)."""
        rows = x.shape[0]
        self._buffers(rows)
        st = (stream or torch.cuda.current_stream()).cuda_stream
        lib = _lib()
        self.acts[0] = x
        L = len(self.dims) - 1
        for k in range(L):
            W, b = self.layer(k)
            _ck(lib.pnamp_mlp_linear_forward(_p(self.acts[k]), _p(W), _p(b), _p(self.acts[k + 1]), rows,
                                             self.dims[k], self.dims[k + 1], 1 if k < L - 1 else 0,
                                             C.c_void_p(st)), "pnamp_mlp_linear_forward")
        return self.acts[L]

    def backward(self, dout, stream=None):
        """dout [rows, n_out]: gradient of the loss w.r.t. the outputs; fills self.grads."""
        rows = dout.shape[0]
        st = (stream or torch.cuda.current_stream()).cuda_stream
        lib = _lib()
        L = len(self.dims) - 1
        self.dacts[L] = dout
        for k in range(L - 1, -1, -1):
            W, _ = self.layer(k)
            dW, db = self.layer(k, self.grads)
            dX = self.dacts[k] if k > 0 else None
            _ck(lib.pnamp_mlp_linear_backward(_p(self.acts[k]), _p(W), _p(self.acts[k + 1]), _p(self.dacts[k + 1]),
                                              _p(dW), _p(db), _p(dX), rows, self.dims[k], self.dims[k + 1],
                                              1 if k < L - 1 else 0, _p(self.work), C.c_void_p(st)),
                "pnamp_mlp_linear_backward")

    def loss_grad(self, out, y, w=None, mode=0, stream=None):
        """Gaussian loss of `out` [rows, 3] against y [rows, 2] (row weights w); returns (loss tensor, dout).

        mode 0: mean and uncertainty; 1: least squares on the mean; 2: the uncertainty only."""
        rows = out.shape[0]
        st = (stream or torch.cuda.current_stream()).cuda_stream
        dout = torch.empty_like(out)
        lp = self.loss_part
        _ck(_lib().pnamp_mlp_gauss_loss(_p(out), _p(y), _p(w), rows, mode, _p(dout), _p(lp), C.c_void_p(st)),
            "pnamp_mlp_gauss_loss")
        return lp.sum(), dout

    def adam(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, stream=None):
        self.step += 1
        st = (stream or torch.cuda.current_stream()).cuda_stream
        _ck(_lib().pnamp_mlp_adam(_p(self.params), _p(self.grads), _p(self.m), _p(self.v), self.n_params,
                                  lr, beta1, beta2, eps, self.step, C.c_void_p(st)), "pnamp_mlp_adam")

    def train_step(self, x, y, w=None, lr=1e-3, mode=0):
        out = self.forward(x)
        loss, dout = self.loss_grad(out, y, w, mode)
        self.backward(dout)
        self.adam(lr)
        return loss

    def predict(self, x, batch=1 << 16):
        """Outputs for all rows of x, in batches (inference)."""
        outs = []
        for s in range(0, x.shape[0], batch):
            outs.append(self.forward(x[s:s + batch]).clone())
        return torch.cat(outs) if outs else torch.empty((0, self.dims[-1]), device=self.device)
