"""Learned mode: predict H/N on the fine mesh, compute exactly only the flagged points.

The reference evaluates the norm and energy kernels at every point of the
Euler x gauge mesh (Codes/PNAMP/PNAMP_Kernel3D.f90:178-260). Per (q, q') pair
this mode instead

 1. computes the kernels exactly on a coarse Euler mesh (4 x 8 x 4, same gauge
    mesh) and interpolates N and H/N to the fine mesh (trigonometric in alpha
    and gamma, polynomial in cos beta);
 2. computes the norm kernel N exactly on the whole fine mesh (the point
    kernel's norm-only mode: the Pfaffian without T22, densities or energy);
 3. runs the network on every fine point: inputs are the deformations of q and
    q', the Euler and gauge angles, the interpolated H/N and N and the exact N;
    outputs are a correction to the interpolated H/N and its uncertainty;
 4. flags the Euler points whose predicted error, weighted by |N| and the
    quadrature weight, is largest, until what is left is below `flag_kev`, and
    computes those exactly (all observables), plus a random held-out sample;
 5. estimates the energy-kernel error left from the held-out sample; above
    `tol_kev` (0.5 keV) for any angular momentum that carries norm, the whole
    fine mesh of that pair is computed exactly (the fallback);
 6. projects N (exact) and H (exact where computed, N x predicted H/N
    elsewhere) onto J, K1, K2 with the ordinary projection kernel;
 7. (`run_gcm`, over the complete pair set of a GCM basis) the Hill-Wheeler
    gate: with N^J exact for every pair, the norm matrix fixes HNDIAG's cutoff
    subspace, and the first-order weight of each pair's H^J block on the lowest
    GCM levels and on each vacuum's E_J follows from the Hill-Wheeler solutions
    of the learned H^J (`gcm.level_weights`). Pairs are sent to the full mesh,
    largest weight x estimated block error first, until the bound on the level
    error left is below `gcm_safety` x `gcm_kev`.
`run_gcm` first takes the same weights from the coarse-mesh kernels alone
(`precheck`): when even the error the flagging aims for would leave more than
`gcm_kev` on the levels, it computes every pair on the full mesh at once, before
any training, norm pass or network work.

Errors are measured in the basis of normalised states: an error dH in
H^J(q, q') is taken relative to sqrt(N^J(q, q) N^J(q', q')), the diagonal
norms, which the mode computes exactly first. The network is trained on
kernels the method computes itself: for each training pair, `train_euler`
random fine Euler points are computed exactly. Its kernels
(`include/pnamp_mlp.h`) are hand-written. N^J and H^J are the outputs of this
mode (the <N>, <Z>, <J^2> and Q2 fields need every point).
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass

import numpy as np
import torch

from .basis import JJMAX, NOBS, Mesh
from .mlp import MLP, _ck, _lib, _p
from .pnamp import NK, PnampContext

NF = 25                     # network inputs (PNAMP_LEARNED_FEATURES)
FIELDS = 5                  # njkk, hjkk, nn, zz, J2 in the projection output
EIGHT_PI2 = 8.0 * math.pi ** 2


# ------------------------------------------------------------------ interpolation
def _trig_basis(x, n):
    """1, cos x, sin x, then sin kx, cos kx for k = 2, 3, ... (first n functions)."""
    cols = [np.ones_like(x)]
    k = 1
    while len(cols) < n:
        a, b = (np.cos(k * x), np.sin(k * x)) if k == 1 else (np.sin(k * x), np.cos(k * x))
        cols.append(a)
        if len(cols) < n:
            cols.append(b)
        k += 1
    return np.stack(cols[:n], axis=-1)


def interp_periodic(xc, xf):
    """Rows: weights of the coarse nodes xc for the value at each xf (period 2 pi)."""
    if len(xc) == 1:
        return np.ones((len(xf), 1))
    V = _trig_basis(np.asarray(xc), len(xc))
    return _trig_basis(np.asarray(xf), len(xc)) @ np.linalg.pinv(V)


def interp_poly(xc, xf):
    """Lagrange interpolation weights through the nodes xc."""
    xc, xf = np.asarray(xc), np.asarray(xf)
    L = np.ones((len(xf), len(xc)))
    for j in range(len(xc)):
        for m in range(len(xc)):
            if m != j:
                L[:, j] *= (xf - xc[m]) / (xc[j] - xc[m])
    return L


def interp_factors(coarse: Mesh, fine: Mesh):
    """The 1-D weights (wb, wa, wg), each [fine nodes, coarse nodes]."""
    ia = interp_periodic(coarse.alpha, fine.alpha)
    ig = interp_periodic(coarse.gamma, fine.gamma)
    ib = interp_poly(np.cos(coarse.beta[:coarse.nbet_used]), np.cos(fine.beta[:fine.nbet_used]))
    return ib, ia, ig


def interp_matrix(coarse: Mesh, fine: Mesh):
    """[P_fine, P_coarse] weights in the Euler order beta outer, alpha, gamma inner."""
    ib, ia, ig = interp_factors(coarse, fine)
    return np.kron(ib, np.kron(ia, ig))


# ------------------------------------------------------------------ configuration
@dataclass
class LearnedConfig:
    coarse: tuple = (4, 8, 4)   # coarse Euler mesh (alpha, beta, gamma)
    width: int = 256
    depth: int = 4
    train_euler: int = 64       # exactly computed Euler points per training pair
    epochs: int = 12
    batch: int = 16384
    lr: float = 1e-3
    flag_kev: float = 0.05      # predicted error left in the unflagged points
    tol_kev: float = 0.5        # held-out estimate above this: full-mesh fallback
    heldout: float = 0.01       # fraction of Euler points held out per pair
    min_heldout: int = 32
    chunk: int = 4              # pairs per device batch
    rel_norm: float = 1e-3      # J checked when its diagonal-norm scale >= rel_norm x the largest
    gcm_kev: float = 1.0        # Hill-Wheeler gate: bound on the GCM-level / E_J error left
    gcm_safety: float = 0.5     # ... aimed at gcm_safety x gcm_kev
    seed: int = 0


# ------------------------------------------------------------------ the mode
class LearnedPNAMP:
    """Learned + mixed PNAMP for one workload (model space, interaction, fine mesh, vacua)."""

    def __init__(self, wl, cfg: LearnedConfig | None = None, form="df64", device="cuda"):
        self.wl = wl
        self.cfg = cfg or LearnedConfig()
        self.dev = torch.device(device)
        fine = wl.mesh
        self.cmesh = Mesh(self.cfg.coarse[0], self.cfg.coarse[1], self.cfg.coarse[2], fine.nfom)
        self.fine = PnampContext(wl.sp, wl.e0, wl.t1b, wl.recs, wl.vbar, fine, q2=None, form=form)
        self.coarse = PnampContext(wl.sp, wl.e0, wl.t1b, wl.recs, wl.vbar, self.cmesh, q2=None, form=form)
        self.nfom = fine.nfom
        self.P, self.Pc, self.G = self.fine.n_euler, self.coarse.n_euler, fine.nfom ** 2
        self.euler = torch.from_numpy(fine.euler_points()).to(self.dev)          # [P, 4]
        self.wts = self.euler[:, 3].contiguous()
        # separable interpolation weights (pnamp_learned_interp): beta, alpha, gamma
        self.wi = [torch.from_numpy(np.ascontiguousarray(w)).to(self.dev) for w in interp_factors(self.cmesh, fine)]
        self.net = MLP(NF, self.cfg.width, self.cfg.depth, 3, seed=self.cfg.seed, device=self.dev)
        self.mean = torch.zeros(NF, dtype=torch.float32, device=self.dev)
        self.inv_std = torch.ones(NF, dtype=torch.float32, device=self.dev)
        self.scale = 1.0
        self.rng = np.random.default_rng(self.cfg.seed)
        self.history = []
        self._diag = {}
        self.last_timing = {}

    def close(self):
        self.fine.close()
        self.coarse.close()

    # ------------------------------------------------------------------ device passes
    def _stream(self):
        return torch.cuda.current_stream().cuda_stream

    def _upload(self, pairs):
        wl = self.wl
        packed = PnampContext.pack_pairs([(*wl.vacua[i], *wl.vacua[j]) for i, j in pairs])
        uv = torch.from_numpy(packed).to(self.dev)
        deform = torch.tensor([[*wl.deform[i], *wl.deform[j]] for i, j in pairs], dtype=torch.float64,
                              device=self.dev)
        return uv, deform

    def _all_items(self, npairs, n_euler):
        p = torch.arange(npairs, dtype=torch.int32, device=self.dev).repeat_interleave(n_euler)
        e = torch.arange(n_euler, dtype=torch.int32, device=self.dev).repeat(npairs)
        return torch.stack([p, e], 1).contiguous()

    def _run_items(self, ctx, uv, npairs, items, z, st, g, outputs):
        ctx.set_outputs(outputs)
        ctx.batch_items_device(npairs, uv.data_ptr(), items.shape[0], items.data_ptr(), z.data_ptr(),
                               st.data_ptr(), g.data_ptr(), self._stream())
        ctx.set_outputs("all")

    def _buffers(self, npairs, n_euler):
        g = torch.zeros((npairs, n_euler, self.G, 4), dtype=torch.float64, device=self.dev)
        z = torch.zeros((npairs, NOBS, n_euler, 2), dtype=torch.float64, device=self.dev)
        st = torch.zeros((npairs, n_euler), dtype=torch.int32, device=self.dev)
        return g, z, st

    def coarse_pass(self, uv, npairs):
        """Exact coarse kernels, interpolated: (H/N, N) [npairs, P, G, 2] each, and nscale [npairs]."""
        Pc, G = self.Pc, self.G
        gc, zc, sc = self._buffers(npairs, Pc)
        self._run_items(self.coarse, uv, npairs, self._all_items(npairs, Pc), zc, sc, gc, "all")
        h_i = torch.empty((npairs, self.P, G, 2), dtype=torch.float64, device=self.dev)
        n_i = torch.empty_like(h_i)
        wb, wa, wg = self.wi
        (fb, cb), (fa, ca), (fg, cg) = wb.shape, wa.shape, wg.shape
        _ck(_lib().pnamp_learned_interp(npairs, cb, ca, cg, fb, fa, fg, G, _p(wb), _p(wa), _p(wg), _p(gc),
                                        _p(h_i), _p(n_i), self._stream()), "pnamp_learned_interp")
        nscale = torch.linalg.vector_norm(gc[..., 0:2], dim=-1).amax(dim=(1, 2))
        return h_i, n_i, nscale.contiguous()

    def features(self, npairs, deform, g, h_i, n_i, nscale, sel=None):
        nsel = 0 if sel is None else sel.shape[0]
        rows = (nsel if sel is not None else npairs * self.P) * self.G
        x = torch.empty((rows, NF), dtype=torch.float32, device=self.dev)
        _ck(_lib().pnamp_learned_features(npairs, self.P, self.nfom, _p(sel), nsel, _p(deform), _p(self.euler),
                                          _p(g), _p(h_i), _p(n_i), _p(nscale), _p(self.mean), _p(self.inv_std),
                                          _p(x), self._stream()), "pnamp_learned_features")
        return x

    def project(self, z, npairs):
        """ZRES [npairs, NOBS, P, 2] -> (njkk, hjkk) complex [npairs, J, K1, K2] on the host."""
        out = torch.zeros((npairs, FIELDS, JJMAX + 1, NK, NK, 2), dtype=torch.float64, device=self.dev)
        self.fine.project_device(npairs, z.data_ptr(), out.data_ptr(), False, self._stream())
        o = out.cpu().numpy()
        c = o[..., 0] + 1j * o[..., 1]
        return c[:, 0], c[:, 1]

    # ------------------------------------------------------------------ training
    def exact_rows(self, pairs, n_euler):
        """Exact kernels at `n_euler` random fine Euler points of each pair -> (x raw, residual, weight).

        x is the network input (unstandardised), residual = exact H/N minus
        the interpolated H/N (MeV, [rows, 2]), weight = |N| / the pair's scale."""
        cfg = self.cfg
        P = self.P
        xs, rs, ws = [], [], []
        mean, inv_std = self.mean, self.inv_std
        self.mean = torch.zeros(NF, dtype=torch.float32, device=self.dev)     # raw inputs
        self.inv_std = torch.ones(NF, dtype=torch.float32, device=self.dev)
        for s in range(0, len(pairs), cfg.chunk):
            chunk = pairs[s:s + cfg.chunk]
            npairs = len(chunk)
            uv, deform = self._upload(chunk)
            h_i, n_i, nscale = self.coarse_pass(uv, npairs)
            sel = np.concatenate([np.stack([np.full(n_euler, k), self.rng.choice(P, n_euler, replace=False)], 1)
                                  for k in range(npairs)]).astype(np.int32)
            sel_d = torch.from_numpy(sel).to(self.dev)
            g, z, st = self._buffers(npairs, P)
            self._run_items(self.fine, uv, npairs, sel_d, z, st, g, "all")
            xs.append(self.features(npairs, deform, g, h_i, n_i, nscale, sel_d))
            pk, ek = sel_d[:, 0].long(), sel_d[:, 1].long()
            rs.append((g[pk, ek, :, 2:4] - h_i[pk, ek]).reshape(-1, 2))
            ws.append((torch.linalg.vector_norm(g[pk, ek, :, 0:2], dim=-1) / nscale[pk, None]).reshape(-1))
        self.mean, self.inv_std = mean, inv_std
        return torch.cat(xs), torch.cat(rs), torch.cat(ws)

    def fit(self, x_raw, resid, weight, epochs=None, val_frac=0.1):
        """Standardise the inputs, scale the targets, train with Adam; returns the loss history.

        The mean and the uncertainty are fitted jointly (Gaussian likelihood,
        |N|-weighted rows). A random `val_frac` of the rows is held out; the
        parameters with the lowest held-out loss are kept (early stopping):
        with the output layer starting at zero, the kept network is never
        worse on held-out rows than the interpolation alone."""
        cfg = self.cfg
        epochs = cfg.epochs if epochs is None else epochs
        self.mean = x_raw.mean(0).float().contiguous()
        std = x_raw.std(0).float()
        self.inv_std = torch.where(std > 1e-6, 1.0 / std, torch.ones_like(std)).contiguous()
        x = ((x_raw - self.mean) * self.inv_std).contiguous()
        wn = weight / weight.mean()
        self.scale = float(torch.sqrt((wn * (resid ** 2).sum(1)).mean() / 2.0).clamp_min(1e-9))
        y = (resid / self.scale).float().contiguous()
        w = wn.float().contiguous()
        gen = torch.Generator(device=self.dev)
        gen.manual_seed(cfg.seed)
        perm = torch.randperm(x.shape[0], device=self.dev, generator=gen)
        nval = int(val_frac * x.shape[0])
        vi, ti = perm[:nval], perm[nval:]
        xv, yv, wv = x[vi].contiguous(), y[vi].contiguous(), w[vi].contiguous()
        xt, yt, wt = x[ti].contiguous(), y[ti].contiguous(), w[ti].contiguous()
        rows = xt.shape[0]
        nb = max(1, rows // cfg.batch)
        bs = rows // nb

        def val_loss():
            if nval == 0:
                return 0.0
            out = self.net.predict(xv)
            s = out[:, 2].clamp(-12.0, 6.0)
            e2 = ((yv - out[:, :2]) ** 2).sum(1)
            return float((wv * (0.5 * e2 * torch.exp(-2.0 * s) + 2.0 * s)).mean())

        best, best_params = val_loss(), self.net.params.clone()
        hist = []
        for ep in range(epochs):
            order = torch.randperm(rows, device=self.dev, generator=gen)
            lr = cfg.lr * (0.5 * (1 + math.cos(math.pi * ep / epochs)))       # cosine decay
            tot = torch.zeros((), device=self.dev)
            for b in range(nb):
                idx = order[b * bs:(b + 1) * bs]
                tot += self.net.train_step(xt[idx].contiguous(), yt[idx].contiguous(), wt[idx].contiguous(), lr=lr)
            hist.append(float(tot) / nb)
            v = val_loss()
            if v < best:
                best, best_params = v, self.net.params.clone()
        self.net.params.copy_(best_params)
        self.val_loss = best
        self.history += hist
        return hist

    def train(self, pairs):
        """Generate exact training rows for `pairs` and fit; returns timing and loss."""
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        x, r, w = self.exact_rows(pairs, self.cfg.train_euler)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        hist = self.fit(x, r, w)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        return {"pairs": len(pairs), "rows": int(x.shape[0]),
                "exact_points": len(pairs) * (self.cfg.train_euler + self.Pc) * self.G,
                "data_s": t1 - t0, "fit_s": t2 - t1, "loss_first": hist[0], "loss_last": hist[-1],
                "target_scale_MeV": self.scale}

    def validation_rms(self, pairs, n_euler=32):
        """|N|-weighted RMS error of H/N (MeV) at fresh exact points: (interpolation alone, with the network)."""
        x_raw, r, w = self.exact_rows(pairs, n_euler)
        x = ((x_raw - self.mean) * self.inv_std).contiguous()
        out = self.net.predict(x)
        mu = out[:, :2].double() * self.scale
        wn = w / w.mean()
        rms_i = float(torch.sqrt((wn * (r ** 2).sum(1)).mean()))
        rms_n = float(torch.sqrt((wn * ((r - mu) ** 2).sum(1)).mean()))
        return rms_i, rms_n

    # ------------------------------------------------------------------ inference
    def diagonal_norms(self, vacua):
        """max_K |N^J_KK(q, q)| per J for each vacuum q (exact; norm-only passes), cached."""
        todo = [q for q in vacua if q not in self._diag]
        P = self.P
        for s in range(0, len(todo), self.cfg.chunk):
            qs = todo[s:s + self.cfg.chunk]
            uv, _ = self._upload([(q, q) for q in qs])
            npairs = len(qs)
            g, z, st = self._buffers(npairs, P)
            self._run_items(self.fine, uv, npairs, self._all_items(npairs, P), z, st, g, "norm")
            nj, _ = self.project(z, npairs)
            for k, q in enumerate(qs):
                self._diag[q] = {J: float(np.abs(np.diagonal(nj[k, J])).max()) for J in range(0, JJMAX + 1, 2)}
        return self._diag

    def scales(self, pair):
        """Per J the kernel scale sqrt(N^J(q,q) N^J(q',q')) of a pair, for the J that carry norm.

        An error dH in H^J(q, q') moves the GCM energies by about dH / that
        scale (the kernels in the basis of normalised states), so budgets and
        error estimates are taken relative to it."""
        i, j = pair
        di, dj = self._diag[i], self._diag[j]
        sc = {J: math.sqrt(di[J] * dj[J]) for J in di}
        top = max(sc.values())
        return {J: v for J, v in sc.items() if v > 0 and v >= self.cfg.rel_norm * top}

    def run(self, pairs, collect=False, use_net=True):
        """Learned + mixed kernels of `pairs` -> list of per-pair dicts (njkk, hjkk, counts, estimates).

        use_net=False is the method without the network: the interpolated H/N
        with the training residual's RMS as its uncertainty everywhere."""
        cfg = self.cfg
        P, G = self.P, self.G
        res = []
        tm = {"diag": 0.0, "coarse": 0.0, "norm": 0.0, "network": 0.0, "exact": 0.0, "project": 0.0}

        def mark(key, t):
            torch.cuda.synchronize()
            now = time.perf_counter()
            tm[key] += now - t
            return now

        torch.cuda.synchronize()
        t = time.perf_counter()
        self.diagonal_norms(sorted({q for pr in pairs for q in pr}))
        mark("diag", t)
        for s in range(0, len(pairs), cfg.chunk):
            chunk = pairs[s:s + cfg.chunk]
            npairs = len(chunk)
            torch.cuda.synchronize()
            t = time.perf_counter()
            uv, deform = self._upload(chunk)
            h_i, n_i, nscale = self.coarse_pass(uv, npairs)
            t = mark("coarse", t)
            g, z, st = self._buffers(npairs, P)
            self._run_items(self.fine, uv, npairs, self._all_items(npairs, P), z, st, g, "norm")
            t = mark("norm", t)
            if use_net:
                x = self.features(npairs, deform, g, h_i, n_i, nscale)
                out = self.net.predict(x, batch=1 << 17)
                del x
            else:
                out = torch.zeros((npairs * P * G, 3), dtype=torch.float32, device=self.dev)
            hp = torch.empty((npairs * P * G, 2), dtype=torch.float64, device=self.dev)
            imp = torch.empty((npairs, P), dtype=torch.float64, device=self.dev)
            _ck(_lib().pnamp_learned_assemble(npairs, P, G, _p(g), _p(h_i), _p(out), float(self.scale),
                                              _p(self.wts), _p(z), _p(imp), _p(hp), self._stream()),
                "pnamp_learned_assemble")
            del out
            t = mark("network", t)
            # flag by predicted error; hold out a random sample of the rest
            imp_h = imp.cpu().numpy()
            budgets = [self.scales(pr) for pr in chunk]
            sel, flagged, held = [], [], []
            for k in range(npairs):
                use = budgets[k]
                B = cfg.flag_kev * 1e-3 * min(v / (2 * J + 1) for J, v in use.items()) if use else 0.0
                order = np.argsort(-imp_h[k])
                tail = np.cumsum((imp_h[k][order] ** 2)[::-1])[::-1]      # error left if flagging [0, m)
                ok = tail <= B * B
                m = int(np.argmax(ok)) if ok.any() else P
                fl = order[:m]
                rest = order[m:]
                nh = min(len(rest), max(cfg.min_heldout, int(round(cfg.heldout * P))))
                ho = self.rng.choice(rest, nh, replace=False) if nh else np.zeros(0, dtype=np.int64)
                flagged.append(fl)
                held.append(ho)
                sel.append(np.stack([np.full(len(fl) + len(ho), k), np.concatenate([fl, ho])], 1))
            sel = torch.from_numpy(np.concatenate(sel).astype(np.int32)).to(self.dev)
            zh_pred = z[:, 6].clone()
            if sel.shape[0]:
                self._run_items(self.fine, uv, npairs, sel, z, st, g, "all")
            # held-out estimate of the energy-kernel error left; fallback above tol
            err = torch.linalg.vector_norm(zh_pred - z[:, 6], dim=-1) * self.wts / EIGHT_PI2     # [npairs, P]
            err_h = err.cpu().numpy()
            fb_sel, info = [], []
            for k in range(npairs):
                ho = held[k]
                n_rest = P - len(flagged[k])
                est = math.sqrt(n_rest / max(len(ho), 1) * float(np.sum(err_h[k][ho] ** 2))) if len(ho) else 0.0
                use = budgets[k]
                est_kev = max(((2 * J + 1) * est / v for J, v in use.items()), default=0.0) * 1e3
                fallback = est_kev > cfg.tol_kev
                if fallback:
                    done = np.zeros(P, bool)
                    done[flagged[k]] = True
                    done[ho] = True
                    rest = np.nonzero(~done)[0]
                    fb_sel.append(np.stack([np.full(len(rest), k), rest], 1))
                info.append({"flagged": int(len(flagged[k])), "heldout": int(len(ho)), "est_err_keV": est_kev,
                             "est_err_MeV": est,
                             "fallback": bool(fallback),
                             "heldout_err_rms": float(np.sqrt(np.mean(err_h[k][ho] ** 2))) if len(ho) else 0.0})
            if fb_sel:
                fb = torch.from_numpy(np.concatenate(fb_sel).astype(np.int32)).to(self.dev)
                self._run_items(self.fine, uv, npairs, fb, z, st, g, "all")
            t = mark("exact", t)
            nj, hj = self.project(z, npairs)
            t = mark("project", t)
            for k in range(npairs):
                r = {"pair": tuple(chunk[k]), "njkk": nj[k], "hjkk": hj[k], **info[k],
                     "exact_euler": int(P if info[k]["fallback"] else info[k]["flagged"] + info[k]["heldout"])}
                if collect:
                    r["zres"] = z[k].cpu().numpy()
                res.append(r)
        self.last_timing = tm
        return res

    def coarse_kernels(self, pairs):
        """Projected N^J, H^J of `pairs` from the exact coarse-mesh kernels alone (cheap: the
        coarse mesh has P_coarse / P_fine of the points), as per-pair dicts."""
        out = []
        for s in range(0, len(pairs), self.cfg.chunk):
            chunk = pairs[s:s + self.cfg.chunk]
            npairs = len(chunk)
            uv, _ = self._upload(chunk)
            z = torch.zeros((npairs, NOBS, self.Pc, 2), dtype=torch.float64, device=self.dev)
            st = torch.zeros((npairs, self.Pc), dtype=torch.int32, device=self.dev)
            self.coarse.batch_device(npairs, uv.data_ptr(), z.data_ptr(), st.data_ptr(), self._stream())
            o = torch.zeros((npairs, FIELDS, JJMAX + 1, NK, NK, 2), dtype=torch.float64, device=self.dev)
            self.coarse.project_device(npairs, z.data_ptr(), o.data_ptr(), False, self._stream())
            c = o.cpu().numpy()
            c = c[..., 0] + 1j * c[..., 1]
            out += [{"pair": tuple(chunk[k]), "njkk": c[k, 0], "hjkk": c[k, 1]} for k in range(npairs)]
        return out

    def precheck(self, pairs, nvac, jvals=(0, 2, 4, 6), eps=1e-5, nlev=3):
        """Bound on the GCM-level error the learned kernels could reach, before any fine-mesh work.

        The Hill-Wheeler weights come from the coarse-mesh kernels; each pair's H^J error is
        taken at the level the flagging aims for (flag_kev in the basis of normalised states,
        times sqrt(N^J(q,q) N^J(q',q')) from the coarse diagonal norms), so the bound is what
        the mode achieves at best. Returns (bound in keV, coarse kernels)."""
        from .gcm import diagonal_norms, level_error_bound, level_weights
        ck = self.coarse_kernels(pairs)
        W = level_weights(ck, pairs, nvac, jvals, eps, nlev)
        bound = level_error_bound(W, pairs, diagonal_norms(ck, pairs, jvals), self.cfg.flag_kev, jvals)
        return bound, ck

    def run_gcm(self, pairs, nvac, jvals=(0, 2, 4, 6), eps=1e-5, nlev=3, exact_ctx=None, train_pairs=None):
        """`run` over the complete pair set of `nvac` vacua, then the Hill-Wheeler gate.

        First `precheck`: when even the flagging's target error would leave more than
        gcm_kev on the GCM levels, every pair goes to the full mesh at once (no training, no
        norm pass, no network), so the mode costs the exact quadrature plus the coarse pass.
        Otherwise the network is trained on `train_pairs` (if given) and the mode runs.

        Each pair's estimated H^J block error is (2J+1)^2 x its held-out estimate (the
        spectral norm of a (2J+1)^2 block whose entries are each at most (2J+1) x the
        Euler-summed error; 0 for pairs computed on the full mesh). The gate sends pairs
        to the full mesh, the one with the largest weight x error first, until
        max_J sum_pairs weight x error <= gcm_safety x gcm_kev, and recomputes them with
        `exact_ctx` (a context of the fine mesh; None: this mode's own, in its form).
        Returns (per-pair results, gate record)."""
        from .gcm import level_weights
        cfg = self.cfg
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pre, _ = self.precheck(pairs, nvac, jvals, eps, nlev)
        torch.cuda.synchronize()
        tp = time.perf_counter()
        if pre > cfg.gcm_kev:
            res = [dict(r, fallback=True, gated=True, exact_euler=self.P, est_err_MeV=0.0)
                   for r in self.exact(pairs, ctx=exact_ctx)]
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            self.last_timing = {"precheck": tp - t0, "exact": t1 - tp}
            return res, {"precheck_bound_keV": pre, "bound_before_keV": None, "bound_after_keV": 0.0,
                         "gated_pairs": len(pairs), "fallback_pairs": 0, "run_s": t1 - t0, "gate_s": 0.0,
                         "precheck_s": tp - t0, "exact_s": t1 - tp, "training": None,
                         "exact_fraction": 1.0, "decision": "all pairs exact: the precheck bound exceeds gcm_kev"}
        train_rec = self.train(train_pairs) if train_pairs else None
        res = self.run(pairs)
        t1 = time.perf_counter()
        W = level_weights(res, pairs, nvac, jvals, eps, nlev)
        est = np.array([0.0 if r["fallback"] else r["est_err_MeV"] for r in res])
        err = {J: W[J] * (2 * J + 1) ** 2 * est for J in jvals}
        bound = lambda: max(float(err[J].sum()) for J in jvals) * 1e3
        b0 = bound()
        target = cfg.gcm_safety * cfg.gcm_kev
        gated = []
        while bound() > target:
            worst = max(jvals, key=lambda J: err[J].sum())
            p = int(np.argmax(err[worst]))
            if err[worst][p] == 0.0:
                break
            gated.append(p)
            for J in jvals:
                err[J][p] = 0.0
        if gated:
            gp = [pairs[p] for p in gated]
            ex = self.exact(gp, ctx=exact_ctx)
            for p, e in zip(gated, ex):
                res[p]["hjkk"] = e["hjkk"]
                res[p]["gated"] = True
                res[p]["exact_euler"] = self.P
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        rec = {"precheck_bound_keV": pre, "bound_before_keV": b0, "bound_after_keV": bound(),
               "gated_pairs": len(gated), "decision": "learned, with the gate",
               "fallback_pairs": int(sum(r["fallback"] for r in res if not r.get("gated"))),
               "run_s": t1 - t0, "gate_s": t2 - t1, "training": train_rec,
               "exact_fraction": float(sum(r["exact_euler"] for r in res)) / (self.P * len(res))}
        return res, rec

    # ------------------------------------------------------------------ the plain method
    def exact(self, pairs, ctx=None):
        """Every fine point exact (the plain quadrature) -> list of per-pair dicts (njkk, hjkk).

        ctx: a context of the fine mesh to compute with (None: this mode's own)."""
        ctx = ctx or self.fine
        out = []
        P = self.P
        for s in range(0, len(pairs), self.cfg.chunk):
            chunk = pairs[s:s + self.cfg.chunk]
            npairs = len(chunk)
            uv, _ = self._upload(chunk)
            z = torch.zeros((npairs, NOBS, P, 2), dtype=torch.float64, device=self.dev)
            st = torch.zeros((npairs, P), dtype=torch.int32, device=self.dev)
            ctx.batch_device(npairs, uv.data_ptr(), z.data_ptr(), st.data_ptr(), self._stream())
            nj, hj = self.project(z, npairs)
            out += [{"pair": tuple(c), "njkk": nj[k], "hjkk": hj[k]} for k, c in enumerate(chunk)]
        return out


def energy_errors_kev(learned, exact, nvac=None, pairs=None, rel_norm=1e-3):
    """Errors of the learned kernels against the full quadrature, in keV.

    Per pair: max over J, K1, K2 of |H^J_a - H^J_b| / sqrt(N^J(q,q) N^J(q',q'))
    (the energy-kernel error in the basis of normalised states, over the J that
    carry norm), using the exact diagonal norms max_K |N^J_KK|. With the
    complete pair set of `nvac` vacua: the lowest GCM levels per J and each
    vacuum's K-mixed E_J.
    """
    from .gcm import compare_levels, gcm_levels
    diag = {}
    for b in exact:
        i, j = b["pair"]
        if i == j:
            diag[i] = {J: float(np.abs(np.diagonal(b["njkk"][J])).max()) for J in range(0, JJMAX + 1, 2)}
    worst = 0.0
    per = []
    for a, b in zip(learned, exact):
        i, j = b["pair"]
        w = 0.0
        if i in diag and j in diag:
            sc = {J: math.sqrt(diag[i][J] * diag[j][J]) for J in diag[i]}
            top = max(sc.values())
            for J, v in sc.items():
                if v > 0 and v >= rel_norm * top:
                    w = max(w, float(np.abs(a["hjkk"][J] - b["hjkk"][J]).max()) / v * 1e3)
        per.append(w)
        worst = max(worst, w)
    out = {"max_kernel_EJ_err_keV": worst, "per_pair_keV": per}
    if nvac is not None and pairs is not None:
        la = gcm_levels([{"njkk": r["njkk"], "hjkk": r["hjkk"]} for r in learned], pairs, nvac)
        lb = gcm_levels([{"njkk": r["njkk"], "hjkk": r["hjkk"]} for r in exact], pairs, nvac)
        dl, dq = compare_levels(la, lb)
        out["gcm_levels_err_keV"] = 1e3 * dl
        out["EJ_per_vacuum_err_keV"] = 1e3 * dq
    return out
