"""Hill-Wheeler (GCM) solve on projected kernels: the consumer of PNAMP's output.

`hndiag` restates HNDIAG (Codes/GCM/GCM_HNDiag.f90:2-103): diagonalise the norm
matrix, keep the natural states whose eigenvalue is at least `eps` times the
largest (the driver's cutoff `1.e-5`, Codes/exec/GCM.sh:59), and diagonalise
N^-1/2 H N^-1/2 in that subspace. `gcm_levels` assembles, for each even J, the
basis (q, K), K = -J..J, from the projected N^J_{K1K2}(q, q') and
H^J_{K1K2}(q, q') of every computed pair (q <= q'; the other triangle by
Hermiticity, N^J_{K1K2}(q', q) = conj(N^J_{K2K1}(q, q'))) and returns the levels.
Host-side by default: a few matrices of size (number of vacua x (2J+1)).
`hndiag_batch_gpu` solves a batch of such problems on the GPU, one CTA each
(`include/pnamp_gcm.h`, `sccm_gb300/csrc/hw_kernels.cu`); `gcm_levels(..., gpu=True)`
puts every angular momentum and every vacuum's K-mixing of a basis in one launch.
"""
from __future__ import annotations

import numpy as np

from .basis import JJMAX


HW_EXPORTS = ("pnamp_hw_work_bytes", "pnamp_hw_solve")


def _hw_lib():
    import ctypes as C
    from .pnamp import load_library
    lib = load_library()
    if not getattr(lib, "_hw_bound", False):
        vp = C.c_void_p
        lib.pnamp_hw_work_bytes.restype = C.c_longlong
        lib.pnamp_hw_work_bytes.argtypes = [C.c_int, vp]
        lib.pnamp_hw_solve.argtypes = [C.c_int, vp, vp, vp, vp, C.c_double, vp, vp, vp, vp, vp]
        lib._hw_bound = True
    return lib


def hndiag_batch_gpu(problems, eps=1e-5, vectors=False, device="cuda"):
    """HNDIAG for a batch of (H, N) pairs on the GPU, one CTA per problem.

    Returns per problem (E ascending over the kept subspace, number kept, F): F (only with
    `vectors`) holds the solutions f_k in its columns, normalised f_k^+ N f_k = 1."""
    import ctypes as C
    import torch
    lib = _hw_lib()
    dims = np.array([np.asarray(H).shape[0] for H, _ in problems], dtype=np.int32)
    offs = np.zeros(len(problems), dtype=np.int64)
    if len(problems) > 1:
        offs[1:] = np.cumsum(dims.astype(np.int64) ** 2)[:-1]
    tot = int((dims.astype(np.int64) ** 2).sum())
    Hh = np.concatenate([np.ascontiguousarray(H, dtype=np.complex128).ravel() for H, _ in problems]) if tot else \
        np.zeros(1, np.complex128)
    Nh = np.concatenate([np.ascontiguousarray(N, dtype=np.complex128).ravel() for _, N in problems]) if tot else \
        np.zeros(1, np.complex128)
    dev = torch.device(device)
    Hd = torch.from_numpy(Hh.view(np.float64)).to(dev)
    Nd = torch.from_numpy(Nh.view(np.float64)).to(dev)
    E = torch.zeros(max(tot, 1), dtype=torch.float64, device=dev)
    kept = torch.zeros(max(len(problems), 1), dtype=torch.int32, device=dev)
    F = torch.zeros(2 * max(tot, 1), dtype=torch.float64, device=dev) if vectors else None
    nb = lib.pnamp_hw_work_bytes(len(problems), dims.ctypes.data)
    if nb < 0:
        raise ValueError("problem sizes out of range")
    work = torch.empty(max(nb, 1), dtype=torch.uint8, device=dev)
    st = torch.cuda.current_stream(dev).cuda_stream
    # E takes problem b's energies at off[b] (a slot of dim[b]^2 doubles, the first dim[b] used)
    rc = lib.pnamp_hw_solve(len(problems), dims.ctypes.data, offs.ctypes.data, C.c_void_p(Hd.data_ptr()),
                            C.c_void_p(Nd.data_ptr()), float(eps), C.c_void_p(E.data_ptr()),
                            C.c_void_p(kept.data_ptr()), C.c_void_p(F.data_ptr()) if vectors else None,
                            C.c_void_p(work.data_ptr()), C.c_void_p(st))
    if rc != 0:
        raise RuntimeError(f"pnamp_hw_solve failed with code {rc}")
    torch.cuda.synchronize(dev)
    Eh, kh = E.cpu().numpy(), kept.cpu().numpy()
    Fh = F.cpu().numpy().view(np.complex128) if vectors else None
    out = []
    for b, (m, o) in enumerate(zip(dims, offs)):
        k = int(kh[b])
        f = Fh[o:o + m * m].reshape(m, m)[:, :k].copy() if vectors else None
        out.append((Eh[o:o + k].copy(), k, f))
    return out


def hndiag(H, N, eps=1e-5, nos=None):
    """Generalised eigenproblem H f = E N f with the norm cutoff of HNDIAG.

    Returns (E ascending, norm eigenvalues descending, number kept).
    """
    H = 0.5 * (H + H.conj().T)
    N = 0.5 * (N + N.conj().T)
    en, dd = np.linalg.eigh(N)
    order = np.argsort(-en)
    en, dd = en[order], dd[:, order]
    if en.size == 0 or en[0] <= 0:
        return np.array([]), en, 0
    m = 0
    while m < en.size and en[m] / en[0] >= eps:
        m += 1
    if nos is not None:
        m = min(m, nos)
    rr = dd[:, :m] / np.sqrt(en[:m])
    gg = rr.conj().T @ H @ rr
    e = np.linalg.eigvalsh(0.5 * (gg + gg.conj().T))
    return e, en, m


def hw_vectors(H, N, eps=1e-5, nlev=3):
    """Lowest `nlev` Hill-Wheeler solutions f (columns), normalised f^+ N f = 1, of HNDIAG's
    cutoff subspace: f_k = N^-1/2 g_k in the kept natural basis."""
    H = 0.5 * (H + H.conj().T)
    N = 0.5 * (N + N.conj().T)
    en, dd = np.linalg.eigh(N)
    order = np.argsort(-en)
    en, dd = en[order], dd[:, order]
    if en.size == 0 or en[0] <= 0:
        return np.zeros((N.shape[0], 0), complex)
    m = int(np.count_nonzero(en / en[0] >= eps))
    rr = dd[:, :m] / np.sqrt(en[:m])
    gg = rr.conj().T @ H @ rr
    _, v = np.linalg.eigh(0.5 * (gg + gg.conj().T))
    return rr @ v[:, :nlev]


def level_weights(kernels, pairs, nvac, jvals=(0, 2, 4, 6), eps=1e-5, nlev=3):
    """First-order weight of each pair's H^J block on the lowest GCM levels and on E_J.

    A Hermitian error dH moves a level by f^+ dH f (f the normalised Hill-Wheeler
    solution), so |dE| <= sum over pairs (i, j) of c |f_i| |f_j| ||dH^J_ij||, with f_i
    the (2J+1) K components of vacuum i and c = 2 off the diagonal (the block and its
    Hermitian image). The per-vacuum K-mixed E_J (a solution of the diagonal block
    alone) adds |g|^2 on its own pair. Returns {J: weights [len(pairs)]}: the largest
    of these factors over the `nlev` lowest levels and the per-vacuum energies. The
    norm matrix decides the cutoff subspace, so these are known once N^J is exact and
    any approximation of H^J is at hand."""
    out = {}
    for J in jvals:
        d = 2 * J + 1
        sl = slice(JJMAX - J, JJMAX + J + 1)
        Nm = np.zeros((nvac * d, nvac * d), complex)
        Hm = np.zeros_like(Nm)
        for (i, j), k in zip(pairs, kernels):
            for M, f in ((Nm, "njkk"), (Hm, "hjkk")):
                blk = k[f][J, sl, sl]
                M[i * d:(i + 1) * d, j * d:(j + 1) * d] = blk
                if i != j:
                    M[j * d:(j + 1) * d, i * d:(i + 1) * d] = blk.conj().T
        F = hw_vectors(Hm, Nm, eps, nlev)
        amp = np.sqrt((np.abs(F.reshape(nvac, d, -1)) ** 2).sum(1))     # [vacuum, level]
        w = np.zeros(len(pairs))
        for p, (i, j) in enumerate(pairs):
            c = 1.0 if i == j else 2.0
            w[p] = c * float(np.max(amp[i] * amp[j])) if amp.shape[1] else 0.0
        for q in range(nvac):
            if (q, q) not in pairs:
                continue
            g = hw_vectors(Hm[q * d:(q + 1) * d, q * d:(q + 1) * d], Nm[q * d:(q + 1) * d, q * d:(q + 1) * d],
                           eps, 1)
            if g.shape[1]:
                p = pairs.index((q, q))
                w[p] = max(w[p], float(np.sum(np.abs(g[:, 0]) ** 2)))
        out[J] = w
    return out


def diagonal_norms(kernels, pairs, jvals=(0, 2, 4, 6)):
    """max_K |N^J_KK(q, q)| per vacuum q and J, from the diagonal pairs of a pair set."""
    diag = {}
    for (i, j), k in zip(pairs, kernels):
        if i == j:
            diag[i] = {J: float(np.abs(np.diagonal(k["njkk"][J])).max()) for J in jvals}
    return diag


def level_error_bound(W, pairs, diag, err_norm, jvals=(0, 2, 4, 6)):
    """First-order bound on the GCM-level / E_J error (in the units of `err_norm`) when every
    pair's H^J entries carry an error of err_norm in the basis of normalised states, i.e.
    err_norm x sqrt(N^J(q,q) N^J(q',q')) absolute, the (2J+1)-row block's spectral norm
    taken as (2J+1) times that. W: `level_weights` of the same pairs."""
    bound = 0.0
    for J in jvals:
        tot = 0.0
        for p, (i, j) in enumerate(pairs):
            if i in diag and j in diag:
                tot += W[J][p] * (2 * J + 1) * err_norm * np.sqrt(diag[i][J] * diag[j][J])
        bound = max(bound, tot)
    return float(bound)


def assemble(kernels, pairs, nvac, J, field):
    """Matrix over (q, K) of one projected field for angular momentum J."""
    d = 2 * J + 1
    M = np.zeros((nvac * d, nvac * d), complex)
    sl = slice(JJMAX - J, JJMAX + J + 1)
    for (i, j), k in zip(pairs, kernels):
        blk = k[field][J, sl, sl]
        M[i * d:(i + 1) * d, j * d:(j + 1) * d] = blk
        if i != j:
            M[j * d:(j + 1) * d, i * d:(i + 1) * d] = blk.conj().T
    return M


def gcm_levels(kernels, pairs, nvac, jvals=(0, 2, 4, 6), eps=1e-5, axial=False, gpu=False):
    """Lowest GCM energies per J and the K-mixed projected energy of each vacuum.

    `kernels[k]` holds the projected fields of pair `pairs[k]` (njkk, hjkk arrays
    [J][K1+6][K2+6]); `axial` restricts the basis to K = 0; `gpu` solves every problem
    in one batched launch (`hndiag_batch_gpu`) instead of numpy.
    Returns {J: {"levels": array, "per_q": array(nvac)}}.
    """
    if gpu:
        return _gcm_levels_gpu(kernels, pairs, nvac, jvals, eps, axial)
    out = {}
    for J in jvals:
        if axial:
            d = 1
            sl = slice(JJMAX, JJMAX + 1)
        else:
            d = 2 * J + 1
            sl = slice(JJMAX - J, JJMAX + J + 1)
        Nm = np.zeros((nvac * d, nvac * d), complex)
        Hm = np.zeros_like(Nm)
        for (i, j), k in zip(pairs, kernels):
            for M, f in ((Nm, "njkk"), (Hm, "hjkk")):
                blk = k[f][J, sl, sl]
                M[i * d:(i + 1) * d, j * d:(j + 1) * d] = blk
                if i != j:
                    M[j * d:(j + 1) * d, i * d:(i + 1) * d] = blk.conj().T
        levels, _, m = hndiag(Hm, Nm, eps)
        per_q = np.full(nvac, np.nan)
        for q in range(nvac):
            e, _, mq = hndiag(Hm[q * d:(q + 1) * d, q * d:(q + 1) * d], Nm[q * d:(q + 1) * d, q * d:(q + 1) * d], eps)
            if mq:
                per_q[q] = e[0]
        out[J] = {"levels": levels, "per_q": per_q, "kept": m}
    return out


def _basis_matrices(kernels, pairs, nvac, J, axial):
    d = 1 if axial else 2 * J + 1
    sl = slice(JJMAX, JJMAX + 1) if axial else slice(JJMAX - J, JJMAX + J + 1)
    Nm = np.zeros((nvac * d, nvac * d), complex)
    Hm = np.zeros_like(Nm)
    for (i, j), k in zip(pairs, kernels):
        for M, f in ((Nm, "njkk"), (Hm, "hjkk")):
            blk = k[f][J, sl, sl]
            M[i * d:(i + 1) * d, j * d:(j + 1) * d] = blk
            if i != j:
                M[j * d:(j + 1) * d, i * d:(i + 1) * d] = blk.conj().T
    return Hm, Nm, d


def _gcm_levels_gpu(kernels, pairs, nvac, jvals, eps, axial):
    probs, index = [], []
    for J in jvals:
        Hm, Nm, d = _basis_matrices(kernels, pairs, nvac, J, axial)
        probs.append((Hm, Nm))
        index.append((J, None))
        for q in range(nvac):
            s = slice(q * d, (q + 1) * d)
            probs.append((Hm[s, s], Nm[s, s]))
            index.append((J, q))
    res = hndiag_batch_gpu(probs, eps)
    out = {J: {"levels": None, "per_q": np.full(nvac, np.nan), "kept": 0} for J in jvals}
    for (J, q), (e, k, _) in zip(index, res):
        if q is None:
            out[J]["levels"] = e
            out[J]["kept"] = k
        elif k:
            out[J]["per_q"][q] = e[0]
    return out


def compare_levels(a, b, nlev=3):
    """Largest |E_a - E_b| over the lowest `nlev` GCM levels and over per-vacuum E_J."""
    worst_levels, worst_q = 0.0, 0.0
    for J in a:
        la, lb = a[J]["levels"], b[J]["levels"]
        k = min(nlev, la.size, lb.size)
        if k:
            worst_levels = max(worst_levels, float(np.max(np.abs(la[:k] - lb[:k]))))
        qa, qb = a[J]["per_q"], b[J]["per_q"]
        ok = np.isfinite(qa) & np.isfinite(qb)
        if ok.any():
            worst_q = max(worst_q, float(np.max(np.abs(qa[ok] - qb[ok]))))
    return worst_levels, worst_q
