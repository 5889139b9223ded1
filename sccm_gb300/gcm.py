"""Hill-Wheeler (GCM) solve on projected kernels: the consumer of PNAMP's output.

`hndiag` restates HNDIAG (Codes/GCM/GCM_HNDiag.f90:2-103): diagonalise the norm
matrix, keep the natural states whose eigenvalue is at least `eps` times the
largest (the driver's cutoff `1.e-5`, Codes/exec/GCM.sh:59), and diagonalise
N^-1/2 H N^-1/2 in that subspace. `gcm_levels` assembles, for each even J, the
basis (q, K), K = -J..J, from the projected N^J_{K1K2}(q, q') and
H^J_{K1K2}(q, q') of every computed pair (q <= q'; the other triangle by
Hermiticity, N^J_{K1K2}(q', q) = conj(N^J_{K2K1}(q, q'))) and returns the levels.
Host-side: a few matrices of size (number of vacua x (2J+1)).
"""
from __future__ import annotations

import numpy as np

from .basis import JJMAX


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


def gcm_levels(kernels, pairs, nvac, jvals=(0, 2, 4, 6), eps=1e-5, axial=False):
    """Lowest GCM energies per J and the K-mixed projected energy of each vacuum.

    `kernels[k]` holds the projected fields of pair `pairs[k]` (njkk, hjkk arrays
    [J][K1+6][K2+6]); `axial` restricts the basis to K = 0.
    Returns {J: {"levels": array, "per_q": array(nvac)}}.
    """
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
