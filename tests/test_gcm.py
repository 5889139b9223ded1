"""Hill-Wheeler solve on projected kernels (host): HNDIAG's cutoff and the first-order
level weights the learned mode's Hill-Wheeler gate uses (no GPU)."""
import numpy as np

from sccm_gb300.basis import JJMAX
from sccm_gb300.gcm import diagonal_norms, gcm_levels, hndiag, level_error_bound, level_weights


def _random_kernels(nvac, jvals, rng, small=1e-4):
    """Projected kernels of a complete pair set: per J a positive norm matrix with one
    near-null direction (eigenvalue `small` x the largest, kept by the 1e-5 cutoff) and a
    Hermitian H, cut into (i <= j) blocks."""
    pairs = [(i, j) for i in range(nvac) for j in range(i, nvac)]
    ker = [{"njkk": np.zeros((JJMAX + 1, 2 * JJMAX + 1, 2 * JJMAX + 1), complex),
            "hjkk": np.zeros((JJMAX + 1, 2 * JJMAX + 1, 2 * JJMAX + 1), complex)} for _ in pairs]
    for J in jvals:
        d = 2 * J + 1
        m = nvac * d
        Q, _ = np.linalg.qr(rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m)))
        ev = np.exp(rng.uniform(np.log(0.05), 0.0, m))
        ev[-1] = small
        N = (Q * ev) @ Q.conj().T
        A = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
        H = -10.0 * N + 0.5 * (A + A.conj().T) * 0.3
        H = 0.5 * (H + H.conj().T)
        sl = slice(JJMAX - J, JJMAX + J + 1)
        for k, (i, j) in enumerate(pairs):
            ker[k]["njkk"][J, sl, sl] = N[i * d:(i + 1) * d, j * d:(j + 1) * d]
            ker[k]["hjkk"][J, sl, sl] = H[i * d:(i + 1) * d, j * d:(j + 1) * d]
    return ker, pairs


def test_hndiag_cutoff_and_identity_norm():
    rng = np.random.default_rng(1)
    A = rng.normal(size=(6, 6))
    H = A + A.T
    e, en, m = hndiag(H, np.eye(6))
    assert m == 6 and np.allclose(e, np.linalg.eigvalsh(H))
    N = np.diag([1.0, 0.5, 0.2, 1e-7, 1e-3, 0.9])
    e, en, m = hndiag(H, N)
    assert m == 5   # 1e-7 is below the 1e-5 cutoff
    keep = [0, 1, 2, 4, 5]
    Nk = N[np.ix_(keep, keep)]
    Hk = H[np.ix_(keep, keep)]
    s = np.diag(1 / np.sqrt(np.diag(Nk)))
    assert np.allclose(e, np.linalg.eigvalsh(s @ Hk @ s))


def test_level_weights_bound_first_order_shifts():
    """A small Hermitian error on each pair's block moves every low level and every
    per-vacuum E_J by at most sum over pairs of weight x ||dH_block|| (to first order)."""
    rng = np.random.default_rng(7)
    nvac, jvals = 4, (0, 2)
    ker, pairs = _random_kernels(nvac, jvals, rng)
    W = level_weights(ker, pairs, nvac, jvals, nlev=3)
    base = gcm_levels(ker, pairs, nvac, jvals)
    eps = 1e-7
    for trial in range(3):
        pert = []
        bound = {J: 0.0 for J in jvals}
        for k, (i, j) in enumerate(pairs):
            r = {f: v.copy() for f, v in ker[k].items()}
            for J in jvals:
                d = 2 * J + 1
                sl = slice(JJMAX - J, JJMAX + J + 1)
                D = eps * (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))
                if i == j:
                    D = 0.5 * (D + D.conj().T)
                r["hjkk"][J, sl, sl] += D
                bound[J] += W[J][k] * np.linalg.norm(D, 2)
            pert.append(r)
        got = gcm_levels(pert, pairs, nvac, jvals)
        for J in jvals:
            dl = np.abs(got[J]["levels"][:3] - base[J]["levels"][:3]).max()
            dq = np.abs(got[J]["per_q"] - base[J]["per_q"]).max()
            assert dl <= 1.01 * bound[J], (J, dl, bound[J])
            assert dq <= 1.01 * bound[J], (J, dq, bound[J])
            assert bound[J] < 1e3 * max(dl, dq)   # and the bound is not vacuous


def test_level_weights_grow_with_norm_conditioning():
    """The near-null natural state amplifies H errors by about 1/its norm eigenvalue."""
    rng = np.random.default_rng(3)
    w_ok = level_weights(*_random_kernels(3, (0,), rng, small=1e-1), 3, (0,))
    rng = np.random.default_rng(3)
    w_bad = level_weights(*_random_kernels(3, (0,), rng, small=1e-4), 3, (0,))
    assert w_bad[0].max() > 10 * w_ok[0].max()


def test_level_error_bound_covers_errors_of_that_size():
    """Errors of a given size in the basis of normalised states on every pair's H^J entries
    move the levels and E_J by at most level_error_bound (first order, small errors)."""
    rng = np.random.default_rng(9)
    nvac, jvals = 4, (0, 2)
    ker, pairs = _random_kernels(nvac, jvals, rng)
    W = level_weights(ker, pairs, nvac, jvals, nlev=3)
    diag = diagonal_norms(ker, pairs, jvals)
    err = 1e-8
    bound = level_error_bound(W, pairs, diag, err, jvals)
    base = gcm_levels(ker, pairs, nvac, jvals)
    for trial in range(3):
        pert = []
        for k, (i, j) in enumerate(pairs):
            r = {f: v.copy() for f, v in ker[k].items()}
            for J in jvals:
                d = 2 * J + 1
                sl = slice(JJMAX - J, JJMAX + J + 1)
                sc = np.sqrt(diag[i][J] * diag[j][J])
                ph = np.exp(2j * np.pi * rng.uniform(size=(d, d)))
                D = err * sc * ph            # every entry exactly err in normalised units
                if i == j:
                    D = 0.5 * (D + D.conj().T)
                r["hjkk"][J, sl, sl] += D
            pert.append(r)
        got = gcm_levels(pert, pairs, nvac, jvals)
        for J in jvals:
            dl = np.abs(got[J]["levels"][:3] - base[J]["levels"][:3]).max()
            dq = np.abs(got[J]["per_q"] - base[J]["per_q"]).max()
            assert max(dl, dq) <= 1.01 * bound
