"""Batched Hill-Wheeler solves on the GPU (`pnamp_hw_solve`) against the numpy HNDIAG
restatement (Codes/GCM/GCM_HNDiag.f90:2-103): energies, number of natural states kept by
the 1e-5 cutoff, and the solutions' normalisation f^+ N f = 1 with f^+ H f = diag(E)."""
import numpy as np
import pytest

from sccm_gb300.gcm import gcm_levels, hndiag, hndiag_batch_gpu

pytestmark = pytest.mark.gpu


def _problem(m, rng, small=None, scale=1.0):
    Q, _ = np.linalg.qr(rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m)))
    ev = np.exp(rng.uniform(np.log(1e-3), 0.0, m)) * scale
    if small is not None:
        ev[-1] = small * scale          # near-null natural state(s)
        ev[-2 if m > 2 else -1] = 1e-7 * scale   # below the 1e-5 cutoff
    N = (Q * ev) @ Q.conj().T
    A = rng.normal(size=(m, m)) + 1j * rng.normal(size=(m, m))
    H = -8.0 * N + 0.4 * (A + A.conj().T)
    return H, N


def test_batch_matches_numpy_hndiag():
    rng = np.random.default_rng(21)
    probs = [_problem(m, rng, small=s) for m, s in
             ((1, None), (2, None), (7, 2e-5), (26, None), (65, 3e-5), (130, 1e-4))]
    res = hndiag_batch_gpu(probs, 1e-5, vectors=True)
    for (H, N), (e, k, F) in zip(probs, res):
        e_ref, en, m_ref = hndiag(H, N, 1e-5)
        assert k == m_ref
        scale = np.abs(e_ref).max()
        assert np.abs(e - e_ref).max() <= 1e-9 * scale, (H.shape, np.abs(e - e_ref).max() / scale)
        Hh, Nh = 0.5 * (H + H.conj().T), 0.5 * (N + N.conj().T)
        # the solutions diagonalise the kept subspace: F^+ N F = 1 and F^+ H F = diag(E)
        # (the residual H f - E N f itself keeps a component along the cut natural states)
        assert np.abs(F.conj().T @ Nh @ F - np.eye(k)).max() <= 1e-8
        assert np.abs(F.conj().T @ Hh @ F - np.diag(e)).max() <= 1e-8 * scale


def test_no_positive_norm_keeps_nothing():
    H = np.eye(3, dtype=complex)
    N = -np.eye(3, dtype=complex)
    (e, k, _), = hndiag_batch_gpu([(H, N)], 1e-5)
    assert k == 0 and e.size == 0


def test_gcm_levels_on_projected_kernels_gpu_equals_host():
    """The levels and per-vacuum E_J of a small pf basis from the library's own projected kernels."""
    from sccm_gb300.basis import Mesh
    from sccm_gb300.pnamp import PnampContext
    from sccm_gb300.synth import make_workload
    w = make_workload("pf", 3, Mesh(4, 6, 4, 5), seed=77)
    with PnampContext(w.sp, w.e0, w.t1b, w.recs, w.vbar, w.mesh, q2=w.q2, form="df64") as ctx:
        kern = [ctx.project(ctx.pair(*w.vacua[i], *w.vacua[j]).zres) for i, j in w.pairs]
    a = gcm_levels(kern, w.pairs, len(w.vacua))
    b = gcm_levels(kern, w.pairs, len(w.vacua), gpu=True)
    for J in a:
        assert a[J]["kept"] == b[J]["kept"]
        la, lb = a[J]["levels"], b[J]["levels"]
        assert np.abs(la - lb).max() <= 1e-8 * max(1.0, np.abs(la).max())
        qa, qb = a[J]["per_q"], b[J]["per_q"]
        ok = np.isfinite(qa)
        assert np.array_equal(ok, np.isfinite(qb))
        assert np.abs(qa[ok] - qb[ok]).max() <= 1e-8 * max(1.0, np.abs(qa[ok]).max())
