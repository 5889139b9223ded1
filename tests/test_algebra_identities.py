"""The exact rearrangements the GPU form makes of the reference's per-point sequence,
checked on the CPU against the oracle's literal restatement with random inputs:

  * the reduced Pfaffian  Pf(c[[M, -I], [I, -Z0]]) = Pf(c(M - Z0^-1)) Pf(-c Z0);
  * for species-block-diagonal skew matrices, Pf = product of the blocks' Pfaffians;
  * the energy's regrouping of the 8-term sum of HFB_Energy_COMPLEX into
    V[rho_ki rho_lj - rho_li rho_kj + d(rho_ik rho_jl - rho_jk rho_il)]
    + V/4 [K01_ij K10_kl + d K01_kl K10_ij], K_xy = kappa_xy - kappa_yx,
    and its proton-neutron short form for species-split densities;
  * Y T22^-1 by column Gauss-Jordan elimination with row pivoting, as the solve runs it;
  * the tensor-core recast of the two-body energy (contract_tc.cu): a particle-hole form
    s^T Q s over the entries s = rho(r, c) and a particle-particle form u^T C w over the
    antisymmetric pair vectors u = K01, w = K10, both block-diagonal by conserved labels
    and packed into groups (closed under label negation for the ph form) whose rows and
    columns are one contiguous storage range.
"""
import numpy as np
import pytest

from sccm_gb300.basis import SHELLS, ModelSpace
from sccm_gb300.synth import mscheme_pairs
from sccm_gb300.contraction import contraction_groups
from oracle.pnamp_oracle import Hamiltonian, energy, zpfaffian

rng = np.random.default_rng(20261203)


def skew(n):
    a = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    return a - a.T


@pytest.mark.parametrize("n,c", [(4, 1.0), (10, 0.7), (16, 1.3)])
def test_reduced_pfaffian(n, c):
    M, Z0 = skew(n), skew(n)
    S = np.zeros((2 * n, 2 * n), complex)
    S[:n, :n], S[:n, n:], S[n:, :n], S[n:, n:] = M, -np.eye(n), np.eye(n), -Z0
    full = zpfaffian(c * S)[0]
    red = zpfaffian(c * (M - np.linalg.inv(Z0)))[0] * zpfaffian(-c * Z0)[0]
    assert abs(full - red) <= 1e-10 * abs(full)


def test_block_diagonal_pfaffian_factorises():
    h = 8
    A, B = skew(h), skew(h)
    S = np.zeros((2 * h, 2 * h), complex)
    S[:h, :h], S[h:, h:] = A, B
    assert abs(zpfaffian(S)[0] - zpfaffian(A)[0] * zpfaffian(B)[0]) <= 1e-11 * abs(zpfaffian(S)[0])


def regrouped_energy(rho, k10, k01, ham, short_pn=False):
    i, j, k, l = (ham.recs[:, q] for q in range(4))
    d = np.where(i + j == k + l, 0.0, 1.0)
    K01 = k01 - k01.T
    K10 = k10 - k10.T
    t = rho[k, i] * rho[l, j] - rho[l, i] * rho[k, j] + d * (rho[i, k] * rho[j, l] - rho[j, k] * rho[i, l])
    u = K01[i, j] * K10[k, l] + d * K01[k, l] * K10[i, j]
    full = ham.vbar * (t + 0.25 * u)
    if short_pn:
        h = rho.shape[0] // 2
        pn = (i < h) & (j >= h) & (k < h) & (l >= h)
        ts = rho[k, i] * rho[l, j] + d * rho[i, k] * rho[j, l]
        full = np.where(pn, ham.vbar * ts, full)
    return np.sum(full)


def test_energy_regrouping_is_exact():
    sp = ModelSpace(SHELLS["sd"], 2, 2)
    n = sp.nlev
    recs = np.asarray(mscheme_pairs(sp))
    vbar = rng.normal(size=len(recs))
    ham = Hamiltonian(0.0, np.zeros((n, n)), recs, vbar, None, None)
    rho, k10, k01 = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)) for _ in range(3))
    ekin, etot = energy(rho, k10, k01, ham)
    assert abs(regrouped_energy(rho, k10, k01, ham) - (etot - ekin)) <= 1e-12 * abs(etot - ekin)


def test_proton_neutron_short_form_for_split_densities():
    sp = ModelSpace(SHELLS["sd"], 2, 2)
    n, h = sp.nlev, sp.nlev // 2
    recs = np.asarray(mscheme_pairs(sp))
    vbar = rng.normal(size=len(recs))
    ham = Hamiltonian(0.0, np.zeros((n, n)), recs, vbar, None, None)
    mask = np.zeros((n, n))
    mask[:h, :h] = mask[h:, h:] = 1.0       # charge-conserving: no proton-neutron entries
    rho, k10, k01 = ((rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))) * mask for _ in range(3))
    e_full = regrouped_energy(rho, k10, k01, ham)
    e_short = regrouped_energy(rho, k10, k01, ham, short_pn=True)
    assert abs(e_full - e_short) <= 1e-12 * abs(e_full)


def test_column_gauss_jordan_with_row_pivoting():
    """The solve's sequence: step k takes the pivot column c = argmax |A[k][j]|, j >= k;
    every later row of A and every row of Y gets m = row[c] / A[k][c] into column k, its
    old column k into column c, and row[j] -= m P[j] (P = row k of A, columns c, k
    exchanged); A's row k is then finished. The result is Y A^-1."""
    for h, ny in [(5, 10), (20, 40)]:
        A = rng.normal(size=(h, h)) + 1j * rng.normal(size=(h, h))
        Y = rng.normal(size=(ny, h)) + 1j * rng.normal(size=(ny, h))
        M, W = A.copy(), Y.copy()
        for k in range(h):
            c = k + int(np.argmax(np.abs(M[k, k:].real) + np.abs(M[k, k:].imag)))
            P = M[k].copy()
            P[c], P[k] = P[k], P[c]
            piv = M[k, c]
            rows = [M[r] for r in range(k + 1, h)] + [W[r] for r in range(ny)]
            for row in rows:
                m = row[c] / piv
                old_k = row[k]
                row[k] = m
                if c != k:
                    row[c] = old_k
                for j in range(h):
                    if j != k:
                        row[j] -= m * P[j]
        assert np.abs(W - Y @ np.linalg.inv(A)).max() <= 1e-10 * np.abs(Y @ np.linalg.inv(A)).max()


@pytest.mark.parametrize("shell", ["sd", "pf", "sdpf"])
def test_contraction_groups_reproduce_the_energy_loop(shell):
    sp = ModelSpace(SHELLS[shell], 2, 2)
    recs = mscheme_pairs(sp)
    vbar = rng.normal(size=len(recs))
    n = sp.nlev
    pos, ranges, mats, nk = contraction_groups(sp, recs, vbar)
    assert all(dp <= 384 and dp % 64 == 0 for _, _, dp in ranges)
    ham = Hamiltonian(0.0, np.zeros((n, n)), recs, vbar, None, None)
    rho, k10, k01 = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n)) for _ in range(3))
    ekin, etot = energy(rho, k10, k01, ham)
    x = np.zeros(nk, complex)   # operand vector: s (ph), w = K10 (pp)
    y = np.zeros(nk, complex)   # epilogue vector: s (ph), u = K01 (pp)
    for (kind, e), p in pos.items():
        if kind == "ph":
            x[p] = y[p] = rho[e]
        else:
            i, j = e
            x[p] = k10[i, j] - k10[j, i]
            y[p] = k01[i, j] - k01[j, i]
    e2 = sum(y[o:o + dp] @ (M @ x[o:o + dp]) for (_, o, dp), M in zip(ranges, mats))
    assert abs(e2 - (etot - ekin)) <= 1e-12 * abs(etot - ekin)
