"""Oracle self-checks: Pfaffian identities and kernel invariants (no GPU)."""
import numpy as np
import pytest

from sccm_gb300.basis import JJMAX, Mesh
from sccm_gb300.synth import make_workload
from oracle.pnamp_oracle import (Hamiltonian, gauge_matrix, kernel_triaxial, onishi, pfaf_over,
                                 project, rotation_mat, uvphiomega, zbareover, zpfaffian)


def brute_pfaffian(A):
    n = A.shape[0]
    if n == 0:
        return 1.0
    tot = 0.0
    for j in range(1, n):
        idx = [k for k in range(n) if k not in (0, j)]
        tot += (-1) ** (j + 1) * A[0, j] * brute_pfaffian(A[np.ix_(idx, idx)])
    return tot


@pytest.mark.parametrize("N", [2, 4, 6, 8])
def test_pfaffian_matches_expansion(N):
    rng = np.random.default_rng(N)
    X = rng.standard_normal((N, N)) + 1j * rng.standard_normal((N, N))
    A = X - X.T
    pf, st = zpfaffian(A)
    assert st == 0
    assert abs(pf - brute_pfaffian(A)) < 1e-11 * max(1.0, abs(pf))


def test_pfaffian_squared_is_determinant():
    rng = np.random.default_rng(7)
    X = rng.standard_normal((24, 24)) + 1j * rng.standard_normal((24, 24))
    A = X - X.T
    pf, _ = zpfaffian(A)
    assert abs(pf ** 2 - np.linalg.det(A)) < 1e-9 * abs(pf) ** 2


def test_pfaffian_zero_pivot_early_exit():
    A = np.zeros((6, 6), complex)
    pf, st = zpfaffian(A)
    assert pf == 0 and st == 1


@pytest.fixture(scope="module")
def sd_pair():
    return make_workload("sd", 2, Mesh(2, 3, 2, 3), seed=11, deformed=False)


def test_norm_is_one_at_identity(sd_pair):
    w = sd_pair
    U, V = w.vacua[0]
    zzc, d = zbareover(V, U)
    A = gauge_matrix(rotation_mat(w.sp, 0, 0, 0), 0, 0)
    ub, vb = uvphiomega(A, U, V)
    pf, _ = pfaf_over(zzc, ub, vb)
    assert abs(d * d * pf - 1.0) < 1e-12


def test_pfaffian_norm_agrees_with_onishi_magnitude(sd_pair):
    w = sd_pair
    (U0, V0), (U1, V1) = w.vacua
    zzc0, d0 = zbareover(V0, U0)
    _, d1 = zbareover(V1, U1)
    for (a, b, g, pp, pn) in [(0.3, 0.7, 1.1, 0.4, 2.0), (1.2, 2.1, 0.2, 3.0, 1.0)]:
        A = gauge_matrix(rotation_mat(w.sp, a, b, g), pp, pn)
        ub, vb = uvphiomega(A, U1, V1)
        pf, _ = pfaf_over(zzc0, ub, vb)
        on = onishi(U0, V0, ub, vb)
        assert abs(abs(d0 * d1 * pf) - abs(on)) < 1e-10


def test_projected_norm_matrix_is_hermitian_psd():
    """N^J_{K1K2} of q = q' is Hermitian and positive semi-definite. Gauss-Legendre
    in alpha, gamma converges exponentially (6: 1.6e-3, 10: 8.6e-5, 14: 1.2e-6
    relative non-Hermiticity at J = 2); 8 points bound it by 1e-3."""
    w = make_workload("sd", 1, Mesh(8, 6, 8, 1), seed=5, deformed=True)
    U, V = w.vacua[0]
    ham = Hamiltonian(0.0, w.t1b, w.recs, w.vbar, w.q2, w.jops)
    z = kernel_triaxial(w.sp, ham, w.mesh, U, V, U, V, iE2=False)
    k = project(z, w.mesh, chop=0.0)
    for J in (0, 2):
        N = k["zsum"][J, JJMAX - J:JJMAX + J + 1, JJMAX - J:JJMAX + J + 1, 0]
        assert np.abs(N - N.conj().T).max() < 1e-3 * np.abs(N).max()
        assert np.linalg.eigvalsh(0.5 * (N + N.conj().T)).min() > -1e-9 * np.abs(N).max()
