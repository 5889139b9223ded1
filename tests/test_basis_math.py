"""The special functions the reference takes from an unshipped library, restated from their
definitions (Wigner small-d, Gauss-Legendre, Clebsch-Gordan / 3j), checked against the
identities that define them: unitarity and the composition law of d^j, exactness of the
quadrature, orthogonality of the Clebsch-Gordan coefficients and the symmetries of 3j."""
import math

import numpy as np
import pytest

from sccm_gb300.basis import cg, dwig, gauss_legendre, threej


def dmat(tj, beta):
    ms = range(tj, -tj - 1, -2)
    return np.array([[dwig(tj, m1, m2, beta) for m2 in ms] for m1 in ms])


@pytest.mark.parametrize("tj", [1, 2, 3, 5, 7, 9, 12])
def test_wigner_d_is_orthogonal_and_composes(tj):
    b1, b2 = 0.37, 1.91
    d1, d2 = dmat(tj, b1), dmat(tj, b2)
    assert np.abs(d1 @ d1.T - np.eye(tj + 1)).max() < 1e-12
    assert np.abs(d1 @ d2 - dmat(tj, b1 + b2)).max() < 1e-12          # rotations about y add
    assert np.abs(dmat(tj, 0.0) - np.eye(tj + 1)).max() < 1e-15


def test_wigner_d_known_values_and_symmetry():
    b = 0.8
    c, s = math.cos(b / 2), math.sin(b / 2)
    assert abs(dwig(1, 1, 1, b) - c) < 1e-15 and abs(dwig(1, 1, -1, b) + s) < 1e-15
    assert abs(dwig(2, 0, 0, b) - math.cos(b)) < 1e-15
    assert abs(dwig(4, 0, 0, b) - 0.5 * (3 * math.cos(b) ** 2 - 1)) < 1e-14   # P_2
    for tj in (3, 5):
        for m1 in range(-tj, tj + 1, 2):
            for m2 in range(-tj, tj + 1, 2):
                sgn = (-1) ** ((m1 - m2) // 2)
                assert abs(dwig(tj, m1, m2, b) - sgn * dwig(tj, m2, m1, b)) < 1e-14
                assert abs(dwig(tj, m1, m2, -b) - dwig(tj, m2, m1, b)) < 1e-14


@pytest.mark.parametrize("n", [1, 4, 9, 16])
def test_gauss_legendre_integrates_degree_2n_minus_1(n):
    x, w = gauss_legendre(0.0, 2 * math.pi, n)
    assert np.all(np.diff(x) > 0) and abs(w.sum() - 2 * math.pi) < 1e-12
    for k in range(2 * n):
        exact = (2 * math.pi) ** (k + 1) / (k + 1)
        assert abs(np.sum(w * x ** k) - exact) < 1e-10 * exact


def test_clebsch_gordan_orthogonality():
    for tj1, tj2 in [(1, 1), (3, 5), (7, 7), (5, 2)]:
        for tM in range(-(tj1 + tj2), tj1 + tj2 + 1, 2):
            Js = [tJ for tJ in range(abs(tj1 - tj2), tj1 + tj2 + 1, 2) if abs(tM) <= tJ]
            pairs = [(m1, tM - m1) for m1 in range(-tj1, tj1 + 1, 2) if abs(tM - m1) <= tj2]
            C = np.array([[cg(tj1, tj2, tJ, m1, m2, tM) for tJ in Js] for m1, m2 in pairs])
            assert np.abs(C.T @ C - np.eye(len(Js))).max() < 1e-12
            assert np.abs(C @ C.T - np.eye(len(pairs))).max() < 1e-12


def test_threej_symmetries():
    args = (5, 4, 3, 1, -2, 1)
    v = threej(*args)
    tj1, tj2, tj3, m1, m2, m3 = args
    assert abs(v) > 1e-3
    assert abs(threej(tj2, tj3, tj1, m2, m3, m1) - v) < 1e-14                 # cyclic
    ph = (-1) ** ((tj1 + tj2 + tj3) // 2)
    assert abs(threej(tj2, tj1, tj3, m2, m1, m3) - ph * v) < 1e-14            # odd permutation
    assert abs(threej(tj1, tj2, tj3, -m1, -m2, -m3) - ph * v) < 1e-14         # m -> -m
    assert threej(4, 4, 4, 2, 2, -2) == 0.0                                   # sum of m != 0
