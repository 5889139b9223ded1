"""Build tests/golden/ti48_highprec.npz: the norm kernel of ill-conditioned Ti48 pairs in
30-digit arithmetic.

The reference's per-point sequence (Pfaf_Over inverts the rotated U1 at every point,
Codes/PNAMP/PNAMP_Proj.f90:162-184) loses up to ~1e-7 relative on the shipped Ti48
vacua whose U has condition numbers ~1e4-1e5 (beta2 = -0.3 and -0.2), so an FP64
restatement of it cannot judge the GPU at 1e-10 there. This script evaluates the same
formula,

    N(Omega) = (1/NFOM^2) sum_phi (-1)^(n(n+1)/2) Det0 Det1 Pf(S) e^{-i Z phi_p} e^{-i N phi_n},
    S = [[A W A^T, -I], [I, -Z0]],  A = D_phi R(Omega),  W = V1 U1^-1,  Z0 = V0 U0^-1,
    Det = det(1 + Z^T Z)^(-1/4)                     (PNAMP_Kernel3D.f90:286-294),

in mpmath at 30 digits on the FP64 input values (vacua from tests/golden/reference_pins.npz,
mesh nodes as the library computes them), with Wigner's explicit sum for d^j(beta) and
the Pfaffian of the skew matrix defined by the upper triangle, as ZPfaffianF reads it.

    python tests/golden/make_ti48_highprec.py      (a few minutes; needs mpmath)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

import mpmath as mpm  # noqa: E402
from mpmath import mp  # noqa: E402

from sccm_gb300.basis import Mesh, dwig  # noqa: E402
from sccm_gb300.synth import ti48_workload  # noqa: E402

MESH = (2, 3, 2, 5)                 # nalp, nbet, ngam, nfom: the mesh of the Ti48 GPU tests
CASES = [(4, 0, (5, 8)), (5, 1, (7, 9))]   # (bra, ket, Euler indices)


def wigner_d_mp(tj, tm1, tm2, beta):
    """Edmonds' d^j_{m1 m2}(beta) from Wigner's explicit sum (doubled j, m)."""
    j, m1, m2 = mpm.mpf(tj) / 2, mpm.mpf(tm1) / 2, mpm.mpf(tm2) / 2
    c, s = mpm.cos(mpm.mpf(beta) / 2), mpm.sin(mpm.mpf(beta) / 2)
    f = lambda x: mpm.factorial(int(x))
    pre = mpm.sqrt(f(j + m1) * f(j - m1) * f(j + m2) * f(j - m2))
    tot = mpm.mpf(0)
    kmin = int(max(0, m2 - m1))
    kmax = int(min(j + m2, j - m1))
    for k in range(kmin, kmax + 1):
        den = f(j + m2 - k) * f(k) * f(j - k - m1) * f(k - m2 + m1)
        tot += (-1) ** (k - int(m2 - m1)) * c ** int(2 * j - 2 * k + m2 - m1) * s ** int(2 * k - m2 + m1) / den
    return pre * tot


def mpmat(a):
    return [[mpm.mpc(complex(x)) for x in row] for row in np.asarray(a)]


def matmul(A, B):
    n, m, p = len(A), len(B), len(B[0])
    return [[mpm.fsum(A[i][k] * B[k][j] for k in range(m)) for j in range(p)] for i in range(n)]


def inverse(A):
    n = len(A)
    M = mpm.matrix(A)
    Mi = M ** -1
    return [[Mi[i, j] for j in range(n)] for i in range(n)]


def pfaffian_upper(S):
    """Pfaffian of the skew matrix defined by the strict upper triangle of S (row pivoting)."""
    N = len(S)
    T = [[S[i][j] if j > i else mpm.mpc(0) for j in range(N)] for i in range(N)]
    for i in range(N):
        for j in range(i):
            T[i][j] = -T[j][i]
    pf = mpm.mpc(1)
    for k in range(0, N - 2, 2):
        jm = max(range(k + 1, N), key=lambda j: abs(T[k][j]))
        if jm != k + 1:
            T[k + 1], T[jm] = T[jm], T[k + 1]
            for row in T:
                row[k + 1], row[jm] = row[jm], row[k + 1]
            pf = -pf
        piv = T[k][k + 1]
        pf *= piv
        a, b = T[k], T[k + 1]
        for i in range(k + 2, N):
            ai, bi, Ti = a[i], b[i], T[i]
            for j in range(k + 2, N):
                Ti[j] = Ti[j] + (bi * a[j] - ai * b[j]) / piv
    return pf * T[N - 2][N - 1]


def det_factor(Z):
    n = len(Z)
    ZtZ = matmul([list(r) for r in zip(*Z)], Z)
    for i in range(n):
        ZtZ[i][i] += 1
    return mpm.det(mpm.matrix(ZtZ)) ** mpm.mpf(-0.25)


def main(out=os.path.join(HERE, "ti48_highprec.npz")):
    mp.dps = 30
    mesh = Mesh(*MESH)
    w = ti48_workload(mesh)
    sp = w.sp
    n, h = sp.nlev, sp.nlev // 2
    pts = mesh.euler_points()
    phis = mesh.gauge_angles()
    snpfaf = -1 if (n * (n + 1) // 2) % 2 else 1
    rows = []
    for bra, ket, ies in CASES:
        (U0, V0), (U1, V1) = w.vacua[bra], w.vacua[ket]
        Z0 = matmul(mpmat(V0), inverse(mpmat(U0)))
        W = matmul(mpmat(V1), inverse(mpmat(U1)))
        d01 = det_factor(Z0) * det_factor(W)
        for ie in ies:
            alp, bet, gam, _ = pts[ie]
            R = [[mpm.mpc(0)] * n for _ in range(n)]
            for s, d in sp.blocks():
                tj = int(sp.twoj[s])
                for i in range(d):
                    for k in range(d):
                        ma, mb = int(sp.twom[s + i]), int(sp.twom[s + k])
                        dv = wigner_d_mp(tj, ma, mb, bet)
                        assert abs(float(dv) - dwig(tj, ma, mb, bet)) < 1e-13
                        R[s + i][s + k] = (mpm.expj(-mpm.mpf(alp) * ma / 2) * mpm.expj(-mpm.mpf(gam) * mb / 2) * dv)
            RW = matmul(R, W)
            X = matmul(RW, [list(r) for r in zip(*R)])
            acc = mpm.mpc(0)
            for php in phis:
                for phn in phis:
                    e = [mpm.expj(mpm.mpf(php))] * h + [mpm.expj(mpm.mpf(phn))] * h
                    S = [[mpm.mpc(0)] * (2 * n) for _ in range(2 * n)]
                    for i in range(n):
                        for j in range(n):
                            S[i][j] = e[i] * X[i][j] * e[j]
                            S[n + i][n + j] = -Z0[i][j]
                        S[i][n + i] = mpm.mpc(-1)
                    pf = pfaffian_upper(S)
                    ph = mpm.expj(-mpm.mpf(php) * sp.nprot) * mpm.expj(-mpm.mpf(phn) * sp.nneut)
                    acc += snpfaf * d01 * pf * ph
            val = acc / len(phis) ** 2
            rows.append((bra, ket, ie, float(val.real), float(val.imag)))
            print(bra, ket, ie, complex(val), flush=True)
    np.savez_compressed(out, mesh=np.array(MESH), cases=np.array([r[:3] for r in rows], dtype=np.int32),
                        norm=np.array([complex(r[3], r[4]) for r in rows]))
    print(f"wrote {out}")


if __name__ == "__main__":
    main()
