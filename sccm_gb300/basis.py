"""Single-particle basis, angular-momentum algebra and the projection mesh.

Host-side preparation for the PNAMP kernels. Everything here is one-off table
building (O(n^2) or less per run); none of it is on the per-point path.

Reference layout this module follows:
  * m-scheme ordering: protons (t=-1) first, then neutrons (t=+1); inside each
    species the orbits in `.val` order, and inside an orbit m = j, j-1, ..., -j
    (Codes/GCM/HFBA_Hamiltonian.f90:43-68). `n` is stored 1-based as
    `tnljm%n = SPB%n + 1` (HFBA_Hamiltonian.f90:51,85).
  * Gauss-Legendre mesh: alpha, gamma on [0, 2pi]; cos(beta) on [-1, 1] with
    beta = acos(x); a one-point direction collapses to angle 0, weight 1
    (Codes/GCM/PNAMP_Gaus.f90:27-46).
  * Wigner small-d: the reference calls `dwignerI_gen`, which is not shipped.
    The rotation is R = exp(-i alp Jz) exp(-i bet Jy) exp(-i gam Jz)
    (Codes/PNAMP/PNAMP_Kernel3D.f90:7, PNAMP_Proj.f90:85) with Edmonds'
    d^j_{m m'}(beta); the reference's Ge76 kernel files pin this choice: with
    <q| the first vacuum of the pair, 16 of the 25 shipped pairs are reproduced
    to their 8 printed digits at every J only with this sign of beta. `dwig`
    implements it from Wigner's explicit sum.
  * J operators: `zJiME` (Codes/PNAMP/PNAMP_ME1B.f90:332-422).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from functools import lru_cache

import numpy as np

NOBS = 19          # observables per Euler point (Codes/PNAMP/VAPHFB_Par.f90:168)
JJMAX = 6          # max projected J (Codes/PNAMP/VAPHFB_Par.f90:278)
CHOP = 1.0e-8      # |N^J| below this is not written (VAPHFB_Par.f90:160, Kernel3D.f90:732)

# named shells used by the synthetic workloads: (n, l, 2j), n counted from 0
SHELLS = {
    "sd": [(0, 2, 5), (1, 0, 1), (0, 2, 3)],
    "pf": [(0, 3, 7), (1, 1, 3), (0, 3, 5), (1, 1, 1)],
    "pf5g9": [(0, 3, 5), (1, 1, 3), (1, 1, 1), (0, 4, 9)],
    "sdpf": [(0, 2, 5), (1, 0, 1), (0, 2, 3), (0, 3, 7), (1, 1, 3), (0, 3, 5), (1, 1, 1)],
    # two p1/2 orbits: one-body density blocks with n1 != n2 (test space)
    "p2": [(0, 1, 3), (0, 1, 1), (1, 1, 1)],
}


@dataclass
class ModelSpace:
    """m-scheme single-particle basis (the reference's `tnljm` arrays)."""
    orbits: list                     # [(n0, l, twoj)] in .val order, n0 from 0
    nprot: int                       # valence protons Z
    nneut: int                       # valence neutrons N
    core_prot: int = 0
    core_neut: int = 0
    t: np.ndarray = field(init=False)      # -1 proton, +1 neutron
    n: np.ndarray = field(init=False)      # 1-based radial index
    l: np.ndarray = field(init=False)
    twoj: np.ndarray = field(init=False)
    twom: np.ndarray = field(init=False)
    lj: np.ndarray = field(init=False)     # (2l + 2j - 1)/2
    orbit: np.ndarray = field(init=False)  # orbit index (0-based, per species)

    def __post_init__(self):
        rows = []
        for t in (-1, 1):
            for io, (n0, l, tj) in enumerate(self.orbits):
                for tm in range(tj, -tj - 1, -2):
                    rows.append((t, n0 + 1, l, tj, tm, (2 * l + tj - 1) // 2, io))
        a = np.array(rows, dtype=np.int32)
        self.t, self.n, self.l, self.twoj, self.twom, self.lj, self.orbit = (a[:, k].copy() for k in range(7))

    @property
    def nlev(self) -> int:
        return int(self.t.size)

    @property
    def half(self) -> int:
        return self.nlev // 2

    def blocks(self):
        """Diagonal blocks of the rotation matrix: (start, size) per (t, n, l, j)."""
        out = []
        i = 0
        while i < self.nlev:
            d = int(self.twoj[i]) + 1
            out.append((i, d))
            i += d
        return out


# --------------------------------------------------------------------------
# Factorials / Clebsch-Gordan / Wigner d (from the closed-form definitions)
# --------------------------------------------------------------------------
@lru_cache(maxsize=None)
def _fact(k: int) -> float:
    return float(math.factorial(k))


def cg(tj1, tj2, tJ, tm1, tm2, tM) -> float:
    """<j1 m1 j2 m2 | J M> with all arguments doubled (Racah's formula).

    Same argument convention as the reference's CJJ(j1,j2,J,m1,m2,M)
    (called at Codes/GCM/HFBA_Hamiltonian.f90:342-355).
    """
    if tm1 + tm2 != tM:
        return 0.0
    if tJ < abs(tj1 - tj2) or tJ > tj1 + tj2 or (tj1 + tj2 + tJ) % 2:
        return 0.0
    if abs(tm1) > tj1 or abs(tm2) > tj2 or abs(tM) > tJ:
        return 0.0
    if (tj1 + tm1) % 2 or (tj2 + tm2) % 2 or (tJ + tM) % 2:
        return 0.0
    j1p, j2p, Jp = (tj1 + tj2 - tJ) // 2, (tj1 - tj2 + tJ) // 2, (-tj1 + tj2 + tJ) // 2
    tri = _fact(j1p) * _fact(j2p) * _fact(Jp) / _fact((tj1 + tj2 + tJ) // 2 + 1)
    pre = math.sqrt((tJ + 1) * tri
                    * _fact((tj1 + tm1) // 2) * _fact((tj1 - tm1) // 2)
                    * _fact((tj2 + tm2) // 2) * _fact((tj2 - tm2) // 2)
                    * _fact((tJ + tM) // 2) * _fact((tJ - tM) // 2))
    s = 0.0
    for k in range(0, 200):
        a1 = (tj1 + tj2 - tJ) // 2 - k
        a2 = (tj1 - tm1) // 2 - k
        a3 = (tj2 + tm2) // 2 - k
        a4 = (tJ - tj2 + tm1) // 2 + k
        a5 = (tJ - tj1 - tm2) // 2 + k
        if a1 < 0 or a2 < 0 or a3 < 0:
            break
        if a4 < 0 or a5 < 0:
            continue
        s += (-1) ** k / (_fact(k) * _fact(a1) * _fact(a2) * _fact(a3) * _fact(a4) * _fact(a5))
    return pre * s


def threej(tj1, tj2, tj3, tm1, tm2, tm3) -> float:
    """Wigner 3j symbol, doubled arguments."""
    if tm1 + tm2 + tm3 != 0:
        return 0.0
    ph = -1.0 if ((tj1 - tj2 - tm3) // 2) % 2 else 1.0
    return ph * cg(tj1, tj2, tj3, tm1, tm2, -tm3) / math.sqrt(tj3 + 1)


def wigner_d_edmonds(tj, tm1, tm2, beta) -> float:
    """Edmonds/Wigner d^j_{m1 m2}(beta) = <j m1| exp(-i beta J_y) |j m2>, doubled j, m."""
    if abs(tm1) > tj or abs(tm2) > tj or (tj + tm1) % 2 or (tj + tm2) % 2:
        return 0.0
    jpm1, jmm1 = (tj + tm1) // 2, (tj - tm1) // 2
    jpm2, jmm2 = (tj + tm2) // 2, (tj - tm2) // 2
    pre = math.sqrt(_fact(jpm1) * _fact(jmm1) * _fact(jpm2) * _fact(jmm2))
    c, s = math.cos(beta / 2.0), math.sin(beta / 2.0)
    d = 0.0
    dm = (tm1 - tm2) // 2
    for k in range(0, tj + 1):
        a, b, e, f = jpm2 - k, k, jmm1 - k, k + dm
        if a < 0 or e < 0 or f < 0:
            continue
        ec = tj - 2 * k - dm      # exponent of cos(beta/2): 2j - 2k + m2 - m1
        es = 2 * k + dm           # exponent of sin(beta/2): 2k + m1 - m2
        term = (-1) ** f / (_fact(a) * _fact(b) * _fact(e) * _fact(f))
        d += term * (c ** ec if ec else 1.0) * (s ** es if es else 1.0)
    return pre * d


def dwig(tj, tm1, tm2, beta) -> float:
    """d-function of the single-particle rotation (PNAMP_Proj.f90:126) and of the
    J projection weights D^J*_{K1K2} = e^{i K1 alp} d^J_{K1K2}(bet) e^{i K2 gam}
    (PNAMP_Kernel3D.f90:8, 498-503): Edmonds' d^j_{m1 m2}(beta)."""
    return wigner_d_edmonds(tj, tm1, tm2, beta)


# --------------------------------------------------------------------------
# Mesh
# --------------------------------------------------------------------------
def gauss_legendre(a: float, b: float, n: int):
    """Nodes ascending in [a, b] and weights (Golub-Welsch via numpy)."""
    x, w = np.polynomial.legendre.leggauss(n)
    xm, xl = 0.5 * (b + a), 0.5 * (b - a)
    return xm + xl * x, xl * w


@dataclass
class Mesh:
    """Euler (alpha, beta, gamma) Gauss-Legendre mesh and Fomenko gauge mesh.

    `ncosbet` = 2 uses the beta <-> pi - beta symmetry of the axial loop
    (Codes/PNAMP/PNAMP_Kernel1D.f90:64-66,195,215,463,498): only the first
    nbet/2 Gauss nodes (cos beta < 0) are evaluated, with doubled weight.
    The reference's Ge76 kernel files were produced this way.
    """
    nalp: int
    nbet: int
    ngam: int
    nfom: int
    ncosbet: int = 1
    alpha: np.ndarray = field(init=False)
    beta: np.ndarray = field(init=False)
    gamma: np.ndarray = field(init=False)
    walp: np.ndarray = field(init=False)
    wbet: np.ndarray = field(init=False)
    wgam: np.ndarray = field(init=False)

    def __post_init__(self):
        self.alpha, self.walp = gauss_legendre(0.0, 2 * math.pi, self.nalp)
        xb, self.wbet = gauss_legendre(-1.0, 1.0, self.nbet)
        self.beta = np.arccos(xb)
        self.gamma, self.wgam = gauss_legendre(0.0, 2 * math.pi, self.ngam)
        if self.nalp == 1:
            self.alpha[:] = 0.0
            self.walp[:] = 1.0
        if self.nbet == 1:
            self.beta[:] = 0.0
            self.wbet[:] = 1.0
        if self.ngam == 1:
            self.gamma[:] = 0.0
            self.wgam[:] = 1.0

    @property
    def nbet_used(self) -> int:
        return max(self.nbet // self.ncosbet, 1)

    @property
    def n_euler(self) -> int:
        return self.nalp * self.nbet_used * self.ngam

    @property
    def n_gauge(self) -> int:
        return self.nfom * self.nfom

    def euler_points(self):
        """(alpha, beta, gamma, w_a*w_b*w_g) in the reference's loop order:
        beta outer, alpha, gamma inner (Codes/PNAMP/PNAMP_Kernel3D.f90:200-217)."""
        pts = []
        for k in range(self.nbet_used):
            for kk in range(self.nalp):
                for kg in range(self.ngam):
                    pts.append((self.alpha[kk], self.beta[k], self.gamma[kg],
                                self.walp[kk] * self.wbet[k] * self.wgam[kg] * self.ncosbet))
        return np.array(pts, dtype=np.float64)

    def gauge_angles(self):
        """phi_l = 2 pi l / NFOM, l = 0..NFOM-1 (Kernel3D.f90:264,273); 0 if NFOM = 1."""
        if self.nfom == 1:
            return np.zeros(1)
        return (2 * math.pi / self.nfom) * np.arange(self.nfom)


# --------------------------------------------------------------------------
# One-body operators
# --------------------------------------------------------------------------
def j_operators(sp: ModelSpace):
    """Jx, Jy, Jz, Jx^2, Jy^2, Jz^2 in the m-scheme (zJiME, PNAMP_ME1B.f90:332-422).

    Returned as complex n x n arrays indexed [a, b] (row a, column b).
    """
    n = sp.nlev
    JX, JY, JZ = (np.zeros((n, n), complex) for _ in range(3))
    JX2, JY2, JZ2 = (np.zeros((n, n), complex) for _ in range(3))
    for a in range(n):
        for b in range(n):
            if not (sp.n[a] == sp.n[b] and sp.l[a] == sp.l[b] and sp.twoj[a] == sp.twoj[b] and sp.t[a] == sp.t[b]):
                continue
            jb, mb = sp.twoj[b] / 2.0, sp.twom[b] / 2.0
            ma2, mb2 = int(sp.twom[a]), int(sp.twom[b])
            fp1 = jb * (jb + 1) - mb * (mb + 1)
            fm1 = jb * (jb + 1) - mb * (mb - 1)
            fp1p2 = jb * (jb + 1) - (mb + 1) * (mb + 2)
            fm1m2 = jb * (jb + 1) - (mb - 1) * (mb - 2)
            f02 = jb * (jb + 1) - mb ** 2
            dp1 = 1.0 if ma2 == mb2 + 2 else 0.0
            dm1 = 1.0 if ma2 == mb2 - 2 else 0.0
            dp2 = 1.0 if ma2 == mb2 + 4 else 0.0
            dm2 = 1.0 if ma2 == mb2 - 4 else 0.0
            d0 = 1.0 if ma2 == mb2 else 0.0
            sfp1 = math.sqrt(max(fp1, 0.0))
            sfm1 = math.sqrt(max(fm1, 0.0))
            JX[a, b] = 0.5 * (sfp1 * dp1 + sfm1 * dm1)
            JY[a, b] = -0.5j * (sfp1 * dp1 - sfm1 * dm1)
            JZ[a, b] = mb * d0
            s1 = math.sqrt(max(fp1 * fp1p2, 0.0))
            s2 = math.sqrt(max(fm1 * fm1m2, 0.0))
            JX2[a, b] = 0.25 * (s1 * dp2 + s2 * dm2 + 2 * f02 * d0)
            JY2[a, b] = -0.25 * (s1 * dp2 + s2 * dm2 - 2 * f02 * d0)
            JZ2[a, b] = (mb * d0) ** 2
    return JX, JY, JZ, JX2, JY2, JZ2


def _ho_radial_r2(n1: int, l1: int, n2: int, l2: int) -> float:
    """<n1 l1 | r^2 | n2 l2> for harmonic-oscillator radial functions, b = 1.

    n1, n2 counted from 0, l1 + l2 even. With R_nl(r) = N r^l exp(-r^2/2)
    L_n^{l+1/2}(r^2), N^2 = 2 n! / Gamma(n + l + 3/2), and x = r^2 the integral is
    N1 N2 / 2 * int x^{1/2} e^{-x} x^{(l1+l2)/2 + 1} L1 L2 dx: generalized
    Gauss-Laguerre (alpha = 1/2) with 40 nodes integrates it exactly.
    """
    from scipy.special import eval_genlaguerre, gammaln, roots_genlaguerre
    x, w = roots_genlaguerre(40, 0.5)

    def norm(nn, ll):
        return math.sqrt(2.0 * math.exp(gammaln(nn + 1) - gammaln(nn + ll + 1.5)))
    g = (x ** ((l1 + l2) // 2 + 1)
         * eval_genlaguerre(n1, l1 + 0.5, x) * eval_genlaguerre(n2, l2 + 0.5, x))
    return 0.5 * norm(n1, l1) * norm(n2, l2) * float(np.sum(w * g))


def q2_operators(sp: ModelSpace, b2: float = 4.2627833):
    """Quadrupole operators Q_{2mu}, mu = -2..2, in the m-scheme.

    Follows the structure of q2mume_KB (Codes/PNAMP/VAPHFB_Q2.f90:206-312):
    <a| r^2 Y_2mu |b> from the l-s uncoupled sum, isospin-diagonal, with the
    fixed b^2 = 4.2627833 of that routine, the factor sqrt(5/(4 pi)) on both
    species and the division by sqrt(5/(4 pi)). Returned as real arrays
    [mu+2][a, b].
    """
    n = sp.nlev
    Q = np.zeros((5, n, n))
    fac = math.sqrt(5.0 / (4 * math.pi))
    for a in range(n):
        la, ja, ma, ta = int(sp.l[a]), int(sp.twoj[a]), int(sp.twom[a]), int(sp.t[a])
        for b in range(n):
            lb, jb, mb, tb = int(sp.l[b]), int(sp.twoj[b]), int(sp.twom[b]), int(sp.t[b])
            if ta != tb:
                continue
            factor = math.sqrt(((2 * lb + 1) * 5.0) / (4 * math.pi * (2 * la + 1)))
            cbcomm = cg(4, 2 * lb, 2 * la, 0, 0, 0)
            if cbcomm == 0.0:
                continue
            radial = _ho_radial_r2(int(sp.n[a]) - 1, la, int(sp.n[b]) - 1, lb) * b2
            sums = np.zeros(5)
            for mla in range(-la, la + 1):
                for mlb in range(-lb, lb + 1):
                    for jms in (-1, 1):
                        cb1 = cg(2 * la, 1, ja, 2 * mla, jms, ma)
                        cb2 = cg(2 * lb, 1, jb, 2 * mlb, jms, mb)
                        if cb1 == 0.0 or cb2 == 0.0:
                            continue
                        for k, mu in enumerate((-2, -1, 0, 1, 2)):
                            sums[k] += cb1 * cb2 * cg(4, 2 * lb, 2 * la, 2 * mu, 2 * mlb, 2 * mla)
            Q[:, a, b] = fac * factor * cbcomm * radial * sums / fac
    return Q
