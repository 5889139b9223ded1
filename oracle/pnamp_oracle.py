"""ORACLE — test infrastructure only.

CPU FP64 restatement of SCCM's PNAMP per-point algorithm, used by the tests,
`__graft_entry__.smoke()` and the CPU leg of `bench.py` as the checker. The
product path (the CUDA library behind `include/pnamp_gpu.h`) never imports or
calls anything in this directory.

It follows the reference call sequence literally (per-point ZGEMM / LU-inverse
/ Pfaffian, sparse energy loop), not the GPU's algebraically reorganised form,
so a GPU-vs-oracle comparison checks the reorganisation as well as the kernels.

Parity pins: the axial path reproduces the reference's own Ge76 output files
`data/Ge/kern.1D.*.elem` (tests/test_oracle_golden.py). The triaxial Pfaffian
path has no reference output to pin against; it is cross-checked by invariants
(N = 1 at the identity for q = q', Pf^2 = det, Hermiticity of N^J, agreement of
the Pfaffian and Onishi norms where the Onishi sign is unambiguous).

Reference files (paths inside jmyao17/SCCM):
  PNAMP_Kernel3D.f90   mesh loop, norm assembly, projection      (Codes/PNAMP)
  PNAMP_Kernel3D_v2.f90:477-498  plain D-function projection
  PNAMP_Kernel1D.f90   axial loop (Onishi norm) and K=0 projection
  PNAMP_Proj.f90       zbareover, ROTATION_MAT, Pfaf_Over, ZPfaffianF, ZExch,
                       UVphiomega, ROKAPPAphiomega
  PNAMP_Energy_OpenMP.f90  HFB_Energy_COMPLEX
  PNAMP_ME1B.f90       ZN_0, ZQ2, ZQ2t
  PNAMP_ME2B.f90       ZJ2_0
  PNAMP_Onishi.f90     Onishi
  PNAMP_Rho1B.f90      ZRho1B_Angles, ZRho1B_Integral, Write_ME1B
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from sccm_gb300.basis import JJMAX, NOBS, CHOP, ModelSpace, Mesh, dwig


@dataclass
class Hamiltonian:
    """Inputs the reference keeps in module `H` (VAPHFB_Par.f90:45-54)."""
    e0: float
    t1b: np.ndarray          # zME1BM, n x n, [row, col]
    recs: np.ndarray         # (nrec, 4) 0-based a < b, c < d
    vbar: np.ndarray         # (nrec,) antisymmetrised m-scheme V
    q2: np.ndarray           # (5, n, n) Q_{2mu}, mu = -2..2
    jops: tuple              # Jx, Jy, Jz, Jx^2, Jy^2, Jz^2


# ---------------------------------------------------------------- per pair
def zbareover(V, U):
    """PNAMP_Proj.f90:6-79. Returns (ZZc = conj(V U^-1), Det = exp(-1/4 sum log(1+lam)))."""
    uinv = np.linalg.inv(U.astype(complex))             # ZGETRF + ZGETRI
    zz = V.astype(complex) @ uinv                        # Z* = V U^-1
    zzc = np.conj(zz)
    zztz = zzc.T @ zzc
    lam = np.linalg.eigvals(zztz)                        # ZGEEV
    ztest = np.sum(np.log(1.0 + lam))
    return zzc, float(np.real(np.exp(-ztest / 4.0)))


# ---------------------------------------------------------------- per Euler
def rotation_mat(sp: ModelSpace, alp, bet, gam):
    """PNAMP_Proj.f90:83-136: R(a,b) = e^{-i alp m_a} e^{-i gam m_b} d^{j}_{m_a m_b}(bet)."""
    n = sp.nlev
    R = np.zeros((n, n), complex)
    for s, d in sp.blocks():
        tj = int(sp.twoj[s])
        for i in range(d):
            ma = int(sp.twom[s + i])
            for k in range(d):
                mb = int(sp.twom[s + k])
                R[s + i, s + k] = (np.exp(-1j * alp * ma / 2.0) * np.exp(-1j * gam * mb / 2.0)
                                   * dwig(tj, ma, mb, bet))
    return R


def gauge_matrix(R, phip, phin):
    """ZAM_PHI_OMEGA of UVphiomega (PNAMP_Proj.f90:413-439): species blocks of R times e^{i phi}."""
    n = R.shape[0]
    h = n // 2
    A = np.zeros_like(R)
    A[:h, :h] = np.exp(1j * phip) * R[:h, :h]
    A[h:, h:] = np.exp(1j * phin) * R[h:, h:]
    return A


def uvphiomega(A, U1, V1):
    """PNAMP_Proj.f90:441-452: Ubar = A U1, Vbar = conj(A) V1."""
    return A @ U1, np.conj(A) @ V1


# ---------------------------------------------------------------- Pfaffian
def zpfaffian(SK, epsln=1.0e-13):
    """ZPfaffianF (PNAMP_Proj.f90:218-350) with ZExch (:356-392).

    Skew-symmetric Pfaffian by 2x2-block elimination with a global argmax pivot
    over the remaining upper triangle, scanned row by row (first maximum wins),
    sign `phas` per exchange, and Pf = 0 as soon as |pivot| <= epsln. The
    reference reads and exchanges only the upper triangle (ZExch moves upper
    entries with sign flips, PNAMP_Proj.f90:356-392), i.e. it takes the Pfaffian
    of the skew matrix that the upper triangle defines; the input's lower
    triangle (which for a computed M1 = conj(Vbar) conj(Ubar)^-1 is skew only to
    rounding) never enters. Here that matrix is formed once, triu - triu^T, and
    kept in full skew form, so row+column exchanges are pure moves and match the
    reference's upper-triangle storage value for value.
    Returns (Pf, status) with status 1 when the epsln early exit fired.
    """
    A = np.triu(np.asarray(SK, dtype=complex), 1)
    A = A - A.T
    N = A.shape[0]
    if N % 2:
        return 0.0 + 0.0j, 0
    NB = N // 2
    if NB == 1:
        return complex(A[0, 1]), 0
    pf = 1.0 + 0.0j
    iu = None
    for k in range(NB - 1):
        r, c = 2 * k, 2 * k + 1
        sub = np.abs(A[r:, r:])
        m = sub.shape[0]
        if iu is None or iu[0].size != m * (m - 1) // 2:
            iu = np.triu_indices(m, 1)
        flat = sub[iu]
        pos = int(np.argmax(flat))
        i1, i2 = r + int(iu[0][pos]), r + int(iu[1][pos])
        phas = 1.0
        if i1 == r:
            phas = -phas
        if i2 == c:
            phas = -phas
        if i1 != r:
            A[[r, i1], :] = A[[i1, r], :]
            A[:, [r, i1]] = A[:, [i1, r]]
        if i2 != c:
            A[[c, i2], :] = A[[i2, c], :]
            A[:, [c, i2]] = A[:, [i2, c]]
        ss = A[r, c]
        if not abs(ss) > epsln:
            return 0.0 + 0.0j, 1
        if c + 1 < N:
            a = A[c, c + 1:].copy()      # Sk(NC, i)
            b = A[r, c + 1:].copy()      # Sk(NR, i)
            upd = (np.outer(a, b) - np.outer(b, a)) / ss
            blk = A[c + 1:, c + 1:]
            tri = np.triu(np.ones(blk.shape, bool), 1)
            blk[tri] = blk[tri] + upd[tri]
            lowt = np.tril(np.ones(blk.shape, bool), -1)
            blk[lowt] = -blk.T[lowt]
            np.fill_diagonal(blk, 0.0)
            A[c + 1:, c + 1:] = blk
        pf = pf * ss * phas
    pf = pf * A[N - 2, N - 1]
    return complex(pf), 0


def pfaf_over(zzc0, Ubar, Vbar, cscale=1.0):
    """PNAMP_Proj.f90:142-211: Pf( Cscale * [[conj(Vbar) conj(Ubar)^-1, -I], [I, -ZZc0]] )."""
    n = Ubar.shape[0]
    m1 = np.conj(Vbar) @ np.linalg.inv(np.conj(Ubar))
    S = np.zeros((2 * n, 2 * n), complex)
    S[:n, :n] = m1
    S[n:, n:] = -zzc0
    S[:n, n:] = -np.eye(n)
    S[n:, :n] = np.eye(n)
    S *= cscale
    return zpfaffian(S)


# ---------------------------------------------------------------- densities
def rokappa(A, U0, V0, U1, V1):
    """ROKAPPAphiomega (PNAMP_Proj.f90:459-551)."""
    Ac = np.conj(A)
    t22 = V0.T @ A @ V1 + U0.T @ Ac @ U1
    t22inv = np.linalg.inv(t22)
    aux1 = A @ V1
    aux2 = -(Ac @ U1)
    aux3 = t22inv @ V0.T
    aux4 = t22inv @ U0.T
    return aux1 @ aux3, aux1 @ aux4, aux2 @ aux3


def zn0(rho):
    """ZN_0 (PNAMP_ME1B.f90:218-237): proton (first half) and neutron traces."""
    h = rho.shape[0] // 2
    return np.trace(rho[:h, :h]), np.trace(rho[h:, h:])


def energy(rho, k10, k01, ham: Hamiltonian):
    """HFB_Energy_COMPLEX (PNAMP_Energy_OpenMP.f90:31-90). Returns (Ekin, Etot)."""
    i, j, k, l = (ham.recs[:, q] for q in range(4))
    R = rho
    z_ijkl = R[k, i] * R[l, j] - R[l, i] * R[k, j] + k01[i, j] * k10[k, l]
    z_jikl = R[k, j] * R[l, i] - R[l, j] * R[k, i] + k01[j, i] * k10[k, l]
    z_jilk = R[l, j] * R[k, i] - R[k, j] * R[l, i] + k01[j, i] * k10[l, k]
    z_ijlk = R[l, i] * R[k, j] - R[k, i] * R[l, j] + k01[i, j] * k10[l, k]
    z_klij = R[i, k] * R[j, l] - R[j, k] * R[i, l] + k01[k, l] * k10[i, j]
    z_klji = R[j, k] * R[i, l] - R[i, k] * R[j, l] + k01[k, l] * k10[j, i]
    z_lkij = R[i, l] * R[j, k] - R[j, l] * R[i, k] + k01[l, k] * k10[i, j]
    z_lkji = R[j, l] * R[i, k] - R[i, l] * R[j, k] + k01[l, k] * k10[j, i]
    d = np.where(k + l == i + j, 0.0, 1.0)
    e2 = np.sum(0.25 * ham.vbar * (z_ijkl + d * z_klij - z_jikl - d * z_klji
                                   - z_ijlk - d * z_lkij + z_jilk + d * z_lkji))
    ekin = np.sum(R.T * ham.t1b)           # sum_{a,c} rho(c,a) t(a,c)
    return ekin, e2 + ekin


def zj2(rho, k10, k01, jops):
    """ZJ2_0 (PNAMP_ME2B.f90:1-152): <J^2> from J_i, J_i^2 traces."""
    JX, JY, JZ, JX2, JY2, JZ2 = jops
    tot = 0.0 + 0.0j
    for J, J2 in ((JX, JX2), (JY, JY2), (JZ, JZ2)):
        a1 = J2 @ rho
        a2 = J @ rho
        a3 = J @ k10
        a4 = J.T @ k01.T
        tot += np.trace(a1) + np.trace(a2) ** 2 - np.trace(a2 @ a2) + np.trace(a3 @ a4)
    return tot


def zq2(Q, rho):
    """ZQ2 (PNAMP_ME1B.f90:52-79): proton trace of Q rho."""
    h = rho.shape[0] // 2
    aux = Q @ rho
    return np.trace(aux[:h, :h]), np.trace(aux[h:, h:])


def zq2t(Q, rho):
    """ZQ2t (PNAMP_ME1B.f90:112-132): proton trace of Q^dagger rho."""
    h = rho.shape[0] // 2
    aux = np.conj(Q).T @ rho
    return np.trace(aux[:h, :h]), np.trace(aux[h:, h:])


def onishi(U0, V0, Ubar, Vbar):
    """Onishi (PNAMP_Onishi.f90:1-37): sqrt(det(Ubar^T U0 + Vbar^T V0)), principal branch."""
    b = Ubar.T @ U0 + Vbar.T @ V0
    return complex(np.sqrt(np.linalg.det(b) + 0j))


# ---------------------------------------------------------------- one point
def point_observables(sp, ham, A, U0, V0, U1, V1, znorm, iE2=True):
    """Observables 2..18 for one gauge point, weighted by the norm (Kernel3D.f90:296-358)."""
    out = np.zeros(NOBS, complex)
    rho, k10, k01 = rokappa(A, U0, V0, U1, V1)
    zp, zn = zn0(rho)
    out[0] = znorm
    out[1] = znorm * zp
    out[2] = znorm * zn
    ekin, ehfb = energy(rho, k10, k01, ham)
    out[3] = znorm * ekin
    out[6] = znorm * (ehfb + ham.e0)
    out[7] = znorm * zj2(rho, k10, k01, ham.jops)
    if iE2:
        for mu in range(5):
            out[8 + mu] = znorm * zq2(ham.q2[mu], rho)[0]
            out[13 + mu] = znorm * zq2t(ham.q2[mu], rho)[0]
    return out


def rho1b_table(sp: ModelSpace):
    """Blocks of ZRho1B_Angles (PNAMP_Rho1B.f90:14-29): [(it, lj, n1, n2, twoj), [(k1, k2), ...]].

    States k1, k2 of the same isospin, lj and m; it = 1 for protons (t = -1), 0
    for neutrons; n from 0; ordered it, lj, n1, n2 as Write_ME1B loops
    (PNAMP_Rho1B.f90:80-88)."""
    blocks = {}
    n = sp.nlev
    for k1 in range(n):
        for k2 in range(n):
            if sp.t[k1] != sp.t[k2] or sp.lj[k1] != sp.lj[k2] or sp.twom[k1] != sp.twom[k2]:
                continue
            it = 1 if sp.t[k1] == -1 else 0
            key = (it, int(sp.lj[k1]), int(sp.n[k1]) - 1, int(sp.n[k2]) - 1, int(sp.twoj[k1]))
            blocks.setdefault(key, []).append((k1, k2))
    return sorted(blocks.items())


def rho1b_point(table, rho, znorm):
    """ZRho1B_Angles for one gauge point: znorm * sum ZRO(k1, k2) / sqrt(2j + 1) per block
    (the 1/NFOM^2 is applied with the gauge mean)."""
    return np.array([znorm * sum(rho[k1, k2] for k1, k2 in ent) / math.sqrt(key[4] + 1.0)
                     for key, ent in table], complex)


def rho1b_write_me1b(table, zres, r, mesh: Mesh):
    """ZRho1B_Integral at J = 0 and Write_ME1B (PNAMP_Rho1B.f90:36-91) for one pair.

    r [P_E, nblocks] are the gauge means from `kernel_triaxial(..., rho1b=...)`.
    Returns Re(sum_e w_e r_e / N^0) / sqrt(2j + 1) per block (the J = 0 weight
    cancels in the ratio), or None when |N^0| <= CHOP (the reference warns and
    writes nothing)."""
    w = mesh.euler_points()[:, 3]
    zn = np.sum(w * zres[:, 0])
    if abs(zn) <= CHOP:
        return None
    zr = w @ r
    return np.array([np.real(zr[b] / zn) / math.sqrt(key[4] + 1.0) for b, (key, _) in enumerate(table)])


def rho2b_blocks(sp: ModelSpace):
    """Two-particle blocks |(nlj)_1 (nlj)_2; J, PP, tt> of ME2B_Base_Full
    (PNAMP_ME2B_Base.f90:112-205) over the model space's orbits.

    Returns [(tt, PP, J, [(o1, o2), ...])] in the block order bm of
    PNAMP_ME2B_Base.f90:182-205 (tt = 0 nn, 1 np, 2 pp; PP = 0 positive parity;
    J ascending); o1, o2 index `sp.orbits`. Within a block the states follow the
    enumeration of PNAMP_ME2B_Base.f90:128-171: (l1, j1), (l2, j2) ascending by
    LJ = (2l + 2j - 1)/2, then n1, n2; for nn and pp only id1 <= id2
    (id = n + nMax LJ) and identical orbits only at even J. The reference builds
    the blocks over its full oscillator space; restricted to the model space the
    numbering is the reference's whenever the model space is that full space.
    """
    nmax = max(n0 for n0, _, _ in sp.orbits) + 1
    lj = lambda o: (2 * sp.orbits[o][1] + sp.orbits[o][2] - 1) // 2
    ident = lambda o: sp.orbits[o][0] + 1 + nmax * lj(o)
    orbs = sorted(range(len(sp.orbits)), key=lambda o: (lj(o), sp.orbits[o][0]))
    ljs = sorted({lj(o) for o in orbs})
    blocks = {}
    for tt in range(3):
        for lj1 in ljs:
            for lj2 in ljs:
                o1s = [o for o in orbs if lj(o) == lj1]
                o2s = [o for o in orbs if lj(o) == lj2]
                _, l1, tj1 = sp.orbits[o1s[0]]
                _, l2, tj2 = sp.orbits[o2s[0]]
                pp = (l1 + l2) % 2
                for J in range(abs(tj1 - tj2) // 2, (tj1 + tj2) // 2 + 1):
                    for o1 in o1s:
                        for o2 in o2s:
                            if tt != 1 and ident(o1) > ident(o2):
                                continue
                            if J % 2 == 1 and o1 == o2 and tt != 1:
                                continue
                            blocks.setdefault((tt, pp, J), []).append((o1, o2))
    return [(tt, pp, J, blocks[(tt, pp, J)]) for (tt, pp, J) in sorted(blocks)]


def _level(sp: ModelSpace, o, t_ref, tm):
    """tnljm%level(m, lj, n, t) for the reference's t (1 proton, 0 neutron)."""
    t = -1 if t_ref == 1 else 1
    for k in range(sp.nlev):
        if sp.t[k] == t and sp.orbit[k] == o and sp.twom[k] == tm:
            return k
    raise KeyError((o, t_ref, tm))


def rho2b_terms(sp: ModelSpace, blocks=None):
    """The m sums of ZRho2B_Angles (PNAMP_Rho2B.f90:31-118) as a sparse map.

    Returns (quads [nq, 4] of levels (k_i, k_j, k_k, k_l), terms) where terms lists,
    per element (bm, a_ij, a_kl) in block order, [(q, cg1 cg2 / (2J + 1)), ...].
    Every quadruple conserves M = m_i + m_j = m_k + m_l; quads are unique and in
    first-use order."""
    from sccm_gb300.basis import cg
    blocks = rho2b_blocks(sp) if blocks is None else blocks
    qidx, quads, terms = {}, [], []
    for tt, _pp, J, states in blocks:
        t1, t2 = tt // 2, (tt + 1) // 2
        for oi, oj in states:
            tji, tjj = sp.orbits[oi][2], sp.orbits[oj][2]
            for ok, ol in states:
                tjk, tjl = sp.orbits[ok][2], sp.orbits[ol][2]
                el = []
                for mi in range(-tji, tji + 1, 2):
                    ki = _level(sp, oi, t1, mi)
                    for mj in range(-tjj, tjj + 1, 2):
                        kj = _level(sp, oj, t2, mj)
                        c1 = cg(tji, tjj, 2 * J, mi, mj, mi + mj)
                        for mk in range(-tjk, tjk + 1, 2):
                            ml = mi + mj - mk
                            if abs(ml) > tjl:
                                continue
                            c2 = cg(tjk, tjl, 2 * J, mk, ml, mi + mj)
                            if c1 * c2 == 0.0:
                                continue
                            key = (ki, kj, _level(sp, ok, t1, mk), _level(sp, ol, t2, ml))
                            if key not in qidx:
                                qidx[key] = len(quads)
                                quads.append(key)
                            el.append((qidx[key], c1 * c2 / (2 * J + 1)))
                terms.append(el)
    return np.array(quads, dtype=np.int64).reshape(-1, 4), terms


def rho2b_point(quads, rho, k10, k01, znorm):
    """One gauge point of ZRho2B_Angles before the CG sums (PNAMP_Rho2B.f90:105-112):
    znorm [ZRO(k,i) ZRO(l,j) - ZRO(l,i) ZRO(k,j) + ZKAPA01(i,j) ZKAPA10(k,l)] per quadruple
    (the 1/NFOM^2 is applied with the gauge mean)."""
    i, j, k, l = quads.T
    return znorm * (rho[k, i] * rho[l, j] - rho[l, i] * rho[k, j] + k01[i, j] * k10[k, l])


def rho2b_write_me2b(terms, zres, a, mesh: Mesh):
    """ZRho2B_Integral at J = 0 and the valence entries of Write_ME2B
    (PNAMP_Rho2B.f90:137-296) for one pair.

    a [P_E, nq] are the gauge means from `kernel_triaxial(..., rho2b=quads)`. Returns
    the complex Rho2BN per element (bm, a_ij, a_kl) in block order, = sum_e w_e
    sum_q c_q a_eq / N^0 (the J = 0 weight cancels in the ratio), or None when
    |N^0| <= CHOP (Rho2BN = 0 there in the reference)."""
    w = mesh.euler_points()[:, 3]
    zn = np.sum(w * zres[:, 0])
    if abs(zn) <= CHOP:
        return None
    za = w @ a
    return np.array([sum(c * za[q] for q, c in el) for el in terms], complex) / zn


def kernel_triaxial(sp: ModelSpace, ham: Hamiltonian, mesh: Mesh, U0, V0, U1, V1,
                    cscale=1.0, iscale=0, iE2=True, euler_subset=None, point_log=None, rho1b=None,
                    rho2b=None):
    """Kernel4Triaxial mesh loop (PNAMP_Kernel3D.f90:70-407) -> ZRES[P_E, NOBS].

    Shell-model runs take the Pfaffian branch (ide forced to 1, Kernel3D.f90:140-159)
    unless NFOM = 1, where the Onishi formula gives the norm (Kernel3D.f90:286-290). `euler_subset` restricts the loop to a list of Euler
    indices (rows of ZRES left zero elsewhere) so tests can sample large meshes.
    With `rho1b` (a `rho1b_table`), returns (ZRES, R) with R[P_E, nblocks] the
    gauge means of ZRho1B_Angles (Kernel3D.f90:367). With `rho2b` (the quads of
    `rho2b_terms`), returns (ZRES, A) with A[P_E, nq] the gauge means of
    `rho2b_point` (ZRho2B_Angles, Kernel3D.f90:369); both: (ZRES, R, A).
    """
    n = sp.nlev
    U0, V0, U1, V1 = (np.asarray(x, dtype=float) for x in (U0, V0, U1, V1))
    aaa = n * (n + 1) // 2
    snpfaf = -1.0 if aaa % 2 else 1.0
    zzc0, det0 = zbareover(V0, U0)
    _zzc1, det1 = zbareover(V1, U1)
    scale = 10.0 ** (-(n * iscale // 2))
    zdv0, zdv1 = det0 * scale, det1 * scale
    pts = mesh.euler_points()
    phis = mesh.gauge_angles()
    nf = mesh.nfom
    zres = np.zeros((len(pts), NOBS), complex)
    r1 = np.zeros((len(pts), len(rho1b) if rho1b is not None else 0), complex)
    r2 = np.zeros((len(pts), len(rho2b) if rho2b is not None else 0), complex)
    idx = range(len(pts)) if euler_subset is None else euler_subset
    for ie in idx:
        alp, bet, gam, _w = pts[ie]
        R = rotation_mat(sp, alp, bet, gam)
        acc = np.zeros(NOBS, complex)
        for php in phis:
            zph_p = np.exp(-1j * php * sp.nprot)
            for phn in phis:
                zph_n = np.exp(-1j * phn * sp.nneut)
                A = gauge_matrix(R, php, phn)
                ub, vb = uvphiomega(A, U1, V1)
                if nf == 1:   # Kernel3D.f90:286-290: no number projection -> Onishi
                    pf = znorm = onishi(U0, V0, ub, vb)
                else:
                    pf, st = pfaf_over(zzc0, ub, vb, cscale)
                    znorm = snpfaf * zdv0 * zdv1 * pf * zph_p * zph_n
                o = point_observables(sp, ham, A, U0, V0, U1, V1, znorm, iE2)
                if point_log is not None:
                    point_log.append((ie, php, phn, pf, o))
                acc += o
                if rho1b is not None:
                    r1[ie] += rho1b_point(rho1b, rokappa(A, U0, V0, U1, V1)[0], znorm)
                if rho2b is not None:
                    r2[ie] += rho2b_point(rho2b, *rokappa(A, U0, V0, U1, V1), znorm)
        zres[ie] = acc / nf ** 2
        r1[ie] /= nf ** 2
        r2[ie] /= nf ** 2
    out = (zres,) + ((r1,) if rho1b is not None else ()) + ((r2,) if rho2b is not None else ())
    return out if len(out) > 1 else zres


def kernel_axial(sp: ModelSpace, ham: Hamiltonian, mesh: Mesh, U0, V0, U1, V1, iE2=True):
    """Kernel4Axial mesh loop (PNAMP_Kernel1D.f90:190-426): Onishi norm at every gauge point."""
    U0, V0, U1, V1 = (np.asarray(x, dtype=float) for x in (U0, V0, U1, V1))
    pts = mesh.euler_points()
    phis = mesh.gauge_angles()
    nf = mesh.nfom
    zres = np.zeros((len(pts), NOBS), complex)
    for ie, (alp, bet, gam, _w) in enumerate(pts):
        R = rotation_mat(sp, alp, bet, gam)
        acc = np.zeros(NOBS, complex)
        for php in phis:
            zph_p = np.exp(-1j * php * sp.nprot)
            for phn in phis:
                zph_n = np.exp(-1j * phn * sp.nneut)
                A = gauge_matrix(R, php, phn)
                ub, vb = uvphiomega(A, U1, V1)
                znorm = onishi(U0, V0, ub, vb)
                acc += point_observables(sp, ham, A, U0, V0, U1, V1, znorm, iE2)
        zres[ie] = acc / nf ** 2
    return zres


# ---------------------------------------------------------------- projection
def projection_weights(mesh: Mesh, jmax=JJMAX):
    """Plain D-function quadrature weights (PNAMP_Kernel3D_v2.f90:477-498).

    W[J, K1+JJMAX, K2+JJMAX, ie] = weightJ * w_a w_b w_g e^{i K1 alp} d^J_{K1K2}(bet) e^{i K2 gam}
    with weightJ = (2J+1)/(8 pi^2), or (2J+1)/2 when N_alp N_gam = 1 (Kernel3D.f90:78-81).
    """
    pts = mesh.euler_points()
    W = np.zeros((jmax + 1, 2 * JJMAX + 1, 2 * JJMAX + 1, len(pts)), complex)
    axial = mesh.nalp * mesh.ngam == 1
    for J in range(0, jmax + 1):
        wj = (2 * J + 1) / 2.0 if axial else (2 * J + 1) / (8 * math.pi ** 2)
        for K1 in range(-J, J + 1):
            for K2 in range(-J, J + 1):
                for ie, (alp, bet, gam, w) in enumerate(pts):
                    W[J, K1 + JJMAX, K2 + JJMAX, ie] = (wj * w * np.exp(1j * K1 * alp)
                                                       * dwig(2 * J, 2 * K1, 2 * K2, bet)
                                                       * np.exp(1j * K2 * gam))
    return W


def project(zres, mesh: Mesh, core_prot=0, core_neut=0, jmax=JJMAX, jstep=2, chop=CHOP):
    """J/K projection of ZRES into the kernel-file fields (Kernel3D.f90:415-751, plain form).

    Returns dict of arrays [J, K1+JJMAX, K2+JJMAX] for njkk, hjkk, nn, zz, J2
    (only even J are filled: Kernel3D.f90:415). Fields below CHOP are left 0.
    """
    W = projection_weights(mesh, jmax)
    S = np.einsum("jabe,eo->jabo", W, zres[:, :8])          # ZsumJKK(io, K1, K2)
    shape = (JJMAX + 1, 2 * JJMAX + 1, 2 * JJMAX + 1)
    out = {k: np.zeros(shape, complex) for k in ("njkk", "hjkk", "nn", "zz", "J2", "q0p", "q0pc")}
    out["qpred"] = np.zeros(shape + (3,), complex)
    out["qcpred"] = np.zeros(shape + (3,), complex)
    out["zsum"] = S
    for J in range(0, jmax + 1, jstep):
        for K1 in range(-J, J + 1):
            for K2 in range(-J, J + 1):
                s = S[J, K1 + JJMAX, K2 + JJMAX]
                if abs(s[0]) < chop:
                    continue
                ix = (J, K1 + JJMAX, K2 + JJMAX)
                out["njkk"][ix] = s[0]
                out["zz"][ix] = s[1] / s[0] + core_prot
                out["nn"][ix] = s[2] / s[0] + core_neut
                out["hjkk"][ix] = s[6]
                out["J2"][ix] = s[7] / s[0]
    return out


def project_axial(zres, mesh: Mesh, core_prot=0, core_neut=0, jmax=JJMAX):
    """K = 0 projection of the axial path (PNAMP_Kernel1D.f90:432-637): no CHOP."""
    pts = mesh.euler_points()
    shape = (JJMAX + 1, 2 * JJMAX + 1, 2 * JJMAX + 1)
    out = {k: np.zeros(shape, complex) for k in ("njkk", "hjkk", "nn", "zz", "J2", "q0p", "q0pc")}
    out["qpred"] = np.zeros(shape + (3,), complex)
    out["qcpred"] = np.zeros(shape + (3,), complex)
    o = JJMAX
    for J in range(0, jmax + 1, 2):
        wj = (2 * J + 1) / 2.0
        s = np.zeros(8, complex)
        for ie, (alp, bet, gam, w) in enumerate(pts):
            s += wj * w * dwig(2 * J, 0, 0, bet) * zres[ie, :8]
        out["nn"][J, o, o] = s[2] / s[0] + core_neut
        out["zz"][J, o, o] = s[1] / s[0] + core_prot
        out["hjkk"][J, o, o] = s[6]
        out["njkk"][J, o, o] = s[0]
        out["J2"][J, o, o] = s[7] / s[0]
    return out


def project_q(zres, mesh: Mesh, exchange=True, jmax=JJMAX):
    """Quadrupole reduced elements <J1 K1 q1||Q2||J2 K2 q2>, J1 = J2 + dJ, dJ = 0, 1, 2.

    Plain D-function form of PNAMP_Kernel3D_v2.f90:515-600 (spectroscopic dJ = 0
    and the dJ = 2 transition element; dJ = 1 is the same formula, the block
    post_general writes at PNAMP_IO.f90:213):
      qpred = wJ (2J1+1) sum_Omega w sum_mu (-1)^(J1-K1) (J1 2 J2; -K1 mu K2p)
              d^J2_{K2p K2}(bet) e^{i K2p alp} e^{i K2 gam} ZRES(Omega, Q_mu),  K2p = K1 - mu
    and, for q1 != q2, the exchanged element from the Q^dagger traces (:536-546):
      qcpred = wJ (2J1+1) sum w sum_{mu,nu} (-1)^(J1-K1) (-1)^|mu-nu| d^2_{-nu,-mu}(bet)
               e^{-i nu alp} e^{-i mu gam} conj(ZRES(Omega, Qt_nu)) (J1 2 J2; -K1 mu K2p)
               d^J2_{K2 K2p}(bet) e^{-i K2 alp} e^{-i K2p gam}.
    Returns arrays [J2][dJ][K1+8][K2+6] (only even J2 filled).
    """
    from sccm_gb300.basis import threej
    pts = mesh.euler_points()
    axial = mesh.nalp * mesh.ngam == 1
    qp = np.zeros((jmax + 1, 3, 17, 13), complex)
    qc = np.zeros_like(qp)
    for J2 in range(0, jmax + 1, 2):
        wj = (2 * J2 + 1) / 2.0 if axial else (2 * J2 + 1) / (8 * math.pi ** 2)
        for dJ in range(3):
            J1 = J2 + dJ
            for K1 in range(-J1, J1 + 1):
                for K2 in range(-J2, J2 + 1):
                    sd = 0.0 + 0.0j
                    sx = 0.0 + 0.0j
                    for mu in range(-2, 3):
                        K2p = K1 - mu
                        if abs(K2p) > J2:
                            continue
                        tj = threej(2 * J1, 4, 2 * J2, -2 * K1, 2 * mu, 2 * K2p)
                        if tj == 0.0:
                            continue
                        ph = (-1.0) ** (J1 - K1)
                        for ie, (alp, bet, gam, w) in enumerate(pts):
                            sd += (w * ph * tj * dwig(2 * J2, 2 * K2p, 2 * K2, bet)
                                   * np.exp(1j * (K2p * alp + K2 * gam)) * zres[ie, 10 + mu])
                            if exchange:
                                for nu in range(-2, 3):
                                    sx += (w * ph * (-1.0) ** abs(mu - nu) * dwig(4, -2 * nu, -2 * mu, bet)
                                           * np.exp(-1j * (nu * alp + mu * gam)) * np.conj(zres[ie, 15 + nu])
                                           * tj * dwig(2 * J2, 2 * K2, 2 * K2p, bet)
                                           * np.exp(-1j * (K2 * alp + K2p * gam)))
                    qp[J2, dJ, K1 + 8, K2 + 6] = wj * (2 * J1 + 1) * sd
                    qc[J2, dJ, K1 + 8, K2 + 6] = wj * (2 * J1 + 1) * sx
    return qp, qc
