"""Shell-model interactions in the proton-neutron J-scheme and their m-scheme form.

SCCM ships its interactions twice: as J-coupled proton-neutron records
`t1 t2 t3 t4 n1 n2 n3 n4 lj1 lj2 lj3 lj4 J me` (e.g. Codes/int/KB3G/SM_KB3G_ME2B.dat,
the format read at Codes/PNAMP/IMSRG_GenerateH_JTMT.f90:108) and as the
antisymmetrised m-scheme list that PNAMP reads record by record
(Codes/int/KB3G/IMSRG_s000_KB3Gpf_hwHO11_m1m2m3m4.dat, one real*8 per
(a < b, c < d, a + b <= c + d) record of `mscheme_pairs`). The reference goes from
the first to the second through isospin (J -> JT M_T, IMSRG_GenerateH_JTMT.f90:137-190,
then the Clebsch-Gordan sum of Codes/GCM/HFBA_Hamiltonian.f90:295-365). The isospin
Clebsch-Gordan coefficients sum out by completeness, so the m-scheme element is

    V(a b c d) = sum_J <j_a m_a j_b m_b | J M> <j_c m_c j_d m_d | J M> V_J(a b, c d)

with the proton-neutron V_J read per (orbit, charge) and extended by the exchange
phases (-1)^(j1 + j2 + J + 1) of IMSRG_GenerateH_JTMT.f90:117-126; no pair
normalisation and no Condon-Shortley phase enter (iCS = 1). `uncouple_pn`
computes exactly this; on the shipped KB3G files it reproduces all 14,442
m-scheme records to 6e-12 (tests/test_reference_pins.py).

Charge labels: the J-scheme files use t = 0 neutron, 1 proton; the m-scheme basis
uses t = -1 proton, +1 neutron (tnljm%t).
"""
from __future__ import annotations

import math

import numpy as np

from .basis import ModelSpace, cg
from .formats import FormatError, mscheme_pairs


def file_charge(t_mscheme: int) -> int:
    """m-scheme charge label (-1 proton, +1 neutron) -> J-scheme file label (1 proton, 0 neutron)."""
    return 1 if int(t_mscheme) == -1 else 0


def jscheme_table(orbits, records):
    """{((o1, t1), (o2, t2), (o3, t3), (o4, t4), J): V_J} from J-scheme records.

    `orbits` is the model space's orbit list [(n0, l, 2j)] (.val order); `records`
    are (t1..t4, n1..n4, lj1..lj4, J, me) tuples as `formats.read_sm_me2b` returns
    them (n from 0, lj = l + j - 1/2). Each record fills the eight index orders that
    antisymmetry and hermiticity give (IMSRG_GenerateH_JTMT.f90:117-126, real V).
    Orbits the model space does not hold raise FormatError; two records that imply
    different values for one entry raise FormatError as well.
    """
    key = {}
    for io, (n0, l, tj) in enumerate(orbits):
        key[(int(n0), (2 * int(l) + int(tj) - 1) // 2)] = io
    table = {}

    def put(k, v):
        old = table.get(k)
        if old is not None and abs(old - v) > 1e-9 * max(1.0, abs(v)):
            raise FormatError(f"J-scheme records disagree at {k}: {old} vs {v}")
        table[k] = v

    for r in records:
        t1, t2, t3, t4, n1, n2, n3, n4, lj1, lj2, lj3, lj4, J, me = r
        try:
            o = [key[(n1, lj1)], key[(n2, lj2)], key[(n3, lj3)], key[(n4, lj4)]]
        except KeyError as e:
            raise FormatError(f"J-scheme record names an orbit outside the model space: {e}") from None
        tj = [orbits[x][2] for x in o]
        p12 = (-1.0) ** ((tj[0] + tj[1]) // 2 + J + 1)
        p34 = (-1.0) ** ((tj[2] + tj[3]) // 2 + J + 1)
        a, b, c, d = (o[0], t1), (o[1], t2), (o[2], t3), (o[3], t4)
        me = float(me)
        put((a, b, c, d, J), me)
        put((b, a, c, d, J), me * p12)
        put((a, b, d, c, J), me * p34)
        put((b, a, d, c, J), me * p12 * p34)
        put((c, d, a, b, J), me)
        put((d, c, a, b, J), me * p34)
        put((c, d, b, a, J), me * p12)
        put((d, c, b, a, J), me * p12 * p34)
    return table


def uncouple_pn(sp: ModelSpace, table, recs=None, scale=1.0):
    """Antisymmetrised m-scheme V for the record list from a proton-neutron J-scheme table.

    `scale` multiplies every element (the reference's H%ddd_tbme mass scaling,
    1 for the shipped files).
    """
    recs = mscheme_pairs(sp) if recs is None else recs
    tj, tm, orb = sp.twoj.astype(int), sp.twom.astype(int), sp.orbit.astype(int)
    lab = [(int(orb[k]), file_charge(sp.t[k])) for k in range(sp.nlev)]
    out = np.zeros(len(recs))
    for e, (a, b, c, d) in enumerate(recs):
        M2 = int(tm[a] + tm[b])
        ka, kb, kc, kd = lab[a], lab[b], lab[c], lab[d]
        jmin = max(abs(tj[a] - tj[b]), abs(tj[c] - tj[d]), abs(M2)) // 2
        jmin = max(jmin, (abs(M2) + 1) // 2)
        jmax = min(tj[a] + tj[b], tj[c] + tj[d]) // 2
        s = 0.0
        for J in range(jmin, jmax + 1):
            v = table.get((ka, kb, kc, kd, J))
            if v is None or v == 0.0:
                continue
            c1 = cg(int(tj[a]), int(tj[b]), 2 * J, int(tm[a]), int(tm[b]), M2)
            if c1 == 0.0:
                continue
            c2 = cg(int(tj[c]), int(tj[d]), 2 * J, int(tm[c]), int(tm[d]), M2)
            s += c1 * c2 * v
        out[e] = scale * s
    return out


def isospin_to_pn(sp: ModelSpace, vjt):
    """Proton-neutron J-scheme table of an isospin-symmetric V_JT(ab, cd).

    `vjt` is keyed (a, b, c, d, J, T) over orbit indices (as `synth.random_vjt`).
    V_J(a t_a, b t_b, c t_c, d t_d) = sum_T <t_a t_b | T M_T> <t_c t_d | T M_T>
    V_JT / (N_ab N_cd), N_ab = sqrt(1 - d_ab (-1)^(J+T)) / (1 + d_ab): the inverse of
    the isospin step of IMSRG_GenerateH_JTMT.f90:161-180 with the pair normalisation
    that HFBA_Hamiltonian.f90:331-337 divides out. Used to check the isospin
    uncoupling of `synth.uncouple` against `uncouple_pn`.
    """
    from .synth import _vjt_lookup
    orbs = sp.orbits
    no = len(orbs)
    table = {}
    for a in range(no):
        for b in range(no):
            for c in range(no):
                for d in range(no):
                    if (orbs[a][1] + orbs[b][1] + orbs[c][1] + orbs[d][1]) % 2:
                        continue
                    ja, jb, jc, jd = orbs[a][2], orbs[b][2], orbs[c][2], orbs[d][2]
                    for J in range(max(abs(ja - jb), abs(jc - jd)) // 2, min(ja + jb, jc + jd) // 2 + 1):
                        for ta in (0, 1):
                            for tb in (0, 1):
                                for tc in (0, 1):
                                    for td in (0, 1):
                                        if ta + tb != tc + td:
                                            continue
                                        # file labels 1 proton / 0 neutron -> doubled t_z -1 / +1
                                        za, zb, zc, zd = (1 - 2 * x for x in (ta, tb, tc, td))
                                        mt2 = za + zb
                                        s = 0.0
                                        for T in (0, 1):
                                            if abs(mt2) > 2 * T:
                                                continue
                                            ph = (-1.0) ** (J + T)
                                            nab = math.sqrt(1 - (a == b) * ph) / (1 + (a == b))
                                            ncd = math.sqrt(1 - (c == d) * ph) / (1 + (c == d))
                                            if nab <= 1e-15 or ncd <= 1e-15:
                                                continue
                                            c3 = cg(1, 1, 2 * T, za, zb, mt2)
                                            c4 = cg(1, 1, 2 * T, zc, zd, mt2)
                                            s += c3 * c4 * _vjt_lookup(vjt, sp, a, b, c, d, J, T) / (nab * ncd)
                                        if s != 0.0:
                                            table[((a, ta), (b, tb), (c, tc), (d, td), J)] = s
    return table
