"""Seeded synthetic PNAMP inputs: model spaces, HFB vacua and interactions.

There is no public benchmark set for PNAMP; these generators stand in for the
reference's HFB output (`.wf` files) and shell-model interactions with the
shapes, sizes and value distributions of the benchmark configurations:

  * vacua: real, species-diagonal Bogoliubov (U, V) built in the canonical form
    U = O D u, V = O D v (Bloch-Messiah), where D diagonalises a quadrupole-
    deformed single-particle Hamiltonian with parameters (beta2, gamma), the
    occupations come from BCS with a seeded gap, and O = exp(0.3 G) is a random
    real rotation whose generator G commutes with time reversal and conserves
    parity and, unless `pn_mix` is set, charge. Time-reversal pairs (k, Tk)
    carry the pairing, so the vacua are time-reversal symmetric and U is
    invertible (needed by zbareover). With `pn_mix` the generator has proton-
    neutron entries too (a random Hermitian generator with only time reversal
    and parity imposed, as the sd benchmark case is specified), so U and V mix
    the species like the reference's own HFB vacua with proton-neutron pairing
    (data/Ti/Ti48_*.wf) and every pair takes the general, not the species-split,
    path of the kernels.
  * interaction: J-coupled, isospin-symmetric V_JT(ab, cd) ~ N(0, 1 MeV),
    hermitian, parity conserving, uncoupled to the antisymmetrised m-scheme
    list with the Clebsch-Gordan sum of Codes/GCM/HFBA_Hamiltonian.f90:295-365;
    single-particle energies uniform on [-4, 0] MeV; E0 = 0.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .basis import SHELLS, Mesh, ModelSpace, cg, j_operators, q2_operators
from .formats import mscheme_pairs


# ------------------------------------------------------------------ vacua
def time_reversal(sp: ModelSpace):
    """Real matrix tau of time reversal T|j m> = (-1)^(j-m) |j -m> (T = tau K)."""
    n = sp.nlev
    tau = np.zeros((n, n))
    for a in range(n):
        for b in range(n):
            if (sp.t[a], sp.n[a], sp.l[a], sp.twoj[a]) == (sp.t[b], sp.n[b], sp.l[b], sp.twoj[b]) \
                    and sp.twom[b] == -sp.twom[a]:
                tau[b, a] = (-1.0) ** ((int(sp.twoj[a]) - int(sp.twom[a])) // 2)
    return tau


def _conserving_mask(sp: ModelSpace, charge=True):
    same_t = sp.t[:, None] == sp.t[None, :]
    same_par = (sp.l[:, None] - sp.l[None, :]) % 2 == 0
    return (same_t & same_par) if charge else same_par


def random_rotation(sp: ModelSpace, rng, scale=0.3, charge=True):
    """O = exp(scale * G): G real antisymmetric, commuting with tau, parity conserving
    and, with `charge`, charge conserving."""
    from scipy.linalg import expm
    n = sp.nlev
    tau = time_reversal(sp)
    g = rng.standard_normal((n, n)) / math.sqrt(n)
    g = g - g.T
    g = 0.5 * (g - tau @ g @ tau)          # tau^-1 = -tau: commutes with tau
    g *= _conserving_mask(sp, charge)
    return expm(scale * g)


def canonical_pairs(sp: ModelSpace, h, tau, species):
    """Orthonormal time-reversal pairs (v, tau v) spanning one species, by energy."""
    idx = np.where(sp.t == species)[0]
    hs = h[np.ix_(idx, idx)]
    ts = tau[np.ix_(idx, idx)]
    w, vecs = np.linalg.eigh(hs)
    chosen, energies = [], []
    for k in np.argsort(w):
        r = vecs[:, k].copy()
        for c in chosen:
            r -= c * (c @ r)
        nr = np.linalg.norm(r)
        if nr < 0.5:
            continue
        v = r / nr
        vb = ts @ v
        chosen += [v, vb]
        energies.append(float(v @ hs @ v))
        if len(chosen) == len(idx):
            break
    return idx, np.array(chosen).T, np.array(energies)


def bcs_occupations(eps, nval, gap):
    """v_k^2 with sum 2 v^2 = nval (bisection on the Fermi energy)."""
    lo, hi = eps.min() - 50 * gap - 50, eps.max() + 50 * gap + 50
    for _ in range(200):
        lam = 0.5 * (lo + hi)
        v2 = 0.5 * (1 - (eps - lam) / np.sqrt((eps - lam) ** 2 + gap ** 2))
        if 2 * v2.sum() > nval:
            hi = lam
        else:
            lo = lam
    return v2


def deformed_vacuum(sp: ModelSpace, spe_orbit, beta2, gamma_deg, rng, gap=None, rot_scale=0.3,
                    chi=2.0, q2=None, pn_mix=False):
    """Real (U, V) of a deformed BCS vacuum (species-diagonal), then a random T-even
    rotation, which mixes protons and neutrons when `pn_mix` is set."""
    n = sp.nlev
    q2 = q2_operators(sp) if q2 is None else q2
    g = math.radians(gamma_deg)
    qdef = math.cos(g) * q2[2] + math.sin(g) * (q2[0] + q2[4]) / math.sqrt(2.0)
    h = np.diag([spe_orbit[o] for o in sp.orbit]).astype(float) - chi * beta2 * qdef
    h = 0.5 * (h + h.T)
    h += np.diag(1e-6 * np.arange(n) / n)        # split accidental degeneracies reproducibly
    h = 0.5 * (h + (time_reversal(sp) @ h @ time_reversal(sp).T))
    tau = time_reversal(sp)
    U = np.zeros((n, n))
    V = np.zeros((n, n))
    for species, nval in ((-1, sp.nprot), (1, sp.nneut)):
        idx, D, eps = canonical_pairs(sp, h, tau, species)
        gp = gap if gap is not None else 1.0 + 0.5 * rng.random()
        v2 = bcs_occupations(eps, nval, gp)
        u, v = np.sqrt(1 - v2), np.sqrt(v2)
        m = len(idx)
        ub = np.zeros((m, m))
        vb = np.zeros((m, m))
        for k in range(m // 2):
            ub[2 * k, 2 * k] = ub[2 * k + 1, 2 * k + 1] = u[k]
            vb[2 * k + 1, 2 * k] = v[k]
            vb[2 * k, 2 * k + 1] = -v[k]
        U[np.ix_(idx, idx)] = D @ ub
        V[np.ix_(idx, idx)] = D @ vb
    if rot_scale:
        O = random_rotation(sp, rng, rot_scale, charge=not pn_mix)
        U, V = O @ U, O @ V
    return U, V


# ------------------------------------------------------------------ interaction
def random_vjt(sp: ModelSpace, rng, scale=1.0):
    """Hermitian, parity-conserving V_JT(ab, cd) ~ N(0, scale) over orbit quadruples."""
    orbs = sp.orbits
    no = len(orbs)
    V = {}
    keys = []
    for a in range(no):
        for b in range(a, no):
            keys.append((a, b))
    for i1, (a, b) in enumerate(keys):
        for (c, d) in keys[i1:]:
            la, lb, lc, ld = orbs[a][1], orbs[b][1], orbs[c][1], orbs[d][1]
            if (la + lb + lc + ld) % 2:
                continue
            ja, jb, jc, jd = orbs[a][2], orbs[b][2], orbs[c][2], orbs[d][2]
            for J in range(max(abs(ja - jb), abs(jc - jd)) // 2, min(ja + jb, jc + jd) // 2 + 1):
                for T in (0, 1):
                    if a == b and (J + T) % 2 == 0:
                        continue
                    if c == d and (J + T) % 2 == 0:
                        continue
                    V[(a, b, c, d, J, T)] = scale * rng.standard_normal()
    return V


def _vjt_lookup(V, sp, a, b, c, d, J, T):
    """Symmetric extension of the stored V_JT with the exchange phases of
    Codes/GCM/HFBA_Hamiltonian.f90:215-226."""
    orbs = sp.orbits
    ph = lambda x, y: (-1.0) ** ((orbs[x][2] + orbs[y][2]) // 2 + J + T)
    sgn = 1.0
    if a > b:
        a, b = b, a
        sgn *= ph(a, b)
    if c > d:
        c, d = d, c
        sgn *= ph(c, d)
    if (a, b) > (c, d):
        a, b, c, d = c, d, a, b
    return sgn * V.get((a, b, c, d, J, T), 0.0)


def uncouple(sp: ModelSpace, V, recs=None):
    """Antisymmetrised m-scheme V for the record list (HFBA_Hamiltonian.f90:295-365)."""
    recs = mscheme_pairs(sp) if recs is None else recs
    out = np.zeros(len(recs))
    tj, tm, tt, orb = sp.twoj, sp.twom, sp.t, sp.orbit
    for e, (a, b, c, d) in enumerate(recs):
        oa, ob, oc, od = int(orb[a]), int(orb[b]), int(orb[c]), int(orb[d])
        dab = 1.0 if oa == ob else 0.0
        dcd = 1.0 if oc == od else 0.0
        M2 = int(tm[a] + tm[b])
        MT2 = int(tt[a] + tt[b])
        s = 0.0
        jmax = min(int(tj[a] + tj[b]), int(tj[c] + tj[d])) // 2
        jmin = max(abs(int(tj[a] - tj[b])), abs(int(tj[c] - tj[d])), abs(M2)) // 2
        jmin = max(jmin, (abs(M2) + 1) // 2)
        for J in range(jmin, jmax + 1):
            c1 = cg(int(tj[a]), int(tj[b]), 2 * J, int(tm[a]), int(tm[b]), M2)
            if c1 == 0.0:
                continue
            c2 = cg(int(tj[c]), int(tj[d]), 2 * J, int(tm[c]), int(tm[d]), M2)
            if c2 == 0.0:
                continue
            for T in (0, 1):
                if abs(MT2) > 2 * T:
                    continue
                ph = (-1.0) ** (J + T)
                an_ab = math.sqrt(1 - dab * ph) / (1 + dab)
                an_cd = math.sqrt(1 - dcd * ph) / (1 + dcd)
                if an_ab <= 1e-15 or an_cd <= 1e-15:
                    continue
                c3 = cg(1, 1, 2 * T, int(tt[a]), int(tt[b]), MT2)
                c4 = cg(1, 1, 2 * T, int(tt[c]), int(tt[d]), MT2)
                v = _vjt_lookup(V, sp, oa, ob, oc, od, J, T)
                s += c1 * c2 * c3 * c4 * v / (an_ab * an_cd)
        out[e] = s
    return out


# ------------------------------------------------------------------ workloads
@dataclass
class Workload:
    name: str
    sp: ModelSpace
    mesh: Mesh
    e0: float
    t1b: np.ndarray
    recs: np.ndarray
    vbar: np.ndarray
    q2: np.ndarray
    vacua: list          # [(U, V)]
    deform: list         # [(beta2, gamma_deg)]
    pairs: list          # [(i, j)] symmetric pair list, i <= j

    @property
    def jops(self):
        return j_operators(self.sp)


SHELL_NUCLEONS = {"sd": (2, 2), "pf": (4, 4), "sdpf": (4, 4)}


def make_workload(shell, nvac, mesh: Mesh, seed, name=None, rot_scale=0.3, deformed=True,
                  nprot=None, nneut=None, pn_mix=False):
    """A seeded set of `nvac` vacua on one shell with all symmetric pairs i <= j
    (`pn_mix`: vacua that mix protons and neutrons, see the module docstring)."""
    rng = np.random.default_rng(seed)
    z, nn = SHELL_NUCLEONS.get(shell, (2, 2))
    sp = ModelSpace(SHELLS[shell], nprot if nprot is not None else z, nneut if nneut is not None else nn)
    no = len(sp.orbits)
    spe = rng.uniform(-4.0, 0.0, no)
    t1b = np.diag([spe[o] for o in sp.orbit]).astype(complex)
    recs = mscheme_pairs(sp)
    vbar = uncouple(sp, random_vjt(sp, rng), recs)
    q2 = q2_operators(sp)
    vacua, deform = [], []
    for k in range(nvac):
        b2 = rng.uniform(0.0, 0.5) if deformed else rng.uniform(0.0, 0.3)
        gd = rng.uniform(0.0, 60.0)
        vacua.append(deformed_vacuum(sp, spe, b2, gd, rng, rot_scale=rot_scale, q2=q2, pn_mix=pn_mix))
        deform.append((b2, gd))
    pairs = [(i, j) for i in range(nvac) for j in range(i, nvac)]
    return Workload(name or shell, sp, mesh, 0.0, t1b, recs, vbar, q2, vacua, deform, pairs)


def config(idx, small=False, pn_mix=None):
    """Benchmark configurations (mesh sizes as quoted; `small` shrinks the vacuum count).

    The sd case (0) is specified as random vacua with only time reversal and parity
    imposed, so its vacua mix protons and neutrons; the pf cases (1, 2) default to
    charge-conserving deformed vacua (the species-split path) and take `pn_mix=True`
    for the general path.
    """
    if idx == 0:
        return make_workload("sd", 2, Mesh(8, 16, 8, 7), seed=1000, name="sd-2vac-8x16x8-g7", deformed=False,
                             pn_mix=True if pn_mix is None else pn_mix)
    if idx in (1, 2):
        mix = bool(pn_mix)
        return make_workload("pf", 4 if small else 20, Mesh(10, 20, 10, 9), seed=2000,
                             name="pf-20vac-10x20x10-g9" + ("-pnmix" if mix else ""), pn_mix=mix)
    raise ValueError(f"unknown configuration {idx}")


def workload_from_arrays(name, orbits, nprot, nneut, e0, spe, vbar, U, V, mesh: Mesh, core=(0, 0), deform=None):
    """A workload from real inputs: a model space (orbit list), E0 and single-particle
    energies keyed as `formats.read_me1b` returns them, the m-scheme V list in the
    record order of `formats.mscheme_pairs`, and vacua U[k], V[k] (as `formats.read_wf`
    returns them)."""
    from .formats import onebody_matrix
    sp = ModelSpace([tuple(int(x) for x in o) for o in orbits], int(nprot), int(nneut), int(core[0]), int(core[1]))
    recs = mscheme_pairs(sp)
    vbar = np.asarray(vbar, dtype=np.float64)
    if vbar.shape != (len(recs),):
        raise ValueError(f"{len(vbar)} m-scheme values for {len(recs)} records")
    vacua = [(np.asarray(U[k], dtype=np.float64), np.asarray(V[k], dtype=np.float64)) for k in range(len(U))]
    pairs = [(i, j) for i in range(len(vacua)) for j in range(i, len(vacua))]
    return Workload(name, sp, mesh, float(e0), onebody_matrix(sp, spe), recs, vbar, q2_operators(sp), vacua,
                    list(deform) if deform is not None else [(0.0, 0.0)] * len(vacua), pairs)


def ti48_workload(mesh: Mesh, path=None):
    """The reference's own Ti48 / KB3G inputs (pf shell, Z = 2, N = 6 valence, eight HFB
    vacua beta2 = -0.3 ... 0.4 with proton-neutron pairing) from the committed fixture
    `tests/golden/reference_pins.npz` (built from the SCCM tree by
    tests/golden/make_reference_pins.py)."""
    import os
    if path is None:
        path = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                            "tests", "golden", "reference_pins.npz")
    d = np.load(path)
    spe = {tuple(int(x) for x in k): float(v) for k, v in zip(d["kb3g_spe_keys"], d["kb3g_spe_vals"])}
    betas = [float(b) for b in d["ti48_betas"]]
    return workload_from_arrays("ti48-kb3g", d["pf_orbits"], d["ti48_nprot"], d["ti48_nneut"], d["kb3g_e0"], spe,
                                d["kb3g_vbar"], d["ti48_U"], d["ti48_V"], mesh, core=(20, 20),
                                deform=[(b, 0.0) for b in betas])


def uneven_workloads(scale=1):
    """The uneven batch: 64 sd pairs (mesh 8x16x8, gauge 7x7), 128 pf pairs
    (10x20x10, 9x9) and 16 sd+pf cross-shell pairs (n = 64, 12x24x12, 11x11).

    Each part has its own seeded vacua and interaction; the pair lists are the
    first pairs (i <= j) of 11, 16 and 6 vacua. `scale` > 1 divides the pair
    counts (at least one pair per part) for smaller runs of the same mix.
    """
    parts = []
    for shell, nvac, npairs, mesh, seed in (("sd", 11, 64, Mesh(8, 16, 8, 7), 3000),
                                            ("pf", 16, 128, Mesh(10, 20, 10, 9), 3100),
                                            ("sdpf", 6, 16, Mesh(12, 24, 12, 11), 3200)):
        wl = make_workload(shell, nvac, mesh, seed=seed, name=f"uneven-{shell}")
        wl.pairs = wl.pairs[:max(1, npairs // scale)]
        parts.append(wl)
    return parts
