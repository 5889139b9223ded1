"""Readers and writers for SCCM's PNAMP file formats.

PNAMP keeps its inputs and outputs, so the GCM stage and the shell drivers
consume this implementation's files unchanged:

  * `.val` valence space (Codes/PNAMP/PNAMP_Base.f90:29-60)
  * `.wf` HFB vacuum: `ide(0) ide(1)` then n^2 lines `U(i,j) V(i,j)`, i outer,
    j inner (reader Codes/PNAMP/PNAMP_Kernel3D.f90:88-122,
    writer Codes/HFB/HFBA_Main.f90:180-189)
  * one-body file: `E0`, then `t lj n1 n2 e` lines (Codes/GCM/HFBA_Hamiltonian1B.f90:28-35)
  * m-scheme two-body file: Fortran unformatted sequential, one real*8 per
    record (4-byte marker, 8-byte value, 4-byte marker). The record order is the
    m-scheme index list of `mscheme_pairs` (record counts: sd 2,570, pf 14,442,
    pf5g9 10,330 reproduce the shipped files' sizes exactly).
  * J-scheme shell-model two-body file `t1..t4, n1..n4, lj1..lj4, J, me`
    (Codes/PNAMP/IMSRG_GenerateH_JTMT.f90:108)
  * `betgam.dat` coordinates (Codes/PNAMP/PNAMP_IO.f90:98-128)
  * kernel files `kern.*.elem`: `post_axial` / `post_general`
    (Codes/PNAMP/PNAMP_IO.f90:2-96), format `(10i5)` / `(8e15.8)`.
"""
from __future__ import annotations

import math
import os
import struct

import numpy as np

from .basis import CHOP, JJMAX, ModelSpace


class FormatError(ValueError):
    """A malformed or truncated input file (the reference `stop`s here)."""


# --------------------------------------------------------------------------
def read_val(path):
    """Return the orbit list [(n0, l, twoj)] of a `.val` file (neutron block).

    Layout: 3 header lines, one line per orbit `nlj t n l twoj`, a separator
    line, then the same orbits for the other species (PNAMP_Base.f90:295-322).
    """
    with open(path) as f:
        lines = [ln for ln in f.read().splitlines()]
    body = lines[3:]
    orbits, second = [], []
    target = orbits
    for ln in body:
        tok = ln.split()
        if not tok:
            continue
        if not tok[0].lstrip('-').isdigit():
            target = second
            continue
        if len(tok) < 5:
            raise FormatError(f"{path}: bad orbit line {ln!r}")
        idx, _t, n0, l, tj = (int(v) for v in tok[:5])
        if idx != len(target) + 1:
            raise FormatError(f"{path}: orbit index {idx} out of order")
        target.append((n0, l, tj))
    if second and second != orbits:
        raise FormatError(f"{path}: proton and neutron orbit lists differ")
    if not orbits:
        raise FormatError(f"{path}: no orbits")
    return orbits


def read_wf(path, nlev):
    """Read a `.wf` vacuum; returns (ide0, ide1, U, V) with U, V as float64 [i, j]."""
    with open(path) as f:
        head = f.readline().split()
        if len(head) < 2:
            raise FormatError(f"{path}: missing ide header")
        ide = (int(head[0]), int(head[1]))
        data = np.array(f.read().split(), dtype=np.float64)
    want = 2 * nlev * nlev
    if data.size < want:
        raise FormatError(f"{path}: truncated ({data.size} of {want} values)")
    data = data[:want].reshape(nlev, nlev, 2)       # i outer, j inner
    return ide[0], ide[1], np.ascontiguousarray(data[:, :, 0]), np.ascontiguousarray(data[:, :, 1])


def write_wf(path, U, V, ide=(1, 1)):
    n = U.shape[0]
    with open(path, "w") as f:
        f.write(f"{ide[0]:12d}{ide[1]:12d}\n")
        for i in range(n):
            for j in range(n):
                f.write(f"{U[i, j]:25.16E}{V[i, j]:25.16E}\n")


# --------------------------------------------------------------------------
def read_me1b(path):
    """Return (E0, {(t, lj, n1, n2): e}) with t = 0 neutron, 1 proton."""
    with open(path) as f:
        lines = [ln for ln in f.read().splitlines() if ln.strip()]
    if not lines:
        raise FormatError(f"{path}: empty")
    e0 = float(lines[0].split()[0])
    spe = {}
    for ln in lines[1:]:
        tok = ln.split()
        if len(tok) < 5:
            raise FormatError(f"{path}: bad line {ln!r}")
        spe[(int(tok[0]), int(tok[1]), int(tok[2]), int(tok[3]))] = float(tok[4])
    return e0, spe


def onebody_matrix(sp: ModelSpace, spe):
    """Kinetic/single-particle matrix Esp(l,k) (Codes/GCM/HFBA_Hamiltonian1B.f90:45-62).

    The file's t = 0 is the neutron (m-scheme t = +1), t = 1 the proton (t = -1);
    n in the file counts from 0, the m-scheme n from 1.
    """
    n = sp.nlev
    h = np.zeros((n, n))
    tfile = {1: 0, -1: 1}
    for k in range(n):
        for l in range(n):
            if sp.t[k] != sp.t[l] or sp.lj[k] != sp.lj[l] or sp.twom[k] != sp.twom[l]:
                continue
            key = (tfile[int(sp.t[k])], int(sp.lj[k]), int(sp.n[l]) - 1, int(sp.n[k]) - 1)
            h[l, k] = spe.get(key, 0.0)
    return h


# --------------------------------------------------------------------------
def mscheme_pairs(sp: ModelSpace):
    """Index list (a, b, c, d), 0-based, of the stored antisymmetrised m-scheme V.

    a < b, c < d, a + b <= c + d (1-based sums, same ordering), with charge,
    M and parity conservation. Loop nesting a, b, c, d outermost to innermost.
    Both orders of (ab),(cd) are stored when a + b == c + d, which is why the
    energy loop drops the exchanged term there (PNAMP_Energy_OpenMP.f90:73-78).
    """
    n = sp.nlev
    t, m, l = sp.t.astype(int), sp.twom.astype(int), sp.l.astype(int)
    out = []
    for a in range(n):
        for b in range(a + 1, n):
            for c in range(n):
                for d in range(c + 1, n):
                    if a + b > c + d:
                        continue
                    if t[a] + t[b] != t[c] + t[d]:
                        continue
                    if m[a] + m[b] != m[c] + m[d]:
                        continue
                    if (l[a] + l[b] - l[c] - l[d]) % 2:
                        continue
                    out.append((a, b, c, d))
    return np.array(out, dtype=np.int32).reshape(-1, 4)


def read_mscheme_binary(path, nrec=None):
    """Read the Fortran-unformatted list of real*8 records (one value per record)."""
    raw = open(path, "rb").read()
    if len(raw) % 16:
        raise FormatError(f"{path}: size {len(raw)} is not a whole number of 16-byte records")
    arr = np.frombuffer(raw, dtype=np.uint8).reshape(-1, 16)
    lead = arr[:, :4].copy().view("<i4").ravel()
    tail = arr[:, 12:].copy().view("<i4").ravel()
    if not (np.all(lead == 8) and np.all(tail == 8)):
        raise FormatError(f"{path}: record markers are not 8")
    vals = arr[:, 4:12].copy().view("<f8").ravel()
    if nrec is not None and vals.size != nrec:
        raise FormatError(f"{path}: {vals.size} records, expected {nrec}")
    return vals


def write_mscheme_binary(path, values):
    with open(path, "wb") as f:
        for v in np.asarray(values, dtype=np.float64):
            f.write(struct.pack("<idi", 8, float(v), 8))


def read_sm_me2b(path):
    """J-scheme records: (t1..t4, n1..n4, lj1..lj4, J, me)."""
    recs = []
    with open(path) as f:
        for ln in f:
            tok = [x for x in ln.replace(",", " ").split() if x]
            if len(tok) < 14:
                continue
            ints = tuple(int(x) for x in tok[:13])
            recs.append(ints + (float(tok[13]),))
    return recs


# --------------------------------------------------------------------------
def read_betgam(path):
    """Return rows (beta2, gamma, P00, hw) of a `betgam.dat` (4 header lines, NQ)."""
    with open(path) as f:
        lines = f.read().splitlines()
    if len(lines) < 5:
        raise FormatError(f"{path}: truncated header")
    nq = int(lines[4].split()[0])
    rows = []
    for ln in lines[5:5 + nq]:
        tok = ln.split()
        rows.append(tuple(float(x) for x in tok[:4]))
    if len(rows) != nq:
        raise FormatError(f"{path}: {len(rows)} rows, header says {nq}")
    return rows


# --------------------------------------------------------------------------
def _e15(x: float) -> str:
    """Fortran `e15.8`: 0.xxxxxxxxE+yy in a 15-wide field."""
    if x == 0.0 or not np.isfinite(x):
        mant, ex = 0.0, 0
        if not np.isfinite(x):
            return f"{'NaN':>15s}"
    else:
        ex = int(np.floor(np.log10(abs(x)))) + 1
        mant = x / 10.0 ** ex
        if round(abs(mant), 8) >= 1.0:
            mant /= 10.0
            ex += 1
    s = f"{abs(mant):.8f}"[1:]   # ".xxxxxxxx"
    sign = "-" if x < 0 else ""
    body = f"{sign}0{s}E{'+' if ex >= 0 else '-'}{abs(ex):02d}"
    return f"{body:>15s}"


def _line(vals):
    out = []
    for v in vals:
        z = complex(v)
        out.append(_e15(z.real) + _e15(z.imag))
    return "".join(out)


def empty_kernels():
    """Zeroed kernel-file fields: [J][K1+6][K2+6] scalars, [J][dJ][K1+8][K2+6] quadrupole blocks."""
    sh = (JJMAX + 1, 2 * JJMAX + 1, 2 * JJMAX + 1)
    out = {k: np.zeros(sh, complex) for k in ("njkk", "hjkk", "nn", "zz", "J2", "q0p", "q0pc")}
    out["qpred"] = np.zeros((JJMAX + 1, 3, 17, 13), complex)
    out["qcpred"] = np.zeros_like(out["qpred"])
    return out


def write_elem_axial(path, kern, q1=(0.0, 0.0), q2=(0.0, 0.0), jmin=0, jmax=JJMAX, jstep=2):
    """`post_axial` layout (PNAMP_IO.f90:2-36); `kern` maps field -> array [J][K1][K2]."""
    with open(path, "w") as f:
        for J in range(jmin, jmax + 1, jstep):
            if J == 1:
                continue
            f.write(f"{J:5d}\n")
            f.write(_e15(q1[0]) + _e15(q1[1]) + _e15(q2[0]) + _e15(q2[1]) + "\n")
            f.write(f"{0:5d}{0:5d}\n")
            g = lambda k: kern[k][J, JJMAX, JJMAX]
            f.write(_line([g("njkk"), g("hjkk")]) + "\n")
            f.write(_line([g("nn"), g("zz")]) + "\n")
            f.write(_line([g("J2")]) + "\n")
            f.write(_line([g("q0p"), g("q0pc")]) + "\n")
            for dj in range(3):
                f.write(_line([kern["qpred"][J, dj, 8, 6], kern["qcpred"][J, dj, 8, 6]]) + "\n")


def write_elem_general(path, kern, q1=(0.0, 0.0), q2=(0.0, 0.0), jmin=0, jmax=JJMAX, jstep=1):
    """`post_general` layout (PNAMP_IO.f90:39-96): 5 records per (K1, K2)."""
    with open(path, "w") as f:
        for J in range(jmin, jmax + 1, jstep):
            if J == 1:
                continue
            f.write(f"{J:5d}\n")
            f.write(_e15(q1[0]) + _e15(q1[1]) + _e15(q2[0]) + _e15(q2[1]) + "\n")
            k2max = J if J % 2 == 0 else abs(J - 1)
            for k2 in range(-k2max, k2max + 1):
                for k1 in range(-k2max, k2max + 1):
                    g = lambda k: kern[k][J, k1 + JJMAX, k2 + JJMAX]
                    f.write(f"{k1:5d}{k2:5d}\n")
                    f.write(_line([g("njkk"), g("hjkk")]) + "\n")
                    f.write(_line([g("nn"), g("zz")]) + "\n")
                    f.write(_line([g("J2")]) + "\n")
                    f.write(_line([kern["qpred"][J, 0, k1 + 8, k2 + 6],
                                   kern["qcpred"][J, 0, k1 + 8, k2 + 6]]) + "\n")
                    f.write(_line([g("q0p"), g("q0pc")]) + "\n")
            for k2 in range(-k2max, k2max + 1):
                for k1 in range(-k2max - 1, k2max + 2):
                    f.write(_line([kern["qpred"][J, 1, k1 + 8, k2 + 6],
                                   kern["qcpred"][J, 1, k1 + 8, k2 + 6]]) + "\n")
                for k1 in range(-k2max - 2, k2max + 3):
                    f.write(_line([kern["qpred"][J, 2, k1 + 8, k2 + 6],
                                   kern["qcpred"][J, 2, k1 + 8, k2 + 6]]) + "\n")


def read_elem_general(path, jmin=0, jmax=JJMAX, jstep=1):
    """Parse a `post_general` file (the layout write_elem_general produces) into kernel fields."""
    with open(path) as f:
        lines = [ln.rstrip("\n") for ln in f if ln.strip()]

    def nums(s):
        return [float(s[k:k + 15]) for k in range(0, len(s) - 14, 15)]
    out = empty_kernels()
    coords = {}
    i = 0
    for J in range(jmin, jmax + 1, jstep):
        if J == 1:
            continue
        if int(lines[i].split()[0]) != J:
            raise FormatError(f"{path}: expected J = {J}")
        coords[J] = nums(lines[i + 1])
        i += 2
        k2max = J if J % 2 == 0 else abs(J - 1)
        for k2 in range(-k2max, k2max + 1):
            for k1 in range(-k2max, k2max + 1):
                kk = [int(x) for x in lines[i].split()]
                if kk != [k1, k2]:
                    raise FormatError(f"{path}: expected K1 K2 = {k1} {k2}")
                r = [nums(lines[i + 1 + q]) for q in range(5)]
                c = lambda v, q: complex(v[2 * q], v[2 * q + 1])
                ix = (J, k1 + JJMAX, k2 + JJMAX)
                out["njkk"][ix], out["hjkk"][ix] = c(r[0], 0), c(r[0], 1)
                out["nn"][ix], out["zz"][ix] = c(r[1], 0), c(r[1], 1)
                out["J2"][ix] = c(r[2], 0)
                out["qpred"][J, 0, k1 + 8, k2 + 6], out["qcpred"][J, 0, k1 + 8, k2 + 6] = c(r[3], 0), c(r[3], 1)
                out["q0p"][ix], out["q0pc"][ix] = c(r[4], 0), c(r[4], 1)
                i += 6
        for k2 in range(-k2max, k2max + 1):
            for dj, span in ((1, k2max + 1), (2, k2max + 2)):
                for k1 in range(-span, span + 1):
                    v = nums(lines[i])
                    out["qpred"][J, dj, k1 + 8, k2 + 6] = complex(v[0], v[1])
                    out["qcpred"][J, dj, k1 + 8, k2 + 6] = complex(v[2], v[3])
                    i += 1
    return out, coords


def read_elem_axial(path):
    """Parse a `post_axial` file into {J: dict(field -> complex)}."""
    with open(path) as f:
        lines = [ln.rstrip("\n") for ln in f if ln.strip()]
    out, i = {}, 0

    def nums(s):
        return [float(s[k:k + 15]) for k in range(0, len(s) - 14, 15)]
    while i < len(lines):
        J = int(lines[i].split()[0])
        coords = nums(lines[i + 1])
        rec = [nums(lines[i + 3 + k]) for k in range(7)]
        c = lambda v, k: complex(v[2 * k], v[2 * k + 1])
        out[J] = dict(coords=coords,
                      njkk=c(rec[0], 0), hjkk=c(rec[0], 1),
                      nn=c(rec[1], 0), zz=c(rec[1], 1),
                      J2=c(rec[2], 0),
                      q0p=c(rec[3], 0), q0pc=c(rec[3], 1),
                      qpred=[c(rec[4 + m], 0) for m in range(3)],
                      qcpred=[c(rec[4 + m], 1) for m in range(3)])
        i += 10
    return out


def atomic_write_text(path, writer, *args, **kw):
    """Write through a temporary file and rename: a kernel file is the checkpoint."""
    tmp = f"{path}.tmp{os.getpid()}"
    writer(tmp, *args, **kw)
    os.replace(tmp, path)


# ---------------------------------------------------------------- Rho1B density files
def write_rho1b_dens(path, blocks, values, chop=CHOP):
    """Write_ME1B (PNAMP_Rho1B.f90:63-91): one line '(4i5,f20.10)' it, lj, n1, n2, value per
    block whose AE = value * sqrt(2j + 1) exceeds CHOP. `blocks` are (it, lj, n1, n2, twoj)."""
    with open(path, "w") as f:
        for (it, lj, n1, n2, twoj), v in zip(blocks, values):
            if abs(v * math.sqrt(twoj + 1.0)) > chop:
                f.write(f"{it:5d}{lj:5d}{n1:5d}{n2:5d}{v:20.10f}\n")


def read_rho1b_dens(path):
    """A Write_ME1B file -> {(it, lj, n1, n2): value}."""
    out = {}
    with open(path) as f:
        for ln in f:
            tok = ln.split()
            if len(tok) == 5:
                out[tuple(int(x) for x in tok[:4])] = float(tok[4])
    return out


def write_rho2b_dat(path, blocks, values, chop=CHOP):
    """Write_ME2B's kernel-density file (PNAMP_Rho2B.f90:175-296), valence entries.

    `blocks` are (tt, PP, J, states) in block order and `values` the Rho2BN of every
    element (bm, a_ij, a_kl) in that order (complex or real). Layout: the header lines,
    'bMax=' (i6) with the last block index, one '(2i10)' line bm, aMax - 1 per block, a
    blank record pair, then per block '# block' (i6) ':' ' aMax=' (i6) and one '(2i10,f20.10)'
    line b_ij, b_kl, Re(Rho2BN) (indices from 0) per element with |Rho2BN| > CHOP,
    followed by a blank record pair."""
    vals = list(values)
    with open(path, "w") as f:
        f.write("*** 2b DME from GCM calculation ***\n")
        f.write("# basis (block, aMax)\n")
        f.write(f"bMax={len(blocks) - 1:6d}\n")
        for bm, (_tt, _pp, _j, st) in enumerate(blocks):
            f.write(f"{bm:10d}{len(st) - 1:10d}\n")
        f.write("\n\n")
        e = 0
        for bm, (_tt, _pp, _j, st) in enumerate(blocks):
            f.write(f"# block{bm:6d}: aMax={len(st) - 1:6d}\n")
            for a in range(len(st)):
                for b in range(len(st)):
                    v = vals[e]
                    e += 1
                    if abs(v) > chop:
                        f.write(f"{a:10d}{b:10d}{float(np.real(v)):20.10f}\n")
            f.write("\n\n")


def read_rho2b_dat(path):
    """A Write_ME2B file -> {(bm, b_ij, b_kl): value}."""
    out, bm = {}, -1
    with open(path) as f:
        for ln in f:
            if ln.startswith("# block"):
                bm = int(ln.split(":")[0].split()[-1])
                continue
            tok = ln.split()
            if bm >= 0 and len(tok) == 3:
                out[(bm, int(tok[0]), int(tok[1]))] = float(tok[2])
    return out
