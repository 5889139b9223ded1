"""The tensor-core recast of the two-body energy, described on the host.

The energy loop of HFB_Energy_COMPLEX (Codes/PNAMP/PNAMP_Energy_OpenMP.f90:31-90), regrouped
exactly as the GPU's point kernel does, is two bilinear forms of the densities of a point:
a particle-hole form s^T Q s over the entries s = rho(r, c), and a particle-particle form
u^T C w over the antisymmetric pair vectors u = K01, w = K10 (i < j). Q is block-diagonal by
(m_r - m_c, t_r - t_c, parity) up to the negation that the transposed second factor brings,
C by (m_i + m_j, t_i + t_j, parity); blocks are packed into groups of at most 256 storage
entries (ph groups closed under label negation), each group one dense square GEMM block over
one contiguous storage range padded to 64 entries. The library builds the same groups in
C++ (pnamp_capi.cu::build_tc) for its tcgen05 kernel (contract_tc.cu); this module restates
them for the tests and for bench.py's flop count.
"""
from __future__ import annotations

import numpy as np


def contraction_groups(sp, recs=None, vbar=None, cap=256):
    """Storage position and group of every ph entry (r, c) and pp pair (i < j), the groups'
    (kind, offset, padded size), each group's dense square matrix (when `recs` and `vbar` are
    given; else None) and the row length; the packing of pnamp_capi.cu::build_tc."""
    n = sp.nlev
    m, t, l = sp.twom.astype(int), sp.t.astype(int), sp.l.astype(int)
    ph, pp = {}, {}
    for r in range(n):
        for c in range(n):
            ph.setdefault((m[r] - m[c], t[r] - t[c], (l[r] + l[c]) % 2), []).append((r, c))
    for i in range(n):
        for j in range(i + 1, n):
            pp.setdefault((m[i] + m[j], t[i] + t[j], (l[i] + l[j]) % 2), []).append((i, j))
    ph_units = []
    for L in sorted(ph):
        N = (-L[0], -L[1], L[2])
        if N < L and N in ph:
            continue
        ph_units.append([L] if N == L or N not in ph else [L, N])
    pp_units = [[L] for L in sorted(pp)]

    def pack(units, mem):
        order = sorted(range(len(units)), key=lambda u: -sum(len(mem[k]) for k in units[u]))
        groups, fill = [], []
        for u in order:
            sz = sum(len(mem[k]) for k in units[u])
            for g in range(len(groups)):
                if fill[g] + sz <= cap:
                    groups[g] += units[u]
                    fill[g] += sz
                    break
            else:
                groups.append(list(units[u]))
                fill.append(sz)
        return groups
    pos, grp, ranges = {}, {}, []
    off = 0
    for kind, groups, mem in (("ph", pack(ph_units, ph), ph), ("pp", pack(pp_units, pp), pp)):
        for g in groups:
            d = 0
            for L in g:
                for e in mem[L]:
                    pos[(kind, e)] = off + d
                    grp[(kind, e)] = len(ranges)
                    d += 1
            dpad = -(-d // 64) * 64
            ranges.append((kind, off, dpad))
            off += dpad
    if recs is None or vbar is None:
        return pos, ranges, None, off
    mats = [np.zeros((dp, dp)) for _, _, dp in ranges]

    def add(kind, e1, e2, v):
        g = grp[(kind, e1)]
        assert grp[(kind, e2)] == g
        o = ranges[g][1]
        mats[g][pos[(kind, e1)] - o, pos[(kind, e2)] - o] += v
    for (i, j, k, ll), V in zip(recs, vbar):
        d = 0.0 if i + j == k + ll else 1.0
        add("ph", (k, i), (ll, j), V)
        add("ph", (ll, i), (k, j), -V)
        if d:
            add("ph", (i, k), (j, ll), V)
            add("ph", (j, k), (i, ll), -V)
        add("pp", (i, j), (k, ll), V / 4)
        if d:
            add("pp", (k, ll), (i, j), V / 4)
    return pos, ranges, mats, off


def gemm_flops_per_point(sp):
    """Algorithmic flops of the group GEMMs for one kernel point, each product counted once:
    a real group matrix times the point's complex operand (two real rows), 2 x 2 x dpad^2 per
    group. The BF16x3 / BF16x6 forms execute three / six such products."""
    _, ranges, _, _ = contraction_groups(sp)
    return float(sum(4 * dp * dp for _, _, dp in ranges))
