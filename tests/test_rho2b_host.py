"""Two-body transition density (Rho2B) without a GPU: the library's two-particle block
tables against the oracle's restatement of ME2B_Base_Full and ZRho2B_Angles, the
oracle's trace identities, and the Write_ME2B file round trip."""
import numpy as np
import pytest

from sccm_gb300.basis import SHELLS, Mesh, ModelSpace
from sccm_gb300.synth import make_workload
from oracle.pnamp_oracle import (Hamiltonian, kernel_triaxial, rho2b_blocks, rho2b_terms,
                                 rho2b_write_me2b)


@pytest.fixture(scope="module")
def lib():
    from sccm_gb300.build import build
    build()


@pytest.mark.parametrize("shell", ["sd", "pf", "p2", "pf5g9"])
def test_library_tables_equal_oracle(lib, shell):
    from sccm_gb300.pnamp import rho2b_tables
    sp = ModelSpace(SHELLS[shell], 2, 2)
    r = rho2b_tables(sp)
    blocks = rho2b_blocks(sp)
    quads, terms = rho2b_terms(sp, blocks)
    assert r["blocks"] == blocks
    assert np.array_equal(r["quads"], quads)
    ptr = np.cumsum([0] + [len(el) for el in terms])
    assert np.array_equal(r["ptr"], ptr)
    assert np.array_equal(r["term_q"], [q for el in terms for q, _ in el])
    assert np.array_equal(r["term_c"], [c for el in terms for _, c in el])


def test_block_structure():
    """nn and pp keep id1 <= id2 and identical orbits only at even J; np keeps every
    ordered orbit pair; blocks ordered tt, PP, J (PNAMP_ME2B_Base.f90:128-205)."""
    sp = ModelSpace(SHELLS["sd"], 2, 2)
    blocks = rho2b_blocks(sp)
    keys = [(tt, pp, J) for tt, pp, J, _ in blocks]
    assert keys == sorted(keys)
    for tt, pp, J, st in blocks:
        assert len(set(st)) == len(st)
        for o1, o2 in st:
            assert (sp.orbits[o1][1] + sp.orbits[o2][1]) % 2 == pp
            assert abs(sp.orbits[o1][2] - sp.orbits[o2][2]) <= 2 * J <= sp.orbits[o1][2] + sp.orbits[o2][2]
            if tt != 1 and o1 == o2:
                assert J % 2 == 0
    np_pairs = {(o1, o2) for tt, _, _, st in blocks if tt == 1 for o1, o2 in st}
    assert np_pairs == {(a, b) for a in range(3) for b in range(3)}


def test_missing_orbit_rejected(lib):
    from sccm_gb300.pnamp import PnampError, rho2b_tables
    sp = ModelSpace(SHELLS["sd"], 2, 2)
    keep = sp.nlev // 2
    sp.n = sp.n.copy()
    sp.n[keep:keep + 6] = 3          # the neutron d5/2 becomes 2d5/2: not a proton orbit
    with pytest.raises(PnampError):
        rho2b_tables(sp)


def trace_by_species(blocks, vals):
    """Write_ME2B's traces: sum over diagonal elements of (2J + 1) Rho2BN x Metric, with
    Metric = (1 + (-1)^J)/2 for identical (t, n, lj) and 2 otherwise (PNAMP_Rho2B.f90:234-240)."""
    tr, e = {0: 0.0, 1: 0.0, 2: 0.0}, 0
    for tt, _pp, J, st in blocks:
        for a, (o1, o2) in enumerate(st):
            for b in range(len(st)):
                if a == b:
                    metric = (1 + (-1) ** J) / 2 if (o1 == o2 and tt != 1) else 2.0
                    tr[tt] += (2 * J + 1) * vals[e] * metric
                e += 1
    return tr


def test_oracle_traces_count_pairs():
    """For a number-projected state sum_ij <c+_i c+_j c_j c_i> = N (N - 1) per species and
    2 N Z across them: the traces Write_ME2B prints must come out at those values."""
    w = make_workload("sd", 2, Mesh(2, 4, 2, 7), seed=5)
    ham = Hamiltonian(w.e0, w.t1b, w.recs, w.vbar, w.q2, w.jops)
    blocks = rho2b_blocks(w.sp)
    quads, terms = rho2b_terms(w.sp, blocks)
    zres, a = kernel_triaxial(w.sp, ham, w.mesh, *w.vacua[0], *w.vacua[1], rho2b=quads)
    vals = rho2b_write_me2b(terms, zres, a, w.mesh)
    tr = trace_by_species(blocks, vals)
    Z, N = w.sp.nprot, w.sp.nneut
    assert abs(tr[0] - N * (N - 1)) < 1e-4
    assert abs(tr[2] - Z * (Z - 1)) < 1e-4
    assert abs(tr[1] - 2 * N * Z) < 1e-4


def test_rho2b_file_round_trip(tmp_path):
    from sccm_gb300.formats import read_rho2b_dat, write_rho2b_dat
    sp = ModelSpace(SHELLS["sd"], 2, 2)
    blocks = rho2b_blocks(sp)
    ne = sum(len(st) ** 2 for *_, st in blocks)
    rng = np.random.default_rng(3)
    vals = rng.normal(0.0, 0.1, ne) + 1j * rng.normal(0.0, 1e-3, ne)
    vals[::7] = 1e-9                                  # below CHOP: not written
    write_rho2b_dat(tmp_path / "Rho2B.dat", blocks, vals)
    got = read_rho2b_dat(tmp_path / "Rho2B.dat")
    e = 0
    for bm, (*_, st) in enumerate(blocks):
        for a in range(len(st)):
            for b in range(len(st)):
                if abs(vals[e]) > 1e-8:
                    assert abs(got[(bm, a, b)] - vals[e].real) <= 5e-11
                else:
                    assert (bm, a, b) not in got
                e += 1
    txt = (tmp_path / "Rho2B.dat").read_text().splitlines()
    assert txt[2] == f"bMax={len(blocks) - 1:6d}"
