"""The oracle against the reference's own Ge76 kernel files (data/Ge/kern.1D.*.elem).

Tolerance: the files print 8 significant digits; every field of the 16 pairs
whose vacua are shipped intact is reproduced to 2e-7 relative at J = 0..6,
except values whose magnitude is at the noise floor of the 16-point beta
quadrature (|N^J| < 1e-8 of the J=0 norm), which are skipped.
"""
import numpy as np
import pytest

from sccm_gb300.basis import JJMAX, Mesh
from oracle.pnamp_oracle import Hamiltonian, kernel_triaxial, project

PAIRS_CPU = [(1, 1), (1, 3), (0, 2), (3, 3)]   # indices into beta = (-0.1, 0, 0.1, 0.2)


@pytest.mark.parametrize("i,j", PAIRS_CPU)
def test_oracle_reproduces_ge76_kernel_files(ge76, i, j):
    g = ge76
    ham = Hamiltonian(g["e0"], g["t1b"].astype(complex), g["recs"], g["vbar"], g["q2"], g["jops"])
    mesh = Mesh(1, g["nbet"], 1, g["nfom"], ncosbet=g["ncosbet"])
    zres = kernel_triaxial(g["sp"], ham, mesh, g["U"][i], g["V"][i], g["U"][j], g["V"][j], iE2=False)
    k = project(zres, mesh, g["sp"].core_prot, g["sp"].core_neut, chop=0.0)
    gold = g["gold"][i, j]
    n0 = abs(gold[0, 0])
    for jj, J in enumerate(g["jvals"]):
        if abs(gold[jj, 0]) < 1e-8 * n0 * 1e2:
            continue
        for f, name in enumerate(("njkk", "hjkk", "nn", "zz", "J2")):
            mine = k[name][J, JJMAX, JJMAX].real
            ref = gold[jj, f].real
            assert abs(mine - ref) <= 2e-7 * abs(ref) + 1e-12, (J, name, mine, ref)


RHO1B_TOL = 2e-9   # the .dens files print 10 decimals


@pytest.mark.parametrize("i,j", [(1, 1), (0, 2), (2, 3)])
def test_oracle_reproduces_ge76_rho1b_files(ge76, i, j):
    """ZRho1B_Angles / ZRho1B_Integral / Write_ME1B against data/Ge/Rho1B.*.dens."""
    from oracle.pnamp_oracle import rho1b_table, rho1b_write_me1b
    g = ge76
    ham = Hamiltonian(g["e0"], g["t1b"].astype(complex), g["recs"], g["vbar"], g["q2"], g["jops"])
    mesh = Mesh(1, g["nbet"], 1, g["nfom"], ncosbet=g["ncosbet"])
    table = rho1b_table(g["sp"])
    assert [k[:4] for k, _ in table] == g["rho1b_keys"]
    zres, r = kernel_triaxial(g["sp"], ham, mesh, g["U"][i], g["V"][i], g["U"][j], g["V"][j], iE2=False,
                              rho1b=table)
    vals = rho1b_write_me1b(table, zres, r, mesh)
    assert np.abs(vals - g["rho1b_gold"][i, j]).max() <= RHO1B_TOL, (vals, g["rho1b_gold"][i, j])


def test_rho1b_dens_round_trip(tmp_path):
    from sccm_gb300.formats import read_rho1b_dens, write_rho1b_dens
    blocks = [(0, 1, 1, 1, 1), (0, 5, 0, 0, 5), (1, 8, 0, 0, 9)]
    vals = [0.9047578680, 1e-12, 0.0274656496]
    p = tmp_path / "x.dens"
    write_rho1b_dens(p, blocks, vals)
    got = read_rho1b_dens(p)
    assert set(got) == {(0, 1, 1, 1), (1, 8, 0, 0)}          # the 1e-12 entry is below CHOP
    assert abs(got[(0, 1, 1, 1)] - vals[0]) < 1e-10
