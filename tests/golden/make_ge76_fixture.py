"""Build tests/golden/ge76_fixture.npz from the reference's shipped Ge76 data.

Run once with SCCM_REF set to the root of a jmyao17/SCCM checkout:

    SCCM_REF=/path/to/SCCM python tests/golden/make_ge76_fixture.py

The fixture carries everything the Ge76 parity tests need, so the tests never
read the reference tree at run time:

  * the pf5g9 valence space (Codes/val/pf5g9.val)
  * E0 and single-particle energies (Codes/int/GCN2850/SM_GCN2850_ME1B.dat)
  * the antisymmetrised m-scheme V list
    (Codes/int/GCN2850/IMSRG_s000_GCN2850pf5g9_hwHO10_m1m2m3m4.dat)
  * HFB vacua U, V for beta2 = -0.1, 0.0, 0.1, 0.2
    (data/Ge/Ge76_HFB_GCN2850_pf5g9_hwHO09_s000_beta*gam00np00cf000.wf)
  * the reference's kernel files for the 16 pairs among those four vacua
    (data/Ge/kern.1D.05.01.16.01.GCN2850_pf5g9_hwHO09_s000_*.elem):
    N^J, H^J, <N>, <Z>, <J^2> at J = 0, 2, 4, 6;
  * the reference's J = 0 one-body density files of the same pairs
    (data/Ge/Rho1B.Ge76.1D.05.01.16.01.pf5g9_hwHO09_s000_*.dens): per block
    (it, lj, n1, n2) the value Write_ME1B prints.

The beta2 = -0.2 vacuum is left out: no beta sign, pair order or quadrature
reproduces the shipped kernel files of its 9 pairs (errors 1e-4 to 1e-1 where
the other 16 pairs agree to 1e-8), so the shipped .wf is not the vacuum those
kernel files were computed from.

Run parameters of those kernel files: Z = 4, N = 16 valence, core 28 + 28,
NFOM = 5, N_alp = N_gam = 1, N_bet = 16 with the beta <-> pi - beta half range.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

from sccm_gb300.basis import ModelSpace  # noqa: E402
from sccm_gb300.formats import (mscheme_pairs, read_elem_axial, read_me1b,  # noqa: E402
                                read_mscheme_binary, read_rho1b_dens, read_val, read_wf)

REF = os.environ.get("SCCM_REF", "")
BETAS = (-10, 0, 10, 20)       # beta2 x 100


def wf_name(b):
    s = f"+{b:03d}" if b >= 0 else f"-{-b:03d}"
    return f"{REF}/data/Ge/Ge76_HFB_GCN2850_pf5g9_hwHO09_s000_beta{s}gam00np00cf000.wf"


def elem_name(b1, b2):
    f = lambda b: f"+{b * 100:05d}" if b >= 0 else f"-{-b * 100:05d}"
    return (f"{REF}/data/Ge/kern.1D.05.01.16.01.GCN2850_pf5g9_hwHO09_s000_"
            f"{f(b1)}.000cf000_{f(b2)}.000cf000.elem")


def rho1b_name(b1, b2):
    f = lambda b: f"+{b * 100:05d}" if b >= 0 else f"-{-b * 100:05d}"
    return (f"{REF}/data/Ge/Rho1B.Ge76.1D.05.01.16.01.pf5g9_hwHO09_s000_"
            f"{f(b1)}.000cf000_{f(b2)}.000cf000.dens")


def main(out=os.path.join(HERE, "ge76_fixture.npz")):
    if not REF or not os.path.isdir(REF):
        raise SystemExit("set SCCM_REF to the root of the SCCM reference tree")
    orbits = read_val(f"{REF}/Codes/val/pf5g9.val")
    sp = ModelSpace(orbits, 4, 16, 28, 28)
    e0, spe = read_me1b(f"{REF}/Codes/int/GCN2850/SM_GCN2850_ME1B.dat")
    recs = mscheme_pairs(sp)
    vbar = read_mscheme_binary(
        f"{REF}/Codes/int/GCN2850/IMSRG_s000_GCN2850pf5g9_hwHO10_m1m2m3m4.dat", len(recs))
    U = np.zeros((len(BETAS), sp.nlev, sp.nlev))
    V = np.zeros_like(U)
    for k, b in enumerate(BETAS):
        _, _, U[k], V[k] = read_wf(wf_name(b), sp.nlev)
    fields = ("njkk", "hjkk", "nn", "zz", "J2")
    gold = np.zeros((len(BETAS), len(BETAS), 4, len(fields)), complex)
    for i, b1 in enumerate(BETAS):
        for j, b2 in enumerate(BETAS):
            g = read_elem_axial(elem_name(b1, b2))
            for jj, J in enumerate((0, 2, 4, 6)):
                for f, name in enumerate(fields):
                    gold[i, j, jj, f] = g[J][name]
    dens = {(i, j): read_rho1b_dens(rho1b_name(b1, b2))
            for i, b1 in enumerate(BETAS) for j, b2 in enumerate(BETAS)}
    rho1b_keys = sorted({k for d in dens.values() for k in d})
    rho1b_gold = np.full((len(BETAS), len(BETAS), len(rho1b_keys)), np.nan)
    for (i, j), d in dens.items():
        for b, k in enumerate(rho1b_keys):
            if k in d:
                rho1b_gold[i, j, b] = d[k]
    spe_keys = np.array(sorted(spe), dtype=np.int32)
    spe_vals = np.array([spe[tuple(k)] for k in spe_keys])
    np.savez_compressed(out, orbits=np.array(orbits, dtype=np.int32), e0=e0,
                        spe_keys=spe_keys, spe_vals=spe_vals, vbar=vbar,
                        betas=np.array(BETAS) / 100.0, U=U, V=V, gold=gold,
                        fields=np.array(fields), jvals=np.array([0, 2, 4, 6]),
                        nprot=4, nneut=16, core=28, nfom=5, nbet=16, ncosbet=2,
                        rho1b_keys=np.array(rho1b_keys, dtype=np.int32), rho1b_gold=rho1b_gold)
    print(f"wrote {out}: {os.path.getsize(out)} bytes")


if __name__ == "__main__":
    main()
