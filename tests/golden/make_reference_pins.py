"""Build tests/golden/reference_pins.npz from files shipped in the SCCM reference tree.

Run once with SCCM_REF set to the root of a jmyao17/SCCM checkout:

    SCCM_REF=/path/to/SCCM python tests/golden/make_reference_pins.py

The fixture carries everything the pins below need, so the tests never read the
reference tree at run time:

  * kernel files: the text of every shipped `data/Ge/kern.1D.*.elem` (written by
    post_axial, Codes/PNAMP/PNAMP_IO.f90:2-36) -- pins the writer's layout;
  * KB3G interaction (pf shell, Codes/val/pf.val): the proton-neutron J-scheme
    records of Codes/int/KB3G/SM_KB3G_ME2B.dat, E0 and single-particle energies
    of SM_KB3G_ME1B.dat, and the m-scheme values of
    IMSRG_s000_KB3Gpf_hwHO11_m1m2m3m4.dat -- pins the J -> m uncoupling and the
    record order;
  * Ti48 HFB vacua: U, V of the eight shipped
    data/Ti/Ti48_HFB_KB3G_pf_hwHO11_s000_beta*gam00np00cf000.wf (n = 40, Z = 2,
    N = 6 valence). These carry proton-neutron pairing, so every pair among them
    runs the general (not species-split) path.
"""
import glob
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

from sccm_gb300.basis import ModelSpace  # noqa: E402
from sccm_gb300.formats import (mscheme_pairs, read_me1b, read_mscheme_binary, read_sm_me2b,  # noqa: E402
                                read_val, read_wf)

TI48_BETAS = (-30, -20, -10, 0, 10, 20, 30, 40)   # beta2 x 100


def main(out=os.path.join(HERE, "reference_pins.npz")):
    ref = os.environ.get("SCCM_REF")
    if not ref or not os.path.isdir(ref):
        raise SystemExit("set SCCM_REF to the root of the SCCM reference tree")
    elem_paths = sorted(glob.glob(os.path.join(ref, "data", "Ge", "kern.1D.*.elem")))
    elem_names = [os.path.basename(p) for p in elem_paths]
    elem_texts = [open(p).read() for p in elem_paths]

    orbits = read_val(os.path.join(ref, "Codes", "val", "pf.val"))
    sp = ModelSpace(orbits, 2, 6)
    kb = os.path.join(ref, "Codes", "int", "KB3G")
    sm = read_sm_me2b(os.path.join(kb, "SM_KB3G_ME2B.dat"))
    sm_int = np.array([r[:13] for r in sm], dtype=np.int32)
    sm_me = np.array([r[13] for r in sm])
    e0, spe = read_me1b(os.path.join(kb, "SM_KB3G_ME1B.dat"))
    spe_keys = np.array(sorted(spe), dtype=np.int32)
    spe_vals = np.array([spe[tuple(k)] for k in spe_keys])
    vbar = read_mscheme_binary(os.path.join(kb, "IMSRG_s000_KB3Gpf_hwHO11_m1m2m3m4.dat"), len(mscheme_pairs(sp)))

    U = np.zeros((len(TI48_BETAS), sp.nlev, sp.nlev))
    V = np.zeros_like(U)
    for k, b in enumerate(TI48_BETAS):
        s = f"+{b:03d}" if b >= 0 else f"-{-b:03d}"
        _, _, U[k], V[k] = read_wf(os.path.join(ref, "data", "Ti",
                                                f"Ti48_HFB_KB3G_pf_hwHO11_s000_beta{s}gam00np00cf000.wf"), sp.nlev)
    np.savez_compressed(out, elem_names=np.array(elem_names), elem_texts=np.array(elem_texts),
                        pf_orbits=np.array(orbits, dtype=np.int32), kb3g_sm_int=sm_int, kb3g_sm_me=sm_me,
                        kb3g_e0=e0, kb3g_spe_keys=spe_keys, kb3g_spe_vals=spe_vals, kb3g_vbar=vbar,
                        ti48_betas=np.array(TI48_BETAS) / 100.0, ti48_U=U, ti48_V=V, ti48_nprot=2, ti48_nneut=6)
    print(f"wrote {out}: {os.path.getsize(out)} bytes")


if __name__ == "__main__":
    main()
