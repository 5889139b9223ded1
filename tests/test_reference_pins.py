"""Pins against files shipped in the reference tree (no GPU).

The fixture tests/golden/reference_pins.npz is made by
tests/golden/make_reference_pins.py from the SCCM tree:
  * every shipped Ge76 kernel file (post_axial layout, Codes/PNAMP/PNAMP_IO.f90:2-36)
    read and written back by the kernel-file writer must come out character for
    character;
  * the KB3G proton-neutron J-scheme interaction (Codes/int/KB3G/SM_KB3G_ME2B.dat)
    uncoupled to the m-scheme must reproduce the shipped m-scheme file
    IMSRG_s000_KB3Gpf_hwHO11_m1m2m3m4.dat record for record (to its 16 printed
    digits), which pins both the J -> m uncoupling (Codes/GCM/HFBA_Hamiltonian.f90:
    295-365 after Codes/PNAMP/IMSRG_GenerateH_JTMT.f90) and the record order;
  * the isospin uncoupling used for the synthetic interactions equals the proton-
    neutron one on the same interaction, so it is pinned through the same file.
"""
import os

import numpy as np
import pytest

from sccm_gb300.basis import JJMAX, SHELLS, ModelSpace
from sccm_gb300.formats import empty_kernels, mscheme_pairs, read_elem_axial, write_elem_axial
from sccm_gb300.interaction import isospin_to_pn, jscheme_table, uncouple_pn
from sccm_gb300.synth import random_vjt, uncouple

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def pins():
    return np.load(os.path.join(GOLDEN, "reference_pins.npz"))


def test_fixture_holds_every_shipped_kernel_file(pins):
    names = list(pins["elem_names"])
    assert len(names) == 26
    assert all(n.startswith("kern.1D.") and n.endswith(".elem") for n in names)
    # one shipped file (the 14-node beta mesh of the +0.2/+0.2 pair) is empty
    assert sum(len(str(t)) == 0 for t in pins["elem_texts"]) == 1


def test_post_axial_writer_reproduces_shipped_kernel_files(pins, tmp_path):
    checked = 0
    for name, text in zip(pins["elem_names"], pins["elem_texts"]):
        if not str(text):
            continue
        checked += 1
        src = tmp_path / "in.elem"
        src.write_text(str(text))
        parsed = read_elem_axial(src)
        kern = empty_kernels()
        coords = None
        for J, rec in parsed.items():
            for f in ("njkk", "hjkk", "nn", "zz", "J2", "q0p", "q0pc"):
                kern[f][J, JJMAX, JJMAX] = rec[f]
            for dj in range(3):
                kern["qpred"][J, dj, 8, 6] = rec["qpred"][dj]
                kern["qcpred"][J, dj, 8, 6] = rec["qcpred"][dj]
            coords = rec["coords"]
        out = tmp_path / "out.elem"
        Js = sorted(parsed)
        write_elem_axial(out, kern, tuple(coords[:2]), tuple(coords[2:4]), jmin=Js[0], jmax=Js[-1])
        got = out.read_text().splitlines()
        want = str(text).splitlines()
        assert len(got) == len(want), name
        for k, (g, w) in enumerate(zip(got, want)):
            assert g.rstrip() == w.rstrip(), f"{name} line {k + 1}: {g!r} != {w!r}"
    assert checked == 25


def test_kb3g_jscheme_uncouples_to_shipped_mscheme_file(pins):
    orbits = [tuple(int(x) for x in o) for o in pins["pf_orbits"]]
    sp = ModelSpace(orbits, 2, 6)
    recs = mscheme_pairs(sp)
    assert len(recs) == 14442
    records = [tuple(int(x) for x in r) + (float(m),) for r, m in zip(pins["kb3g_sm_int"], pins["kb3g_sm_me"])]
    v = uncouple_pn(sp, jscheme_table(orbits, records), recs)
    want = pins["kb3g_vbar"]
    err = np.abs(v - want).max()
    assert err <= 1e-10 * np.abs(want).max(), err
    # a wrong record order would pair values with the wrong quadruple
    assert np.count_nonzero(np.abs(want) > 1e-8) > 10000


@pytest.mark.parametrize("shell", ["sd", "pf"])
def test_isospin_uncoupling_matches_pn_uncoupling(shell):
    sp = ModelSpace(SHELLS[shell], 2, 2)
    rng = np.random.default_rng(11)
    vjt = random_vjt(sp, rng)
    recs = mscheme_pairs(sp)
    a = uncouple(sp, vjt, recs)
    b = uncouple_pn(sp, isospin_to_pn(sp, vjt), recs)
    assert np.abs(a - b).max() <= 1e-12 * np.abs(a).max()


def test_ti48_vacua_mix_protons_and_neutrons(pins):
    """The shipped Ti48 vacua have proton-neutron entries, so they take the general path."""
    U, V = pins["ti48_U"], pins["ti48_V"]
    h = U.shape[1] // 2
    for k in range(U.shape[0]):
        cross = max(np.abs(U[k][:h, h:]).max(), np.abs(U[k][h:, :h]).max(),
                    np.abs(V[k][:h, h:]).max(), np.abs(V[k][h:, :h]).max())
        assert cross > 1e-3
        # orthogonality of the Bogoliubov transformation (real U, V)
        assert np.abs(U[k].T @ U[k] + V[k].T @ V[k] - np.eye(2 * h)).max() < 1e-8
