"""SCCM file formats: round trips and the reference's failure cases (no GPU)."""
import os

import numpy as np
import pytest

from sccm_gb300.basis import SHELLS, ModelSpace
from sccm_gb300.formats import (FormatError, empty_kernels, mscheme_pairs, read_elem_general, read_mscheme_binary,
                                read_wf, write_elem_general, write_mscheme_binary, write_wf)


def test_mscheme_record_counts_match_shipped_interaction_files():
    # record counts of Codes/int/*/IMSRG_*_m1m2m3m4.dat: sd 2,570, pf 14,442, pf5g9 10,330
    for shell, want in (("sd", 2570), ("pf", 14442), ("pf5g9", 10330)):
        assert len(mscheme_pairs(ModelSpace(SHELLS[shell], 2, 2))) == want


def test_wf_round_trip_and_truncation(tmp_path):
    rng = np.random.default_rng(1)
    U, V = rng.standard_normal((2, 24, 24))
    p = tmp_path / "a.wf"
    write_wf(p, U, V)
    _, _, U2, V2 = read_wf(p, 24)
    assert np.array_equal(U, U2) and np.array_equal(V, V2)
    lines = open(p).read().splitlines()
    open(tmp_path / "b.wf", "w").write("\n".join(lines[:100]))
    with pytest.raises(FormatError):
        read_wf(tmp_path / "b.wf", 24)


def test_mscheme_binary_round_trip_and_corruption(tmp_path):
    v = np.random.default_rng(2).standard_normal(50)
    p = tmp_path / "v.dat"
    write_mscheme_binary(p, v)
    assert np.array_equal(read_mscheme_binary(p, 50), v)
    with pytest.raises(FormatError):
        read_mscheme_binary(p, 49)
    raw = bytearray(open(p, "rb").read())
    open(tmp_path / "t.dat", "wb").write(raw[:-3])
    with pytest.raises(FormatError):
        read_mscheme_binary(tmp_path / "t.dat")
    raw[0] = 7
    open(tmp_path / "m.dat", "wb").write(raw)
    with pytest.raises(FormatError):
        read_mscheme_binary(tmp_path / "m.dat")


def test_post_general_round_trip(tmp_path):
    rng = np.random.default_rng(3)
    k = empty_kernels()
    for f in k:
        k[f][...] = rng.standard_normal(k[f].shape) + 1j * rng.standard_normal(k[f].shape)
    p = tmp_path / "kern.elem"
    write_elem_general(p, k, (0.1, 20.0), (0.25, 30.0))
    r, coords = read_elem_general(p)
    assert coords[0] == [0.1, 20.0, 0.25, 30.0]
    for J in (0, 2, 3, 4, 5, 6):
        k2 = J if J % 2 == 0 else J - 1
        sl = slice(6 - k2, 6 + k2 + 1)
        for f in ("njkk", "hjkk", "nn", "zz", "J2", "q0p", "q0pc"):
            assert np.allclose(r[f][J, sl, sl], k[f][J, sl, sl], rtol=1e-7, atol=1e-7)
        for dj in range(3):
            s1 = slice(8 - k2 - dj, 8 + k2 + dj + 1)
            assert np.allclose(r["qpred"][J, dj, s1, sl], k["qpred"][J, dj, s1, sl], rtol=1e-7, atol=1e-7)
