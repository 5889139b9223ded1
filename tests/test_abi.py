"""The C-ABI library loads and exports every symbol include/*.h declares (no GPU calls)."""
import ctypes
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    inc = os.path.join(ROOT, "include")
    txt = "".join(open(os.path.join(inc, f)).read() for f in sorted(os.listdir(inc)) if f.endswith(".h"))
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+(?:\s+\w+)?\s*\*?\s*(pnamp_\w+)\s*\(", txt, re.M)))


@pytest.fixture(scope="module")
def lib():
    from sccm_gb300.build import build
    path = build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    syms = declared_symbols()
    assert "pnamp_init" in syms and "pnamp_pair" in syms and "pnamp_project" in syms


def test_library_exports_declared_symbols(lib):
    for s in declared_symbols():
        assert hasattr(lib, s), s


def test_python_host_binds_every_export():
    from sccm_gb300.gcm import HW_EXPORTS
    from sccm_gb300.mlp import MLP_EXPORTS
    from sccm_gb300.pnamp import EXPORTS
    assert sorted(EXPORTS + MLP_EXPORTS + HW_EXPORTS) == declared_symbols()


def test_strerror_and_version(lib):
    lib.pnamp_strerror.restype = ctypes.c_char_p
    lib.pnamp_version.restype = ctypes.c_char_p
    assert b"singular" in lib.pnamp_strerror(4)
    assert b"sm_103a" in lib.pnamp_version()
