"""The C ABI from a plain C program (the way a Fortran bind(C) shim or a C++ harness binds
it): compiled with gcc against include/pnamp_gpu.h, linked to the built library, run
without a device on the host-only entry points."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_c_program_calls_the_host_entry_points(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    from sccm_gb300.build import build
    lib = build()
    exe = tmp_path / "abi_host"
    cmd = [gcc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "c", "abi_host.c"), "-o", str(exe), lib,
           "-Wl,-rpath," + os.path.dirname(lib)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stderr
    out = dict(line.split(" ", 1) for line in r.stdout.strip().splitlines())
    fields = out["nlev"].split()
    assert fields[0] == "40"
    vals = dict(zip(fields[1::2], fields[2::2]))
    assert vals == {"blocks": "22", "states": "120", "elements": "916", "quads": "29648", "terms": "76110"}
    assert "CHOP" in out["err"] or "norm" in out["err"].lower()
