"""ORACLE / CPU BASELINE -- test infrastructure only.

ctypes host of oracle/cpu/pnamp_cpu.cpp, the C++/OpenMP restatement of the PNAMP mesh loop
that bench.py times as the CPU baseline (its `--impl reference` arm and the `cpu_baseline`
key). The product path never imports this module.

    build()                      -> path of oracle/_build/libpnamp_cpu.so (g++ -O3 -fopenmp)
    zres(w, mesh, i, j, form, euler=None, threads=0) -> ZRES[P_E, NOBS] (rows outside `euler` 0)

form "as_implemented" follows the reference's per-point ZGEMM / LU sequence, form "minimal"
the GPU library's algebra (see the source file's header).
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "cpu", "pnamp_cpu.cpp")
LIB = os.path.join(HERE, "_build", "libpnamp_cpu.so")
FORMS = {"as_implemented": 0, "minimal": 1}
_lib = None


def build(force=False) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(
            os.path.getmtime(SRC), os.path.getmtime(os.path.join(ROOT, "include", "pnamp_gpu.h"))):
        return LIB
    gxx = shutil.which("g++") or shutil.which("c++")
    if gxx is None:
        raise RuntimeError("no C++ compiler for the CPU baseline")
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    tmp = f"{LIB}.tmp{os.getpid()}"
    cmd = [gxx, "-O3", "-std=c++17", "-fopenmp", "-fcx-limited-range", "-fPIC", "-shared",
           "-I", os.path.join(ROOT, "include"), SRC, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"CPU baseline build failed:\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


def load():
    global _lib
    if _lib is None:
        _lib = C.CDLL(build())
        vp = C.c_void_p
        _lib.cpu_pnamp_pair.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, C.c_int, C.c_int, C.c_int, vp]
        _lib.cpu_pnamp_pair.restype = C.c_int
        _lib.cpu_pnamp_max_threads.restype = C.c_int
    return _lib


def max_threads() -> int:
    return load().cpu_pnamp_max_threads()


def zres(w, mesh, i, j, form="minimal", euler=None, threads=0, cscale=1.0, iscale=0):
    """ZRES[P_E, NOBS] of pair (i, j) of workload `w` on `mesh`."""
    from sccm_gb300.pnamp import abi_structs
    lib = load()
    sp, ham, msh, keep = abi_structs(w.sp, w.e0, w.t1b, w.recs, w.vbar, mesh, w.q2, cscale, iscale)
    (U0, V0), (U1, V1) = w.vacua[i], w.vacua[j]
    mats = [np.asfortranarray(np.asarray(x, dtype=np.float64)) for x in (U0, V0, U1, V1)]
    P = mesh.n_euler
    out = np.zeros((19, P), dtype=np.complex128)
    idx = None if euler is None else np.ascontiguousarray(np.asarray(euler, dtype=np.int32))
    rc = lib.cpu_pnamp_pair(C.addressof(sp), C.addressof(ham), C.addressof(msh),
                            *[m.ctypes.data for m in mats],
                            idx.ctypes.data if idx is not None else None, 0 if idx is None else len(idx),
                            FORMS[form], int(threads), out.ctypes.data)
    del keep
    if rc != 0:
        raise RuntimeError(f"cpu_pnamp_pair returned {rc}")
    return np.ascontiguousarray(out.T)
