"""ORACLE — test infrastructure only.

Runs `pnamp_oracle.kernel_triaxial` over chunks of Euler points in a process pool,
so the tests can check whole benchmark meshes (e.g. the sd case's 50,176 points)
in seconds. The pool uses the `spawn` start method: its workers never touch CUDA,
and a pool forked after the parent has initialised CUDA would hang.
"""
from __future__ import annotations

import multiprocessing as mp
import os

import numpy as np

from .pnamp_oracle import Hamiltonian, kernel_triaxial


def _chunk(args):
    sp, ham, mesh, U0, V0, U1, V1, idx, kw = args
    z = kernel_triaxial(sp, ham, mesh, U0, V0, U1, V1, euler_subset=idx, **kw)
    return idx, z[idx]


def zres_pool(w, mesh, i, j, euler_subset=None, procs=None, chunk=16, **kw):
    """Oracle ZRES [P_E, NOBS] of pair (i, j) of workload `w` on `mesh`; rows outside
    `euler_subset` stay zero."""
    ham = Hamiltonian(w.e0, w.t1b, w.recs, w.vbar, w.q2, w.jops)
    (U0, V0), (U1, V1) = w.vacua[i], w.vacua[j]
    idx = list(range(mesh.n_euler)) if euler_subset is None else [int(x) for x in euler_subset]
    procs = procs or max(1, min(len(os.sched_getaffinity(0)), 32))
    jobs = [(w.sp, ham, mesh, U0, V0, U1, V1, idx[k:k + chunk], kw) for k in range(0, len(idx), chunk)]
    out = np.zeros((mesh.n_euler, 19), complex)
    if procs == 1 or len(jobs) == 1:
        results = map(_chunk, jobs)
        for sub, rows in results:
            out[sub] = rows
        return out
    with mp.get_context("spawn").Pool(procs) as pool:
        for sub, rows in pool.imap_unordered(_chunk, jobs):
            out[sub] = rows
    return out
