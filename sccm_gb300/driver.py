"""Pair scheduling and kernel-file output: the host side of PNAMP_Main.

  * `pair_list`: the (q, q') list of Codes/PNAMP/PNAMP_Main.f90:60-73
    (ICons = 1: every q' in nq1i..nq1f; otherwise only q' >= q).
  * `rank_pairs`: the static round robin of PNAMP_Main.f90:79-84,
    `rank == mod(ic, nprocs)` with ic counted from 1. Pairs are independent,
    so ranks need no collective: each writes its own kernel files.
  * `run_pairs`: batches a rank's pairs through the GPU library, projects
    them and writes `kern.*.elem` files through a temporary name and rename
    (the kernel file is the checkpoint: a finished pair is never redone);
    a manifest lists finished pairs so an interrupted run resumes. With
    `rho1b`, each pair's J = 0 one-body density goes to `Rho1B_*.dens` as
    Write_ME1B writes it (PNAMP_Kernel3D.f90:719, PNAMP_Rho1B.f90:63-91);
    a pair whose projected norm is below CHOP gets no density file, as there.
    With `rho2b`, the two-body density goes to `Rho2B_*.dat` as Write_ME2B writes
    `Rho2B.dat` (PNAMP_Kernel3D.f90:722, PNAMP_Rho2B.f90:175-296), one file per
    pair instead of one overwritten name; both densities come from one pass.
"""
from __future__ import annotations

import json
import os

from .formats import atomic_write_text, empty_kernels, write_elem_general, write_rho1b_dens, write_rho2b_dat
from .pnamp import PNAMP_ERR_SMALL_NORM, PnampError
from .pnamp import PnampContext


def pair_list(nq0i, nq0f, nq1i, nq1f, icons=1):
    out = []
    for q1 in range(nq0i, nq0f + 1):
        start = nq1i if icons == 1 else q1
        for q2 in range(start, nq1f + 1):
            out.append((q1, q2))
    return out


def rank_pairs(pairs, rank, nprocs):
    """Pairs of this rank: ic = 1, 2, ... with rank == ic mod nprocs."""
    return [p for ic, p in enumerate(pairs, start=1) if ic % nprocs == rank]


def elem_name(prefix, q1, q2):
    return f"{prefix}_{q1:03d}_{q2:03d}.elem"


def rho1b_name(q1, q2):
    return f"Rho1B_{q1:03d}_{q2:03d}.dens"


def rho2b_name(q1, q2):
    return f"Rho2B_{q1:03d}_{q2:03d}.dat"


def run_pairs(ctx: PnampContext, vacua, pairs, out_dir, prefix="kern", coords=None, batch=8,
              manifest="manifest.json", rho1b=False, rho2b=False):
    """Compute and write the kernel files of `pairs` ((q1, q2) 1-based into `vacua`)."""
    os.makedirs(out_dir, exist_ok=True)
    mpath = os.path.join(out_dir, manifest)
    done = set()
    if os.path.exists(mpath):
        with open(mpath) as f:
            done = {tuple(x) for x in json.load(f).get("done", [])}
    todo = [p for p in pairs if tuple(p) not in done]
    for s in range(0, len(todo), batch):
        chunk = todo[s:s + batch]
        quads = [(*vacua[q1 - 1], *vacua[q2 - 1]) for (q1, q2) in chunk]
        if rho1b and rho2b:
            zres, status, r1, r2 = ctx.batch_densities(quads)
        elif rho1b:
            zres, status, r1 = ctx.batch_rho1b(quads)
        elif rho2b:
            zres, status, r2 = ctx.batch_rho2b(quads)
        else:
            zres, status = ctx.batch(quads)
        if rho1b:
            blocks = ctx.rho1b_blocks()
        if rho2b:
            blocks2 = ctx.rho2b_tables()["blocks"]
        for k, (q1, q2) in enumerate(chunk):
            if rho1b:
                try:
                    vals = ctx.project_rho1b(zres[k], r1[k])
                    atomic_write_text(os.path.join(out_dir, rho1b_name(q1, q2)), write_rho1b_dens, blocks, vals)
                except PnampError as e:
                    if e.code != PNAMP_ERR_SMALL_NORM:
                        raise
            if rho2b:
                try:
                    vals2 = ctx.project_rho2b(zres[k], r2[k])
                    atomic_write_text(os.path.join(out_dir, rho2b_name(q1, q2)), write_rho2b_dat, blocks2, vals2)
                except PnampError as e:
                    if e.code != PNAMP_ERR_SMALL_NORM:
                        raise
            kern = ctx.project(zres[k], chop=True)
            c1 = coords[q1 - 1] if coords is not None else (0.0, 0.0)
            c2 = coords[q2 - 1] if coords is not None else (0.0, 0.0)
            full = empty_kernels()
            full.update(kern)
            # the reference computes the exchanged element only for q1 != q2 (Kernel3D.f90:620,674)
            full["qpred"], full["qcpred"] = ctx.project_q(zres[k], exchange=(q1 != q2))
            atomic_write_text(os.path.join(out_dir, elem_name(prefix, q1, q2)), write_elem_general,
                              full, c1, c2)
            done.add((q1, q2))
        tmp = mpath + ".tmp"
        with open(tmp, "w") as f:
            json.dump({"done": sorted(done)}, f)
        os.replace(tmp, mpath)
    return sorted(done)
