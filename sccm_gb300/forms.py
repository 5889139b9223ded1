"""Error of an arithmetic form against the plain FP64 path, on a whole workload.

For every pair the GPU computes ZRES in both forms; this module reports the
relative error of the norm kernel N(Omega) and of the Hamiltonian kernel
H(Omega) (ZRES columns 1 and 7), projects both, solves Hill-Wheeler for every
even J (`gcm.gcm_levels`) and reports the largest difference of the lowest GCM
levels and of each vacuum's K-mixed E_J, in keV. The plain FP64 path is itself
pinned to the FP64 oracle at 1e-10 (tests/test_gpu_parity.py), so these are
the form's errors against the oracle up to that bound.

    python -m sccm_gb300.forms --workload pf --nvac 20 --mesh 10,20,10,9 --form df64,tc3,tc6 [--pn-mix]

Several forms are compared against one FP64 run; one JSON line per form.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from .basis import Mesh
from .gcm import compare_levels, gcm_levels
from .pnamp import PnampContext


def run_form(wl, form, batch=8):
    ctx = PnampContext(wl.sp, wl.e0, wl.t1b, wl.recs, wl.vbar, wl.mesh, q2=wl.q2, form=form)
    zs, kerns = [], []
    t0 = time.perf_counter()
    for s in range(0, len(wl.pairs), batch):
        chunk = wl.pairs[s:s + batch]
        z, _ = ctx.batch([(*wl.vacua[i], *wl.vacua[j]) for i, j in chunk])
        for k in range(len(chunk)):
            zs.append(z[k])
            kerns.append(ctx.project(z[k], chop=True))
    dt = time.perf_counter() - t0
    ctx.close()
    return zs, kerns, dt


def compare(wl, form, ref_form="fp64", batch=8, ref=None):
    za, ka, ta = ref if ref is not None else run_form(wl, ref_form, batch)
    zb, kb, tb = run_form(wl, form, batch)
    rel_n = max(float(np.abs(b[:, 0] - a[:, 0]).max() / np.abs(a[:, 0]).max()) for a, b in zip(za, zb))
    rel_h = max(float(np.abs(b[:, 6] - a[:, 6]).max() / np.abs(a[:, 6]).max()) for a, b in zip(za, zb))
    nvac = len(wl.vacua)
    la = gcm_levels(ka, wl.pairs, nvac)
    lb = gcm_levels(kb, wl.pairs, nvac)
    dl, dq = compare_levels(la, lb)
    return {"form": form, "ref_form": ref_form, "pairs": len(wl.pairs), "vacua": nvac,
            "mesh": [wl.mesh.nalp, wl.mesh.nbet, wl.mesh.ngam, wl.mesh.nfom],
            "max_rel_err_norm_kernel": rel_n, "max_rel_err_energy_kernel": rel_h,
            "max_abs_err_gcm_levels_keV": 1e3 * dl, "max_abs_err_EJ_per_vacuum_keV": 1e3 * dq,
            "ground_state_MeV": {str(J): float(la[J]["levels"][0]) for J in la if la[J]["levels"].size},
            "seconds": {ref_form: ta, form: tb}}


def main():
    from .synth import make_workload
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="pf")
    ap.add_argument("--nvac", type=int, default=20)
    ap.add_argument("--mesh", default="10,20,10,9")
    ap.add_argument("--seed", type=int, default=2000)
    ap.add_argument("--form", default="df64", help="comma-separated forms to compare with FP64")
    ap.add_argument("--pn-mix", action="store_true", help="vacua that mix protons and neutrons (general path)")
    args = ap.parse_args()
    wl = make_workload(args.workload, args.nvac, Mesh(*[int(x) for x in args.mesh.split(",")]), seed=args.seed,
                       pn_mix=args.pn_mix)
    ref = run_form(wl, "fp64")
    for form in args.form.split(","):
        r = compare(wl, form, ref=ref)
        r["pn_mix"] = bool(args.pn_mix)
        print(json.dumps(r), flush=True)


if __name__ == "__main__":
    main()
