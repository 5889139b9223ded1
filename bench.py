#!/usr/bin/env python3
"""Benchmark of the GB300 PNAMP kernel path: projected kernel points/s.

Workload (the configuration the metric is quoted on that fits one GPU): pf shell
(0f7/2, 1p3/2, 0f5/2, 1p1/2; n = 40 m-states), 4 + 4 valence nucleons, 20 seeded
quadrupole-deformed HFB vacua (beta2 in [0, 0.5], gamma in [0, 60] deg) giving 210
symmetric (q, q') pairs, Euler mesh 10 x 20 x 10 with 9 x 9 gauge points (162,000 kernel
points per pair), seeded random J-coupled isospin-symmetric TBMEs. A kernel point is one
(q, q', alpha, beta, gamma, phi_n, phi_p) evaluation. These vacua conserve charge, so the
kernels take their species-split path; beside the headline the same run times the general
path on the same set with proton-neutron mixing vacua, and the reference's own Ti48 / KB3G
vacua and interaction (proton-neutron pairing, general path) on the same mesh. One step =
`--pairs-per-step` pairs through setup, mesh loop (and, in the tensor-core forms, the
contraction) and J/K projection; steps walk round robin over the pair list. For N > 1
(torchrun), pairs are dealt to ranks as in the reference's MPI round robin (rank == ic mod
nprocs): weak scaling, no collective on the data path.

`value`: device-resident inputs (uploaded before timing), CUDA-event time of the steps on
the launching stream, L2 flushed (256 MiB write) before each step outside its events.
`e2e`: the same steps through the host-buffer C ABI (`pnamp_batch` + `pnamp_project`) from
pinned host memory, results read back. Per-kernel times for the rooflines come from the
library's own CUDA events around its launches (`pnamp_set_timing`). `--impl reference`: the
C++/OpenMP restatement of the reference's CPU path (oracle/cpu; the reference Fortran cannot
be compiled here), all host cores, bounded samples of the same steps' pairs.

Other workloads (their own JSON lines, not the headline): `--workload uneven` (three model
spaces and meshes in persistent launches and one CUDA graph), `--workload learned` (the
learned mode against the exact mixed form on a fine mesh), `--workload rho2b` (the pf set
with the two-body transition density).
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "projected kernel points/s on 1 GB300: learned+mixed vs plain FP64 at <=1 keV E_J"
WORKLOAD = ("pf shell n=40 (Z=4, N=4 valence), 20 seeded deformed charge-conserving vacua -> 210 pairs, "
            "Euler 10x20x10 x gauge 9x9 = 162000 points/pair (species-split path)")
FORM_TEXT = {"fp64": "plain FP64",
             "df64": "mixed: per-point algebra in double-float (FP32 pairs) on the FP32 pipes, FP64 "
                     "preparation and reductions",
             "tc3": "mixed, with the two-body contraction as block GEMMs on the tcgen05 tensor cores in "
                    "BF16x3 (two bf16 terms per value, three products, FP32 accumulation)",
             "tc6": "mixed, with the two-body contraction as block GEMMs on the tcgen05 tensor cores in "
                    "BF16x6 (three bf16 terms per value, six products, FP32 accumulation)"}
FORMS = ("fp64", "df64", "tc3", "tc6")
# Double-float cost: a complex multiply-add (8 FP64-equivalent flops) is four double-float
# FMAs of 15 FP32 instructions each (pnamp_df64.cuh: one multiply, three FMAs, TwoSum's six
# additions, three additions, FastTwoSum's two), i.e. 7.5 FP32 instructions per flop.
FP32_INSTR_PER_FLOP = 7.5
# DRAM bytes per kernel point of the point kernels (ncu dram__bytes_read + write on launches of
# this workload, scaled by points): all per-point matrices live in shared memory or an
# L2-resident slot, so traffic is tiny.
# DRAM bytes per point (dram__bytes_read.sum + dram__bytes_write.sum of one ncu capture, divided
# by the points of the launch): FP64 point kernel (20,736-point case), double-float point
# kernel (20,736-point case: cold reads of the pair records and tables only), the
# tensor-core forms' point kernel (5,184-point case: the bf16 density rows it writes,
# 32 KB per point, which scale with the points) and the contraction kernel (5,184-point
# case: those rows read back, plus the L2-resident group matrices)
TRAFFIC_BYTES_PER_POINT = {"fp64": (553984.0 + 2560.0) / 20736.0, "df64": 43.0,
                           "tc_point": (0.664064e6 + 166.103552e6) / 5184.0,
                           "tc_contract": (212.85504e6 + 3.983616e6) / 5184.0}


def _pair_paths(wl, pairs):
    """(species-split, reduced Pfaffian) per pair, as the set-up kernel decides them: split
    when the four matrices have no proton-neutron blocks, reduced when V0's LU pivots span
    less than 1e2."""
    import scipy.linalg as sl
    n = wl.sp.nlev
    h = n // 2
    out = []
    for i, j in pairs:
        (U0, V0), (U1, V1) = wl.vacua[i], wl.vacua[j]
        split = all(not np.any(np.asarray(M)[:h, h:]) and not np.any(np.asarray(M)[h:, :h])
                    for M in (U0, V0, U1, V1))
        d = np.abs(np.diag(sl.lu_factor(V0)[0]))
        reduced = bool(d.min() >= 1e-2 * d.max())
        out.append((split and reduced, reduced))
    return out


def algorithmic_flops_per_point(wl, n_gauge, pairs=None, records=True):
    """Algorithmic FP64 work per kernel point of the point kernel, averaged over `pairs`
    (default: all): the minimal flops of the algorithm it runs (complex multiply-add = 8
    flops, complex x real = 4), O(n^2) terms left out.

    Per Euler point, amortised over the n_gauge gauge points: R W, R V1, conj(R) U1 and
    X = (R W) R^T with the block-diagonal rotation, (3 * 4 + 8) n sum_b d_b^2, and the
    four T22 partials (n x n x h, complex x real), 8 n^3.
    Per point: the Pfaffian of the n x n Schur complement c (D X D - Z0^-1), (4/3) n^3, or of
    the 2n x 2n matrix, (4/3) (2n)^3, when V0 is ill conditioned; Y T22^-1 for the 2n x n
    right-hand sides counted as LU + solves, (8/3 + 16) n^3; the density products, 12 n^3.
    For a species-split pair these run on two h x h blocks, h = n/2: a quarter.
    Two-body records (`records`; the tensor-core forms contract them in their own kernel):
    52 flops (28 when i + j = k + l, which halves the terms); for a split pair the proton-
    neutron records keep two of the four density products, 18 (10).
    """
    n = wl.sp.nlev
    h = n // 2
    sd2 = sum(d * d for _, d in wl.sp.blocks())
    r = np.asarray(wl.recs)
    i, j, k, l = r.T
    pn = (i < h) & (j >= h) & (k < h) & (l >= h)
    diag = (i + j) == (k + l)
    tot = 0.0
    paths = _pair_paths(wl, pairs if pairs is not None else wl.pairs)
    for split, reduced in paths:
        pfaff = (4.0 / 3.0) * (n if reduced else 2 * n) ** 3
        dense = (pfaff + (8.0 / 3.0 + 16.0 + 12.0) * n ** 3) * (0.25 if split else 1.0)
        if records:
            if split:
                rec = (52.0 * np.sum(~pn & ~diag) + 28.0 * np.sum(~pn & diag)
                       + 18.0 * np.sum(pn & ~diag) + 10.0 * np.sum(pn & diag))
            else:
                rec = 52.0 * np.sum(~diag) + 28.0 * np.sum(diag)
        else:
            rec = 0.0
        tot += (20.0 * n * sd2 + 8.0 * n ** 3) / n_gauge + dense + float(rec)
    return tot / len(paths)


SMI_FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")


# ------------------------------------------------------------------ CPU baseline
def cpu_rate(wl, pairs, n_euler_sample, form="minimal", threads=0, seed=0):
    """The C++/OpenMP restatement (oracle/cpu) on a sample of Euler points x all gauge points
    spread over `pairs`; returns (points/s, seconds, points)."""
    from oracle import cpu_baseline as cb
    rng = np.random.default_rng(seed)
    P = wl.mesh.n_euler
    per = max(1, n_euler_sample // len(pairs))
    t = 0.0
    pts = 0
    for (i, j) in pairs:
        idx = np.sort(rng.choice(P, size=min(per, P), replace=False))
        t0 = time.perf_counter()
        cb.zres(wl, wl.mesh, i, j, form, euler=idx, threads=threads)
        t += time.perf_counter() - t0
        pts += len(idx) * wl.mesh.n_gauge
    return pts / t, t, pts


def cpu_calibrated(wl, pairs, seconds, form="minimal", threads=0):
    """cpu_rate on a sample sized to take about `seconds`."""
    r0, t0, p0 = cpu_rate(wl, pairs, 4 * len(pairs), form, threads, seed=1)
    n = int(max(len(pairs), 4 * len(pairs) * seconds / max(t0, 1e-3)))
    return cpu_rate(wl, pairs, n, form, threads, seed=2)


# ------------------------------------------------------------------ clocks
def clock_path(args, tag):
    """nvidia-smi samples of one timed region: `--clock-dir` (default: the system temp dir)."""
    import tempfile
    d = args.clock_dir or tempfile.gettempdir()
    os.makedirs(d, exist_ok=True)
    return os.path.join(d, f"pnamp_clocks_{tag}_{os.getpid()}.csv")


class ClockSampler:
    def __init__(self, path):
        self.path = path
        self.proc = None

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={SMI_FIELDS}", "--format=csv",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self, device_index=0):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for ln in open(self.path).read().splitlines()[1:]:
            tok = [t.strip() for t in ln.split(",")]
            if len(tok) < 9 or not tok[0].isdigit() or int(tok[0]) != device_index:
                continue
            try:
                rows.append((float(tok[1].split()[0]), float(tok[2].split()[0]), tok[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for _, _, fl in rows for k in range(4) if fl[k].lower() == "active"})
        mx = max(r[1] for r in rows)
        loaded = [r[0] for r in rows if r[0] > 0.3 * mx] or [r[0] for r in rows]
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": mx, "reasons": reasons,
                "samples": len(rows)}


# ------------------------------------------------------------------ main
def gemm_peak_tflops(torch, dtype, size=4096):
    """cuBLAS GEMM size^3, best of 5, CUDA events: the pipe ceiling of `dtype` on this GPU
    (FP64 for the plain form, FP32 for the double-float form's instruction issue)."""
    a = torch.randn(size, size, dtype=dtype, device="cuda")
    b = torch.randn(size, size, dtype=dtype, device="cuda")
    for _ in range(2):
        a @ b
    best = 1e30
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        a @ b
        e.record()
        torch.cuda.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    return 2 * size ** 3 / best / 1e12


def measured_peaks():
    """MEASURED_PEAKS.json next to this file (HBM GB/s, bf16 TFLOP/s burst and sustained)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


UNEVEN_WORKLOAD = ("uneven batch: 64 sd pairs (n=24, Euler 8x16x8, gauge 7x7), 128 pf pairs (n=40, "
                   "10x20x10, 9x9), 16 sd+pf pairs (n=64, 12x24x12, 11x11)")


def learned_main(args):
    """`--workload learned`: learned + mixed against the exact mixed form on a fine-mesh pf set.

    The learned configuration: pf shell, `--learned-vacua` (40) seeded deformed vacua and
    all their symmetric pairs (820), fine mesh 16 x 32 x 16 Euler x 11 x 11 gauge (991,232
    points per pair), coarse 4 x 8 x 4; the network (4 x 256) is trained on
    `--learned-train` (200) pairs spread over the set. The learned run ends with the
    Hill-Wheeler gate (`LearnedPNAMP.run_gcm`). Reports both throughputs in fine-mesh
    points/s, the fraction of Euler points computed exactly, the gate's record, and the
    errors of the learned kernels against the exact ones (energy kernel in the basis of
    normalised states, per-vacuum E_J, lowest GCM levels) with the 1 keV gates' verdict.
    `--learned-ablation` adds the same method without the network.
    """
    import torch
    from sccm_gb300.basis import Mesh
    from sccm_gb300.learned import LearnedConfig, LearnedPNAMP, energy_errors_kev
    from sccm_gb300.synth import make_workload

    torch.cuda.set_device(0)
    wl = make_workload("pf", args.learned_vacua, Mesh(16, 32, 16, 11), seed=4000)
    nvac = len(wl.vacua)
    lm = LearnedPNAMP(wl, LearnedConfig(train_euler=256, epochs=30, seed=3, chunk=8))
    step = max(1, len(wl.pairs) // max(1, args.learned_train))
    train_pairs = wl.pairs[::step][:args.learned_train]
    pts = len(wl.pairs) * lm.P * lm.G

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = fn()
        torch.cuda.synchronize()
        return out, time.perf_counter() - t0

    # the learned mode's time includes its coarse precheck, its training and its gate
    (learned, gate), tl = timed(lambda: lm.run_gcm(wl.pairs, nvac, train_pairs=train_pairs))
    timing = dict(lm.last_timing)
    if gate["decision"].startswith("all pairs exact"):
        # the mode ran the plain quadrature itself after its precheck: that part is the exact
        # mixed form's time, and its kernels are the reference values
        exact, te = learned, gate["exact_s"]
    else:
        exact, te = timed(lambda: lm.exact(wl.pairs))
    err = energy_errors_kev(learned, exact, nvac=nvac, pairs=wl.pairs)
    out = {
        "metric": "projected kernel points/s, learned + mixed vs exact mixed (fine mesh)", "value": pts / tl,
        "unit": "points/s", "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": 1e3 * tl, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "df64+f32", "data": "synthetic: seeded vacua and TBMEs",
        "config": {"workload": f"pf n=40, {nvac} vacua ({len(wl.pairs)} pairs), Euler 16x32x16 x gauge "
                               f"11x11, coarse 4x8x4, network 4x256 trained on {len(train_pairs)} pairs"},
        "exact_mixed": {"value": pts / te, "seconds": te, "form": "df64"},
        "speed_vs_exact_mixed": te / tl,
        "exact_fraction": gate["exact_fraction"], "gate": gate,
        "fallback_pairs": gate["fallback_pairs"], "timing_s": timing, "training": gate.get("training"),
        "errors_keV": {k: v for k, v in err.items() if k != "per_pair_keV"},
        "gates_1keV": {"gcm_levels": err["gcm_levels_err_keV"] <= 1.0, "E_J": err["EJ_per_vacuum_err_keV"] <= 1.0}}
    if args.learned_ablation:
        if gate.get("training") is None:
            lm.train(train_pairs)
        base, tb = timed(lambda: lm.run(wl.pairs, use_net=False))
        out["without_network"] = {"value": pts / tb, "seconds": tb,
                                  "exact_fraction": sum(r["exact_euler"] for r in base) / (len(base) * lm.P)}
    print(json.dumps(out))
    lm.close()
    return 0


def uneven_main(args):
    """`--workload uneven`: the three-model-space batch in persistent launches.

    One step = one replay of the captured CUDA graph (per-context setup
    kernels, counter resets, the persistent point kernel of each group of
    contexts) over the whole batch, with the groups, shared-memory budgets and
    schedule the autotuner picked (timed on the batch divided by
    `--tune-scale`). Beside it: the same work as one `pnamp_batch_device`
    launch per model space on one stream.
    """
    import torch
    from sccm_gb300.synth import uneven_workloads
    from sccm_gb300.uneven import UnevenBatch, autotune, time_launches

    torch.cuda.set_device(0)
    wls = uneven_workloads(args.uneven_scale)
    ub = UnevenBatch(wls, form=args.form)
    probe = UnevenBatch(uneven_workloads(args.uneven_scale * args.tune_scale), form=args.form)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    tune = autotune(ub, probe=probe, cache=not args.no_tune_cache)
    probe.close()
    ub.capture()
    for _ in range(max(0, args.warmup - 1)):
        ub.replay()
    torch.cuda.synchronize()
    with ClockSampler(clock_path(args, "uneven")) as clk:
        g_ms, g_all = time_launches(ub.replay, args.steps, flush=flush.zero_)
    st = [s.cpu().numpy() for s in ub.status]
    if any((x & ~1).any() for x in st):
        raise RuntimeError("non-trivial point status flags in the uneven batch")

    def per_context():
        s = torch.cuda.current_stream().cuda_stream
        for c, np_, uv, z, stt in zip(ub.ctxs, ub.npairs, ub.uv, ub.zres, ub.status):
            c.batch_device(np_, uv.data_ptr(), z.data_ptr(), stt.data_ptr(), s)
    per_context()
    s_ms, _ = time_launches(per_context, max(1, min(args.steps, 2)), flush=flush.zero_)
    print(json.dumps({
        "metric": "projected kernel points/s, uneven batch in persistent launches (one CUDA graph)", "value": ub.points / (g_ms / 1e3),
        "unit": "points/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": g_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "df64" if args.form == "df64" else "f64", "data": "synthetic: seeded vacua and TBMEs",
        "config": {"workload": UNEVEN_WORKLOAD if args.uneven_scale == 1 else
                   UNEVEN_WORKLOAD + f", pair counts / {args.uneven_scale}",
                   "points": ub.points, "items": ub.nitems, "form": FORM_TEXT[args.form],
                   "l2": "flushed (256 MiB write) before each step"},
        "step_ms": g_all, "tuning": {"schedule": tune["schedule"], "groups": tune["groups"],
                                     "smem_budgets": tune["budgets"],
                                     "smem_bytes": [p.smem_bytes for p in ub.plans], "cached": tune["cached"],
                                     "probe_ms": tune.get("ms")},
        "per_context_launches": {"value": ub.points / (s_ms / 1e3), "ms_per_step": s_ms},
        "clocks": clk.summary(0), "gpu_launches": len(ub.ctxs) + len(ub.plans)}))
    ub.close()
    return 0


def rho2b_main(args):
    """`--workload rho2b`: the pf workload with the two-body transition density on.

    One step = setup + the point kernel with the per-quadruple Rho2B sums
    (`pnamp_batch_rho2b_device`) over `--pairs-per-step` pairs; beside it the same
    pairs without densities (`pnamp_batch_device`). Roofline of the Rho2B pass: per
    point and quadruple one complex product difference, one complex multiply-add
    and the norm-weighted FP64 accumulation, 30 flops, and a 16-byte read and write
    of the CTA's accumulator (L2-resident); the kernel is timed whole.
    """
    import torch
    from sccm_gb300.pnamp import PnampContext
    from sccm_gb300.synth import config
    from sccm_gb300.uneven import time_launches

    torch.cuda.set_device(0)
    wl = config(1)
    pps = args.pairs_per_step
    ctx = PnampContext(wl.sp, wl.e0, wl.t1b, wl.recs, wl.vbar, wl.mesh, q2=wl.q2, form=args.form)
    nq = ctx.rho2b_tables()["quads"].shape[0]
    dev = torch.device("cuda")
    uv = torch.from_numpy(ctx.pack_pairs([(*wl.vacua[i], *wl.vacua[j]) for i, j in wl.pairs[:pps]])).to(dev)
    z = torch.zeros((pps, 19, ctx.n_euler, 2), dtype=torch.float64, device=dev)
    st = torch.zeros((pps, ctx.n_euler), dtype=torch.int32, device=dev)
    r2 = torch.zeros((pps, nq, 2), dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    s = torch.cuda.current_stream().cuda_stream

    def dens():
        ctx.batch_rho2b_device(pps, uv.data_ptr(), z.data_ptr(), st.data_ptr(), r2.data_ptr(), s)

    def plain():
        ctx.batch_device(pps, uv.data_ptr(), z.data_ptr(), st.data_ptr(), s)

    for _ in range(args.warmup):
        dens()
        plain()
    torch.cuda.synchronize()
    with ClockSampler(clock_path(args, "rho2b")) as clk:
        d_ms, d_all = time_launches(dens, args.steps, flush=flush.zero_)
    p_ms, _ = time_launches(plain, args.steps, flush=flush.zero_)
    pts = pps * ctx.n_euler * wl.mesh.n_gauge
    extra_s = (d_ms - p_ms) / 1e3
    print(json.dumps({
        "metric": "projected kernel points/s with the two-body transition density (Rho2B)",
        "value": pts / (d_ms / 1e3), "unit": "points/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": d_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "df64" if args.form == "df64" else "f64",
        "data": "synthetic: seeded vacua and TBMEs",
        "config": {"workload": WORKLOAD, "pairs_per_step": pps, "quadruples": nq, "form": FORM_TEXT[args.form],
                   "l2": "flushed (256 MiB write) before each step"},
        "step_ms": d_all, "without_densities": {"value": pts / (p_ms / 1e3), "ms_per_step": p_ms},
        "rho2b_pass": {"flops_per_point": 30.0 * nq, "extra_ms_per_step": d_ms - p_ms,
                       "tflops_of_extra_time": 30.0 * nq * pts / extra_s / 1e12 if extra_s > 0 else None,
                       "accumulator_bytes_per_point": 32.0 * nq},
        "clocks": clk.summary(0), "gpu_launches": 2}))
    ctx.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--pairs-per-step", type=int, default=4)
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target length of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--form", default="tc6", choices=list(FORMS),
                    help="headline arithmetic form: plain FP64, double-float, or double-float with the "
                         "two-body contraction on the tensor cores (BF16x3, BF16x6)")
    ap.add_argument("--compare-forms", default=None,
                    help="comma-separated forms timed beside the headline on the same pairs (default: all)")
    ap.add_argument("--no-general", action="store_true",
                    help="skip the general-path workloads (pn-mixing vacua, Ti48/KB3G)")
    ap.add_argument("--secondary-steps", type=int, default=3, help="timed steps of the general-path workloads")
    ap.add_argument("--pn-mix", action="store_true",
                    help="headline workload with proton-neutron mixing vacua (the general path), e.g. for profiles")
    ap.add_argument("--mesh", default=None,
                    help="override the mesh as NALP,NBET,NGAM,NFOM (small cases for profiling captures)")
    ap.add_argument("--workload", default="pf", choices=["pf", "uneven", "learned", "rho2b"],
                    help="pf: the 210-pair pf-shell set (headline); uneven: three model spaces in one launch; "
                         "learned: learned + mixed against exact mixed on a fine mesh; rho2b: the pf set with "
                         "the two-body transition density")
    ap.add_argument("--learned-vacua", type=int, default=40)
    ap.add_argument("--learned-train", type=int, default=200)
    ap.add_argument("--learned-ablation", action="store_true",
                    help="learned workload: also time the method without the network")
    ap.add_argument("--uneven-scale", type=int, default=1, help="divide the uneven batch's pair counts")
    ap.add_argument("--tune-scale", type=int, default=16,
                    help="the autotuner times schedules on the uneven batch divided by this")
    ap.add_argument("--no-tune-cache", action="store_true")
    ap.add_argument("--clock-dir", default=None,
                    help="directory for the nvidia-smi clock samples of the timed regions (default: temp dir)")
    args = ap.parse_args()
    if args.workload == "uneven":
        return uneven_main(args)
    if args.workload == "learned":
        return learned_main(args)
    if args.workload == "rho2b":
        return rho2b_main(args)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    ncores = len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()

    from sccm_gb300.basis import Mesh
    from sccm_gb300.driver import rank_pairs
    from sccm_gb300.synth import config, ti48_workload
    wl = config(1, pn_mix=args.pn_mix)
    if args.mesh:
        wl.mesh = Mesh(*[int(x) for x in args.mesh.split(",")])
    pps = args.pairs_per_step
    mine = rank_pairs(wl.pairs, rank, world)
    order = [mine[k % len(mine)] for k in range((args.warmup + args.steps) * pps)]
    workload = WORKLOAD if not args.pn_mix else WORKLOAD.replace(
        "seeded deformed charge-conserving vacua", "seeded deformed vacua mixing protons and neutrons").replace(
        "(species-split path)", "(general path)")
    if args.mesh:
        workload += f", mesh overridden to {args.mesh}"
    line_config = {"workload": workload, "form": FORM_TEXT[args.form], "pairs_per_step": pps,
                   "points_per_pair": wl.mesh.n_euler * wl.mesh.n_gauge,
                   "l2": "flushed (256 MiB write) before each step",
                   "parallelism": f"pairs round-robin over {world} rank(s)"}

    if args.impl == "reference":
        if rank != 0:
            return 0
        # the C++/OpenMP CPU restatement on every host core, each step a bounded sample of
        # Euler points (all gauge points) of that step's pairs
        from oracle import cpu_baseline as cb
        cb.build()
        nth = cb.max_threads()
        first = order[:pps]
        _, t0, _ = cpu_rate(wl, first, 2 * pps)
        per_step = int(max(pps, 2 * pps * args.cpu_seconds / 5.0 / max(t0, 1e-3)))
        for k in range(args.warmup):
            cpu_rate(wl, order[k * pps:(k + 1) * pps], pps, seed=k)
        tot_t = tot_p = 0.0
        for k in range(args.steps):
            r, t, p = cpu_rate(wl, order[(args.warmup + k) * pps:(args.warmup + k + 1) * pps], per_step,
                               seed=100 + k)
            tot_t += t
            tot_p += p
        v = tot_p / tot_t
        sample = (f"{per_step} Euler points x {wl.mesh.n_gauge} gauge points per step, spread over the step's "
                  f"{pps} pairs; oracle/cpu/pnamp_cpu.cpp, minimal form, {nth} OpenMP threads")
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": v, "unit": "points/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: seeded vacua and TBMEs (no public dataset exists)", "config": line_config,
            "cpu_baseline": {"value": v, "unit": "points/s", "cores": nth, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "points/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return 0

    import torch
    from sccm_gb300.contraction import gemm_flops_per_point
    from sccm_gb300.pnamp import PnampContext

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    fs = 5 * 7 * 13 * 13 * 2
    with torch.cuda.stream(stream):
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def timed_forms(w, ctx, pair_order, forms, steps, warmup, tag):
        """W untimed + K timed steps per form on device-resident inputs; per form: total s,
        stage ms (library events), clocks, status."""
        P = ctx.n_euler
        packed = PnampContext.pack_pairs([(*w.vacua[i], *w.vacua[j]) for (i, j) in pair_order])
        per_pair_uv = packed[0].nbytes
        with torch.cuda.stream(stream):
            d_uv = torch.from_numpy(packed).to(dev)
            d_z = torch.zeros((pps, 19 * P * 2), dtype=torch.float64, device=dev)
            d_st = torch.zeros((pps, P), dtype=torch.int32, device=dev)
            d_proj = torch.zeros((pps, fs), dtype=torch.float64, device=dev)

        def step(k, ev=None):
            off = d_uv.data_ptr() + k * pps * per_pair_uv
            if ev:
                ev[0].record(stream)
            ctx.batch_device(pps, off, d_z.data_ptr(), d_st.data_ptr(), sh)
            ctx.project_device(pps, d_z.data_ptr(), d_proj.data_ptr(), True, sh)
            if ev:
                ev[1].record(stream)

        out = {}
        for form in forms:
            ctx.set_form(form)
            ctx.set_timing(False)
            with torch.cuda.stream(stream):
                for k in range(warmup):
                    flush.zero_()
                    step(k)
                torch.cuda.synchronize()
                if dist:
                    dist.barrier()
                evs = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(steps)]
                ctx.set_timing(True)
                with ClockSampler(clock_path(args, f"{tag}_{form}_rank{rank}")) as clk:
                    torch.cuda.synchronize()
                    for k in range(steps):
                        flush.zero_()
                        step(warmup + k, evs[k])
                    torch.cuda.synchronize()
                if dist:
                    dist.barrier()
            stages = ctx.stage_times()
            ctx.set_timing(False)
            tot = sum(e[0].elapsed_time(e[1]) for e in evs) / 1e3
            if dist:
                t = torch.tensor([tot], device=dev)
                dist.all_reduce(t, op=dist.ReduceOp.MAX)
                tot = float(t)
            status = d_st.cpu().numpy()
            if (status & ~1).any():
                raise RuntimeError(f"non-trivial point status flags ({tag}, {form}): {np.unique(status)}")
            out[form] = {"total_s": tot, "ms_per_step": 1e3 * tot / steps,
                         "stage_ms_per_step": {k: v / steps for k, v in stages.items()},
                         "clocks": clk.summary(local_rank)}
        return out, packed

    # ---- the headline workload in every form
    forms = [args.form] + [f for f in (args.compare_forms.split(",") if args.compare_forms else FORMS)
                           if f and f != args.form]
    ctx = PnampContext(wl.sp, wl.e0, wl.t1b, wl.recs, wl.vbar, wl.mesh, q2=wl.q2)
    P, G = ctx.n_euler, wl.mesh.n_gauge
    res, packed = timed_forms(wl, ctx, order, forms, args.steps, args.warmup, "pf")
    pts_step = pps * P * G
    points = args.steps * pts_step * world
    head = res[args.form]
    value = points / head["total_s"]

    # ---- e2e through the host-buffer C ABI, pinned host memory
    e2e = None
    if not args.no_e2e:
        ctx.set_form(args.form)
        pin = torch.empty(packed.shape, dtype=torch.float64).pin_memory().numpy()
        pin[...] = packed
        per_pair_uv = packed[0].nbytes
        h2d = pps * per_pair_uv
        d2h = pps * 19 * P * 16 + pps * P * 4 + pps * fs * 8
        for k in range(min(args.warmup, 1)):
            ctx.batch(pin[k * pps:(k + 1) * pps])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for k in range(args.steps):
            z, st = ctx.batch(pin[(args.warmup + k) * pps:(args.warmup + k + 1) * pps])
            for q in range(pps):
                ctx.project(z[q])
        torch.cuda.synchronize()
        te = time.perf_counter() - t0
        if dist:
            t = torch.tensor([te], device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            te = float(t)
        e2e = {"value": points / te, "unit": "points/s", "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h)}
    ctx.close()

    # ---- the general path: the same set with proton-neutron mixing vacua, and the reference's
    # own Ti48 / KB3G vacua and interaction, on the same mesh
    secondary = {}
    if not args.no_general:
        steps2 = max(1, min(args.steps, args.secondary_steps))
        for tag, w2, forms2 in (("pf_pnmix", config(1, pn_mix=True), [f for f in FORMS]),
                                ("ti48_kb3g", ti48_workload(wl.mesh), ["df64", args.form]
                                 if args.form != "df64" else ["df64", "fp64"])):
            if args.mesh:
                w2.mesh = wl.mesh
            mine2 = rank_pairs(w2.pairs, rank, world)
            order2 = [mine2[k % len(mine2)] for k in range((1 + steps2) * pps)]
            c2 = PnampContext(w2.sp, w2.e0, w2.t1b, w2.recs, w2.vbar, w2.mesh, q2=w2.q2)
            r2, _ = timed_forms(w2, c2, order2, list(dict.fromkeys(forms2)), steps2, 1, tag)
            c2.close()
            pts2 = steps2 * pps * w2.mesh.n_euler * w2.mesh.n_gauge * world
            paths = _pair_paths(w2, order2[pps:])
            secondary[tag] = {
                "workload": ("pf shell n=40, 20 seeded deformed vacua mixing protons and neutrons, same mesh "
                             "(general path)" if tag == "pf_pnmix" else
                             "Ti48 / KB3G (pf shell, Z=2, N=6 valence), the reference's 8 HFB vacua with "
                             "proton-neutron pairing and its m-scheme interaction file, same mesh (general path)"),
                "pairs_timed": len(order2) - pps, "species_split_pairs": sum(a for a, _ in paths),
                "reduced_pfaffian_pairs": sum(b for _, b in paths),
                "forms": {f: {"value": pts2 / v["total_s"], "ms_per_step": v["ms_per_step"],
                              "stage_ms_per_step": v["stage_ms_per_step"]} for f, v in r2.items()}}

    # ---- rooflines from the library's per-launch events over the timed steps
    timed_pairs = order[args.warmup * pps:]
    peaks = measured_peaks()
    tf64 = gemm_peak_tflops(torch, torch.float64) if rank == 0 else None
    tf32 = gemm_peak_tflops(torch, torch.float32, 8192) if rank == 0 else None
    rl = {}
    for form, v in res.items():
        tc = form.startswith("tc")
        flops_pt = algorithmic_flops_per_point(wl, G, timed_pairs, records=not tc)
        t_pts = v["stage_ms_per_step"]["points"] / 1e3
        ach = flops_pt * pts_step / t_pts / 1e12
        if form == "fp64":
            rl[form] = {"kernel": "point_kernel<FP64>", "bound": "fp64", "flops_per_point": flops_pt,
                        "achieved": ach, "peak": tf64, "unit": "TFLOP/s", "frac": ach / tf64 if tf64 else None,
                        "peak_source": "cuBLAS DGEMM 4096^3 measured in this run",
                        "traffic": TRAFFIC_BYTES_PER_POINT["fp64"] * pts_step}
        else:
            fp32 = 2.0 * FP32_INSTR_PER_FLOP * ach   # FP32 flop rate of the double-float instructions
            rl[form] = {"kernel": "point_kernel<double-float>", "bound": "fp32", "flops_per_point": flops_pt,
                        "fp64_equivalent_tflops": ach, "achieved": fp32, "peak": tf32, "unit": "TFLOP/s",
                        "frac": fp32 / tf32 if tf32 else None,
                        "peak_source": "cuBLAS SGEMM 8192^3 measured in this run; achieved = FP64-equivalent "
                                       f"flops x {FP32_INSTR_PER_FLOP} FP32 instructions x 2 (FMA)",
                        "traffic": TRAFFIC_BYTES_PER_POINT["tc_point" if tc else "df64"] * pts_step}
        if tc:
            gf = gemm_flops_per_point(wl.sp)
            t_c = v["stage_ms_per_step"]["contract"] / 1e3
            bf = peaks.get("bf16_tflops_sustained")
            achc = gf * pts_step / t_c / 1e12 if t_c > 0 else None
            nprod = 3 if form == "tc3" else 6
            rl[form]["contraction"] = {
                "kernel": f"contract_kernel<{2 if form == 'tc3' else 3}> (tcgen05 kind::f16, TMA, TMEM)",
                "bound": "tensor", "flops_per_point": gf, "achieved": achc, "peak": bf, "unit": "TFLOP/s",
                "frac": achc / bf if achc and bf else None,
                "executed_tflops": achc * nprod if achc else None,
                "traffic": TRAFFIC_BYTES_PER_POINT["tc_contract"] * pts_step,
                "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (a kernel inside a long step)",
                "note": f"algorithmic = one product of the dense group GEMMs; {form} executes {nprod}"}

    cpu = None
    if not args.no_cpu_baseline and rank == 0 and world == 1:
        from oracle import cpu_baseline as cb
        cb.build()
        nth = cb.max_threads()
        sample_pairs = order[args.warmup * pps:args.warmup * pps + pps]
        r_all, t_all, p_all = cpu_calibrated(wl, sample_pairs, args.cpu_seconds)
        r_one, t_one, p_one = cpu_calibrated(wl, sample_pairs, args.cpu_seconds / 3, threads=1)
        r_imp, t_imp, p_imp = cpu_calibrated(wl, sample_pairs, args.cpu_seconds / 3, form="as_implemented")
        cpu = {"value": r_all, "unit": "points/s", "cores": nth, "kind": "port",
               "sample": f"{p_all} points (Euler points x all gauge points) of the first timed step's {pps} pairs, "
                         f"{t_all:.1f} s; oracle/cpu/pnamp_cpu.cpp minimal form on {nth} OpenMP threads",
               "one_core": {"value": r_one, "points": p_one, "seconds": t_one},
               "as_implemented": {"value": r_imp, "cores": nth, "points": p_imp, "seconds": t_imp,
                                  "note": "the reference's per-point ZGEMM / LU / 2n x 2n Pfaffian sequence"}}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "points/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp64": "f64", "df64": "df64", "tc3": "df64+bf16x3", "tc6": "df64+bf16x6"}[args.form],
            "data": "synthetic: seeded vacua and TBMEs (no public dataset exists)",
            "config": line_config,
            "roofline": dict(rl[args.form]),
            "forms": {f: {"value": points / v["total_s"], "ms_per_step": v["ms_per_step"],
                          "stage_ms_per_step": v["stage_ms_per_step"], "text": FORM_TEXT[f],
                          "roofline": rl[f], "clocks": v["clocks"]} for f, v in res.items()},
            "plain_fp64": ({"value": points / res["fp64"]["total_s"], "ms_per_step": res["fp64"]["ms_per_step"]}
                           if "fp64" in res else None),
            "general_path": secondary or None,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "clocks": head["clocks"],
            "gpu_launches": args.steps * (4 if args.form.startswith("tc") else 3),
        }
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
