"""Uneven batches in persistent launches, with an autotuner and a CUDA graph.

The reference computes one (q, q') pair at a time on each MPI rank, every
pair running its own Euler x gauge loop (Codes/PNAMP/PNAMP_Main.f90:79-115,
Codes/PNAMP/PNAMP_Kernel3D.f90:178-260). Here the pair batches of several
model spaces and meshes (each a `PnampContext`) become (context, pair, Euler
point) items of a persistent launch (`pnamp_multi_*` in the C ABI): CTAs take
items from a device counter, so small sd-shell pairs fill the gaps left by
large cross-shell ones and no launch tail is paid per model space.

All CTAs of one launch hold the same shared memory, and the rest of each SM's
256 KB serves as L1. Model spaces disagree on the best split: n = 24 and
n = 40 run fastest with every per-point array in shared memory, n = 64 (whose
Pfaffian matrix alone exceeds 227 KB) with everything in the global slot and
a large L1. So the contexts may be split into groups, one persistent launch
per group with its own shared-memory budget, launched one after another on
one stream (heaviest items first) and captured together into one CUDA graph.
Launching the groups on forked streams instead was measured slower on GB300:
kernels that run at the same time share the SMs' shared-memory carveout, so
the n = 64 items lost their L1 (8.27 s against 7.06 s for the same two
groups one after another).

`autotune` picks the grouping and budgets, then the schedule (work order x
items per grab), from CUDA-event timings on a probe batch, and caches the
choice on disk by the batch's signature.
"""
from __future__ import annotations

import json
import os
import statistics

import numpy as np
import torch

from .basis import NOBS
from .pnamp import MultiPlan, PnampContext, PnampError

ORDERS = {0: "as given", 1: "heaviest items first", 2: "round robin over contexts"}
DEFAULT_SCHEDULES = tuple((o, g, 0) for o in (0, 1, 2) for g in (1, 4))
# shared-memory budgets per CTA (bytes; 0 = device maximum): with n = 40 they drop,
# in turn, the transposed U0/V0, the solve matrix and the T22 matrix to the global slot
DEFAULT_BUDGETS = (0, 200 * 1024, 150 * 1024, 120 * 1024, 32 * 1024)
CACHE_ENV = "SCCM_GB300_TUNE_CACHE"


def _cache_path():
    return os.environ.get(CACHE_ENV) or os.path.join(os.path.expanduser("~"), ".cache", "sccm_gb300",
                                                      "uneven_schedules.json")


class UnevenBatch:
    """Device buffers, contexts and the persistent-launch plans of a list of workloads.

    Each workload (`synth.Workload`-like: sp, e0, t1b, recs, vbar, q2, mesh,
    vacua, pairs) becomes one context in `form`; its pairs are packed and
    uploaded once. Results stay on the device until `results()`. By default
    all contexts form one group (one persistent launch).
    """

    def __init__(self, workloads, form="df64", device="cuda"):
        self.form = form
        self.ctxs, self.uv, self.zres, self.status, self.parts = [], [], [], [], []
        dev = torch.device(device)
        for wl in workloads:
            ctx = PnampContext(wl.sp, wl.e0, wl.t1b, wl.recs, wl.vbar, wl.mesh, q2=wl.q2, form=form)
            packed = ctx.pack_pairs([(*wl.vacua[i], *wl.vacua[j]) for i, j in wl.pairs])
            npairs = len(wl.pairs)
            uv = torch.from_numpy(packed).to(dev)
            z = torch.zeros((npairs, NOBS, ctx.n_euler, 2), dtype=torch.float64, device=dev)
            st = torch.zeros((npairs, ctx.n_euler), dtype=torch.int32, device=dev)
            self.ctxs.append(ctx)
            self.uv.append(uv)
            self.zres.append(z)
            self.status.append(st)
            self.parts.append((ctx, npairs, uv.data_ptr(), z.data_ptr(), st.data_ptr()))
        self.npairs = [len(wl.pairs) for wl in workloads]
        self.n_gauge = [wl.mesh.n_gauge for wl in workloads]
        self.points = sum(np_ * c.n_euler * g for np_, c, g in zip(self.npairs, self.ctxs, self.n_gauge))
        self.shapes = [(c.n, c.n_euler, g, np_) for c, g, np_ in zip(self.ctxs, self.n_gauge, self.npairs)]
        self.plans, self.groups, self.budgets = [], [], []
        self.schedule_args = (1, 1, 0)
        self.graph = None
        self.set_groups([list(range(len(self.ctxs)))], [0])

    # ------------------------------------------------------------------
    def item_cost(self, c):
        """Relative time of one (pair, Euler point) item of context c: gauge points x n^3."""
        return self.n_gauge[c] * self.ctxs[c].n ** 3

    def set_groups(self, groups, budgets):
        """One persistent launch per group of context indices, each under its shared-memory budget.

        Groups are launched heaviest items first."""
        order = sorted(range(len(groups)), key=lambda g: -max(self.item_cost(c) for c in groups[g]))
        groups = [list(groups[g]) for g in order]
        budgets = [budgets[g] for g in order]
        for p in self.plans:
            p.close()
        self.plans = []
        for grp, b in zip(groups, budgets):
            plan = MultiPlan([self.parts[c] for c in grp])
            plan.placement(b)
            plan.schedule(*self.schedule_args)
            self.plans.append(plan)
        self.groups, self.budgets = groups, list(budgets)
        self.graph = None

    @property
    def plan(self):
        return self.plans[0]

    @property
    def nitems(self):
        return sum(p.nitems for p in self.plans)

    def signature(self):
        name = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
        return json.dumps({"form": self.form, "device": name, "parts": self.shapes}, sort_keys=True)

    def schedule(self, order=1, grab=1, grid=0):
        for p in self.plans:
            p.schedule(order, grab, grid)
        self.schedule_args = (order, grab, grid)
        self.graph = None          # a captured graph holds the old launch configuration

    def placement(self, smem_budget=0):
        """The same budget for every group; returns the first group's shared bytes per CTA."""
        self.graph = None
        out = [p.placement(smem_budget) for p in self.plans]
        self.budgets = [smem_budget] * len(self.plans)
        return out[0]

    def launch(self, stream=None):
        """Enqueue every group's launch on `stream` (default: the current stream), in group order."""
        main = stream if stream is not None else torch.cuda.current_stream()
        for p in self.plans:
            p.launch(main.cuda_stream)

    def capture(self):
        """Capture one launch of every group into a CUDA graph (after one eager warm-up launch)."""
        self.launch()
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.launch(torch.cuda.current_stream())
        self.graph = g
        return g

    def replay(self):
        if self.graph is None:
            self.capture()
        self.graph.replay()

    def results(self):
        """Per context: (zres [npairs, P_E, NOBS] complex128, status [npairs, P_E])."""
        torch.cuda.synchronize()
        out = []
        for z, st in zip(self.zres, self.status):
            zc = z.cpu().numpy().view(np.complex128)[..., 0]          # [npairs, NOBS, P_E]
            out.append((np.ascontiguousarray(zc.transpose(0, 2, 1)), st.cpu().numpy()))
        return out

    def clear(self):
        for z, st in zip(self.zres, self.status):
            z.zero_()
            st.zero_()

    def close(self):
        self.graph = None
        for p in self.plans:
            p.close()
        self.plans = []
        for c in self.ctxs:
            c.close()


def time_launches(fn, reps, flush=None):
    """Median CUDA-event milliseconds of `fn()` over `reps` launches on the current stream."""
    ts = []
    for _ in range(reps):
        if flush is not None:
            flush()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record()
        fn()
        b.record()
        b.synchronize()
        ts.append(a.elapsed_time(b))
    return statistics.median(ts), ts


def _load_table(path):
    if os.path.exists(path):
        try:
            with open(path) as f:
                return json.load(f)
        except (OSError, ValueError):
            pass
    return {}


def autotune(batch: UnevenBatch, schedules=DEFAULT_SCHEDULES, budgets=DEFAULT_BUDGETS, reps=1,
             probe: UnevenBatch | None = None, cache=True):
    """Pick groups, shared-memory budgets and the schedule for `batch`.

    Timed on `probe` (default: the batch itself), a smaller batch with the
    same contexts in the same order. Stage 1 times each context alone under
    each budget (budgets a context cannot fit are skipped). Stage 2 times the
    layouts: all contexts in one launch under each budget; every context in
    its own launch under its best budget; and each pair of contexts merged
    (the others alone) under the budget best for the pair's summed stage-1
    times. Stage 3 times each schedule under the fastest layout. The record
    {"groups", "budgets", "schedule", "ms"} is cached under the batch's
    signature and applied without timing next time.
    """
    sig = batch.signature()
    path = _cache_path()
    table = _load_table(path) if cache else {}
    if sig in table:
        rec = table[sig]
        batch.set_groups(rec["groups"], rec["budgets"])
        batch.schedule(*rec["schedule"])
        return {**rec, "cached": True}
    target = probe if probe is not None else batch
    k = len(target.ctxs)
    ms = {}
    target.schedule(*schedules[0])
    target.launch()                      # warm-up (module load, first-touch of the slots)
    torch.cuda.synchronize()

    # stage 1: each context alone under each budget
    alone = {}
    for c in range(k):
        target.set_groups([[c]], [0])
        for b in budgets:
            try:
                smem = target.placement(b)
            except PnampError:
                continue
            alone[(c, b)], _ = time_launches(target.launch, reps)
            ms[f"ctx{c} smem<={b}:{smem}"] = alone[(c, b)]

    def best_budget(members):
        fits = [b for b in budgets if all((c, b) in alone for c in members)]
        return min(fits, key=lambda b: sum(alone[(c, b)] for c in members)) if fits else None

    # stage 2: layouts
    layouts = [([list(range(k))], [b]) for b in budgets if all((c, b) in alone for c in range(k))]
    if k > 1:
        layouts.append(([[c] for c in range(k)], [best_budget([c]) for c in range(k)]))
    if k > 2:
        for i in range(k):
            for j in range(i + 1, k):
                rest = [c for c in range(k) if c not in (i, j)]
                layouts.append(([[i, j]] + [[c] for c in rest],
                                [best_budget([i, j])] + [best_budget([c]) for c in rest]))
    lt = []
    for groups, bs in layouts:
        if any(b is None for b in bs):
            continue
        target.set_groups(groups, bs)
        t, _ = time_launches(target.launch, reps)
        ms[f"groups {target.groups} budgets {target.budgets}"] = t
        lt.append((t, target.groups, target.budgets))
    _, groups, bs = min(lt, key=lambda x: x[0])
    target.set_groups(groups, bs)

    # stage 3: schedules under the chosen layout
    for s in schedules:
        target.schedule(*s)
        ms[str(tuple(s))], _ = time_launches(target.launch, reps)
    best = min(schedules, key=lambda s: ms[str(tuple(s))])
    batch.set_groups(groups, bs)
    batch.schedule(*best)
    rec = {"groups": batch.groups, "budgets": batch.budgets, "schedule": list(best), "ms": ms,
           "timed_on": "probe" if probe is not None else "batch"}
    if cache:
        table[sig] = rec
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            tmp = path + ".tmp"
            with open(tmp, "w") as f:
                json.dump(table, f, indent=1)
            os.replace(tmp, path)
        except OSError:
            pass
    return {**rec, "cached": False}
