"""Uneven batches in one persistent launch (pnamp_multi_* through the C ABI).

Three model spaces with their own meshes (sd n=24, pf n=40, sd+pf n=64) run
as one launch. Each context's results must equal what the single-context
batch path gives for the same pairs (same per-point code, so to rounding),
for every work order and grab size; the sd part is also checked against the
oracle; a replayed CUDA graph must reproduce an eager launch bit for bit.
"""
import numpy as np
import pytest
import torch

from sccm_gb300.basis import Mesh
from sccm_gb300.pnamp import PNAMP_ERR_ARG, PNAMP_ERR_UNSUPPORTED, MultiPlan, PnampContext, PnampError
from sccm_gb300.synth import make_workload
from sccm_gb300.uneven import UnevenBatch, autotune
from oracle.pnamp_oracle import Hamiltonian, kernel_triaxial

pytestmark = pytest.mark.gpu

NORM_TOL = 1e-10
OBS_TOL = 1e-9
# multi-context vs single-context launch: the same point code, except that a context whose
# shared-memory budget cannot hold two gauge points runs species-split pairs one point at a
# time, which sums the gauge points in another order (double-float rounding, ~3e-13)
SAME_TOL = 1e-12


def _workloads():
    a = make_workload("sd", 3, Mesh(2, 3, 2, 3), seed=71)
    a.pairs = [(0, 1), (2, 2), (1, 0)]
    b = make_workload("pf", 2, Mesh(2, 2, 3, 5), seed=72)
    b.pairs = [(0, 1), (1, 1)]
    c = make_workload("sdpf", 2, Mesh(1, 2, 2, 3), seed=73)
    c.pairs = [(0, 1)]
    return [a, b, c]


def _single(wl, form):
    with PnampContext(wl.sp, wl.e0, wl.t1b, wl.recs, wl.vbar, wl.mesh, q2=wl.q2, form=form) as ctx:
        return ctx.batch([(*wl.vacua[i], *wl.vacua[j]) for i, j in wl.pairs])


def _close(z, ref, tol_norm, tol_obs):
    for k in range(ref.shape[0]):
        for io in range(ref.shape[2]):
            sc = np.abs(ref[k, :, io]).max()
            tol = tol_norm if io == 0 else tol_obs
            assert np.abs(z[k, :, io] - ref[k, :, io]).max() <= tol * max(sc, 1e-300), (k, io)


@pytest.fixture(scope="module")
def wls():
    return _workloads()


@pytest.mark.parametrize("form", ["fp64", "df64"])
def test_multi_matches_single_context(wls, form):
    refs = [_single(w, form) for w in wls]
    ub = UnevenBatch(wls, form=form)
    try:
        assert ub.nitems == sum(len(w.pairs) * c.n_euler for w, c in zip(wls, ub.ctxs))
        for sched, budget in [((0, 1, 0), 0), ((1, 1, 0), 0), ((2, 1, 0), 0), ((1, 3, 0), 120 * 1024),
                              ((2, 2, 7), 32 * 1024)]:
            ub.clear()
            ub.placement(budget)
            ub.schedule(*sched)
            ub.launch()
            for (z, st), (zr, sr) in zip(ub.results(), refs):
                assert np.array_equal(st, sr), sched
                _close(z, zr, SAME_TOL, SAME_TOL)
        # two groups (two persistent launches, one after the other), own budgets
        ub.clear()
        ub.set_groups([[1], [0, 2]], [0, 32 * 1024])
        assert ub.groups[0] == [0, 2]          # heaviest items (n = 64) first
        ub.launch()
        for (z, st), (zr, sr) in zip(ub.results(), refs):
            assert np.array_equal(st, sr)
            _close(z, zr, SAME_TOL, SAME_TOL)
    finally:
        ub.close()


def test_multi_sd_part_matches_oracle(wls):
    w = wls[0]
    ham = Hamiltonian(w.e0, w.t1b, w.recs, w.vbar, w.q2, w.jops)
    ub = UnevenBatch(wls, form="fp64")
    try:
        ub.launch()
        z, _ = ub.results()[0]
    finally:
        ub.close()
    ref = np.stack([kernel_triaxial(w.sp, ham, w.mesh, *w.vacua[i], *w.vacua[j]) for i, j in w.pairs])
    _close(z, ref, NORM_TOL, OBS_TOL)


@pytest.mark.parametrize("groups", [None, ([[2], [0, 1]], [32 * 1024, 0])])
def test_graph_replay_matches_eager(wls, groups):
    ub = UnevenBatch(wls, form="df64")
    try:
        if groups:
            ub.set_groups(*groups)
        ub.schedule(1, 2, 0)
        ub.launch()
        eager = ub.results()
        ub.capture()
        for _ in range(2):
            ub.clear()
            ub.replay()
            for (z, st), (ze, se) in zip(ub.results(), eager):
                assert np.array_equal(z, ze) and np.array_equal(st, se)
    finally:
        ub.close()


def test_autotune_picks_and_caches(wls, tmp_path, monkeypatch):
    monkeypatch.setenv("SCCM_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    ub = UnevenBatch(wls, form="df64")
    try:
        scheds = ((0, 1, 0), (1, 4, 0), (2, 1, 0))
        budgets = (0, 64 * 1024, 4 * 1024)       # the last fits no context: skipped
        rec = autotune(ub, schedules=scheds, budgets=budgets)
        assert not rec["cached"] and tuple(rec["schedule"]) in scheds
        assert sorted(c for g in rec["groups"] for c in g) == [0, 1, 2]
        assert all(b in budgets[:2] for b in rec["budgets"])
        assert {str(s) for s in scheds} <= set(rec["ms"])
        assert sum(1 for key in rec["ms"] if key.startswith("ctx")) == 3 * 2
        again = autotune(ub, schedules=scheds, budgets=budgets)
        assert again["cached"] and again["schedule"] == rec["schedule"]
        assert ub.schedule_args == tuple(rec["schedule"])
        assert ub.groups == rec["groups"] and ub.budgets == rec["budgets"]
    finally:
        ub.close()


def test_multi_rejects_bad_arguments(wls):
    a, b = wls[0], wls[1]
    c1 = PnampContext(a.sp, a.e0, a.t1b, a.recs, a.vbar, a.mesh, q2=a.q2, form="fp64")
    c2 = PnampContext(b.sp, b.e0, b.t1b, b.recs, b.vbar, b.mesh, q2=b.q2, form="df64")
    dev = torch.device("cuda")
    bufs = []
    parts = []
    for c in (c1, c2):
        uv = torch.zeros((1, 4, c.n, c.n), dtype=torch.float64, device=dev)
        z = torch.zeros((1, 19, c.n_euler, 2), dtype=torch.float64, device=dev)
        st = torch.zeros((1, c.n_euler), dtype=torch.int32, device=dev)
        bufs += [uv, z, st]
        parts.append((c, 1, uv.data_ptr(), z.data_ptr(), st.data_ptr()))
    try:
        with pytest.raises(PnampError) as e:          # contexts in different forms
            MultiPlan(parts)
        assert e.value.code == PNAMP_ERR_ARG
        with pytest.raises(PnampError) as e:          # more contexts than one launch carries
            MultiPlan(parts[:1] * 5)
        assert e.value.code == PNAMP_ERR_UNSUPPORTED
        plan = MultiPlan(parts[:1])
        with pytest.raises(PnampError) as e:
            plan.schedule(1, 0, 0)                    # grab must be >= 1
        assert e.value.code == PNAMP_ERR_ARG
        plan.close()
    finally:
        c1.close()
        c2.close()
