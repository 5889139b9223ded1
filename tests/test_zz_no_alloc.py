"""pnamp_batch_device_noalloc through the C ABI.

Some callers cannot allocate device memory per call: code under a runtime that
owns the device memory budget (a caching allocator, an MPS client with a hard
cap), or code that must not risk the implicit device synchronisation of
cudaMalloc/cudaFree between stream-ordered steps. For them the library keeps
this entry point's scratch in one fixed 32 MiB device array. These tests check
that it reproduces pnamp_batch_device on two calls in a row (the array keeps
the previous call's contents, so the second call also shows nothing stale is
read), and that a request larger than the array is refused.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from sccm_gb300.basis import Mesh
from sccm_gb300.pnamp import PNAMP_ERR_SCRATCH_LIMIT, PnampContext, load_library
from sccm_gb300.synth import make_workload

pytestmark = pytest.mark.gpu

NORM_TOL = 1e-10   # same bounds as the oracle parity tests
OBS_TOL = 1e-9
SCRATCH_BYTES = 32 << 20


def _run(fn, ctx, packed):
    dev = torch.device("cuda")
    npairs = packed.shape[0]
    uv = torch.from_numpy(np.ascontiguousarray(packed)).to(dev)
    z = torch.zeros((npairs, 19 * ctx.n_euler * 2), dtype=torch.float64, device=dev)
    st = torch.full((npairs, ctx.n_euler), -1, dtype=torch.int32, device=dev)
    torch.cuda.synchronize()
    rc = fn(ctx.handle, npairs, C.c_void_p(uv.data_ptr()), C.c_void_p(z.data_ptr()),
            C.c_void_p(st.data_ptr()), C.c_void_p(0))
    torch.cuda.synchronize()
    assert rc == 0, rc
    zz = z.cpu().numpy().view(np.complex128).reshape(npairs, 19, ctx.n_euler)
    return zz, st.cpu().numpy()


def test_noalloc_matches_batch_device_on_two_calls():
    lib = load_library()
    w = make_workload("pf", 3, Mesh(2, 3, 2, 3), seed=404)
    with PnampContext(w.sp, w.e0, w.t1b, w.recs, w.vbar, w.mesh, q2=w.q2) as ctx:
        for pairs in ([(0, 1), (1, 2)], [(2, 2), (0, 0), (1, 0)]):
            packed = ctx.pack_pairs([(*w.vacua[i], *w.vacua[j]) for i, j in pairs])
            z_ref, s_ref = _run(lib.pnamp_batch_device, ctx, packed)
            z_new, s_new = _run(lib.pnamp_batch_device_noalloc, ctx, packed)
            assert np.array_equal(s_ref, s_new)
            for k in range(len(pairs)):
                scale = np.abs(z_ref[k, 0]).max()
                assert np.abs(z_new[k, 0] - z_ref[k, 0]).max() <= NORM_TOL * scale
                for io in range(1, 19):
                    sc = np.abs(z_ref[k, io]).max()
                    assert np.abs(z_new[k, io] - z_ref[k, io]).max() <= OBS_TOL * sc


def test_noalloc_refuses_requests_beyond_its_scratch():
    lib = load_library()
    w = make_workload("pf", 1, Mesh(1, 1, 1, 1), seed=405)
    n = w.sp.nlev
    npairs = 500
    assert npairs * (6 * n * n + 4) * 8 > SCRATCH_BYTES     # pair records alone overflow
    with PnampContext(w.sp, w.e0, w.t1b, w.recs, w.vbar, w.mesh, q2=w.q2) as ctx:
        dev = torch.device("cuda")
        uv = torch.zeros((npairs, 4, n, n), dtype=torch.float64, device=dev)
        z = torch.zeros((npairs, 19 * ctx.n_euler * 2), dtype=torch.float64, device=dev)
        st = torch.zeros((npairs, ctx.n_euler), dtype=torch.int32, device=dev)
        rc = lib.pnamp_batch_device_noalloc(ctx.handle, npairs, C.c_void_p(uv.data_ptr()),
                                            C.c_void_p(z.data_ptr()), C.c_void_p(st.data_ptr()),
                                            C.c_void_p(0))
        torch.cuda.synchronize()
        assert rc == PNAMP_ERR_SCRATCH_LIMIT


def test_noalloc_with_fewer_workspaces_than_ctas_allocates_nothing():
    """120 pf pairs: their records fill a third of the array, so only ~110 CTA workspaces fit
    (fewer than the 152-CTA grid of pnamp_batch_device) and the grid-stride loop runs on a cut
    grid. Results equal pnamp_batch_device's, and the device's free memory does not move across
    the call."""
    lib = load_library()
    w = make_workload("pf", 3, Mesh(1, 2, 1, 3), seed=406)
    pairs = (w.pairs * 20)[:120]
    with PnampContext(w.sp, w.e0, w.t1b, w.recs, w.vbar, w.mesh, q2=w.q2) as ctx:
        n = w.sp.nlev
        rec = (7 * n * n + 8) * 8
        assert len(pairs) * rec > SCRATCH_BYTES // 4
        packed = ctx.pack_pairs([(*w.vacua[i], *w.vacua[j]) for i, j in pairs])
        z_ref, s_ref = _run(lib.pnamp_batch_device, ctx, packed)
        _run(lib.pnamp_batch_device_noalloc, ctx, packed)          # first call: address lookup
        dev = torch.device("cuda")
        uv = torch.from_numpy(np.ascontiguousarray(packed)).to(dev)
        z = torch.zeros((len(pairs), 19 * ctx.n_euler * 2), dtype=torch.float64, device=dev)
        st = torch.zeros((len(pairs), ctx.n_euler), dtype=torch.int32, device=dev)
        torch.cuda.synchronize()
        free0, _ = torch.cuda.mem_get_info()
        rc = lib.pnamp_batch_device_noalloc(ctx.handle, len(pairs), C.c_void_p(uv.data_ptr()),
                                            C.c_void_p(z.data_ptr()), C.c_void_p(st.data_ptr()), C.c_void_p(0))
        torch.cuda.synchronize()
        free1, _ = torch.cuda.mem_get_info()
        assert rc == 0 and free1 == free0
        z_new = z.cpu().numpy().view(np.complex128).reshape(len(pairs), 19, ctx.n_euler)
        assert np.array_equal(s_ref, st.cpu().numpy())
        for k in range(len(pairs)):
            scale = np.abs(z_ref[k, 0]).max()
            assert np.abs(z_new[k, 0] - z_ref[k, 0]).max() <= NORM_TOL * scale
