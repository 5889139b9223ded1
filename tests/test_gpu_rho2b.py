"""Two-body transition density (Rho2B) on the GPU through the C ABI, against the oracle.

The kernel sums, per quadruple (k_i, k_j, k_k, k_l), the norm-weighted density product
of every gauge point over the mesh; the host couples them to J and normalises by N^0.
Both are compared with the oracle's literal ZRho2B_Angles sequence on small meshes:
sd (n = 24, general path), pf (n = 40, species-split path), sd+pf (n = 64, per-point
arrays in the global workspace); the traces must count the pairs of nucleons."""
import numpy as np
import pytest

from sccm_gb300.basis import Mesh
from sccm_gb300.pnamp import PNAMP_ERR_STATE, PnampContext, PnampError
from sccm_gb300.synth import make_workload
from oracle.pnamp_oracle import Hamiltonian, kernel_triaxial, rho2b_write_me2b
from test_rho2b_host import trace_by_species

pytestmark = pytest.mark.gpu

SUM_TOL = 1e-10     # quadruple sums, relative to the largest
ELEM_TOL = 1e-10    # coupled and normalised elements, relative to the largest


def ctx_for(w, form):
    return PnampContext(w.sp, w.e0, w.t1b, w.recs, w.vbar, w.mesh, q2=w.q2, form=form)


def oracle(w, i, j, quads):
    ham = Hamiltonian(w.e0, w.t1b, w.recs, w.vbar, w.q2, w.jops)
    return kernel_triaxial(w.sp, ham, w.mesh, *w.vacua[i], *w.vacua[j], rho2b=quads)


CASES = {
    "sd": (("sd", 3, Mesh(2, 3, 2, 3), 61), [(0, 1), (2, 2)]),
    "pf": (("pf", 2, Mesh(1, 2, 2, 3), 62), [(0, 1)]),
    "sdpf": (("sdpf", 2, Mesh(1, 1, 2, 3), 63), [(0, 1)]),
}


@pytest.mark.parametrize("form", ["fp64", "df64"])
@pytest.mark.parametrize("case", sorted(CASES))
def test_rho2b_matches_oracle(case, form):
    (shell, nvac, mesh, seed), pairs = CASES[case]
    w = make_workload(shell, nvac, mesh, seed=seed)
    with ctx_for(w, form) as ctx:
        tab = ctx.rho2b_tables()
        z, st, r2 = ctx.batch_rho2b([(*w.vacua[i], *w.vacua[j]) for i, j in pairs])
        vals = [ctx.project_rho2b(z[k], r2[k]) for k in range(len(pairs))]
        z_plain, st_plain = ctx.batch([(*w.vacua[i], *w.vacua[j]) for i, j in pairs])
    # observables untouched: the plain launch runs split pairs two gauge points at a time and
    # adds the two halves' sums at the end, so the values agree to rounding, not bit for bit
    assert np.abs(z - z_plain).max() <= 1e-13 * np.abs(z_plain).max() and np.array_equal(st, st_plain)
    wts = w.mesh.euler_points()[:, 3]
    terms = [list(zip(tab["term_q"][a:b], tab["term_c"][a:b])) for a, b in zip(tab["ptr"][:-1], tab["ptr"][1:])]
    for k, (i, j) in enumerate(pairs):
        zo, ao = oracle(w, i, j, tab["quads"])
        ref = wts @ ao
        assert np.abs(r2[k] - ref).max() <= SUM_TOL * np.abs(ref).max(), (case, k)
        vo = rho2b_write_me2b(terms, zo, ao, w.mesh)
        assert np.abs(vals[k] - vo).max() <= ELEM_TOL * np.abs(vo).max(), (case, k)


def test_rho2b_traces_count_pairs():
    w = make_workload("sd", 2, Mesh(2, 4, 2, 7), seed=5)
    with ctx_for(w, "df64") as ctx:
        tab = ctx.rho2b_tables()
        z, _, r2 = ctx.batch_rho2b([(*w.vacua[0], *w.vacua[1])])
        vals = ctx.project_rho2b(z[0], r2[0])
    tr = trace_by_species(tab["blocks"], vals)
    Z, N = w.sp.nprot, w.sp.nneut
    assert abs(tr[0] - N * (N - 1)) < 1e-4
    assert abs(tr[2] - Z * (Z - 1)) < 1e-4
    assert abs(tr[1] - 2 * N * Z) < 1e-4


def test_rho2b_device_entry_and_norm_only_mode():
    import torch
    w = make_workload("sd", 2, Mesh(1, 2, 1, 3), seed=64)
    with ctx_for(w, "fp64") as ctx:
        nq = ctx.rho2b_tables()["quads"].shape[0]
        _, _, ref = ctx.batch_rho2b([(*w.vacua[0], *w.vacua[1])])
        dev = torch.device("cuda")
        uv = torch.from_numpy(ctx.pack_pairs([(*w.vacua[0], *w.vacua[1])])).to(dev)
        zr = torch.zeros((1, 19, ctx.n_euler, 2), dtype=torch.float64, device=dev)
        st = torch.zeros((1, ctx.n_euler), dtype=torch.int32, device=dev)
        out = torch.full((1, nq, 2), 7.0, dtype=torch.float64, device=dev)   # overwritten, not added to
        from sccm_gb300.pnamp import load_library
        lib = load_library()
        rc = lib.pnamp_batch_rho2b_device(ctx._h, 1, uv.data_ptr(), zr.data_ptr(), st.data_ptr(),
                                          out.data_ptr(), None)
        assert rc == 0
        torch.cuda.synchronize()
        got = out.cpu().numpy()[0]
        got = got[:, 0] + 1j * got[:, 1]
        assert np.abs(got - ref[0]).max() <= 1e-13 * np.abs(ref).max()
        ctx.set_outputs("norm")
        with pytest.raises(PnampError) as e:
            ctx.batch_rho2b([(*w.vacua[0], *w.vacua[1])])
        assert e.value.code == PNAMP_ERR_STATE


def test_driver_writes_rho2b_files(tmp_path):
    from sccm_gb300.driver import rank_pairs, rho2b_name, run_pairs
    from sccm_gb300.formats import read_rho2b_dat
    w = make_workload("sd", 2, Mesh(1, 2, 1, 3), seed=65)
    with ctx_for(w, "df64") as ctx:
        run_pairs(ctx, w.vacua, rank_pairs([(1, 2)], 0, 1), str(tmp_path), batch=1, rho2b=True)
        z, _, r2 = ctx.batch_rho2b([(*w.vacua[0], *w.vacua[1])])
        vals = ctx.project_rho2b(z[0], r2[0])
        blocks = ctx.rho2b_tables()["blocks"]
    got = read_rho2b_dat(tmp_path / rho2b_name(1, 2))
    e = 0
    for bm, (*_, st) in enumerate(blocks):
        for a in range(len(st)):
            for b in range(len(st)):
                if abs(vals[e]) > 1e-8:
                    assert abs(got[(bm, a, b)] - vals[e].real) <= 5e-11
                e += 1
    assert len(got) > 0


def test_both_densities_in_one_pass(tmp_path):
    """pnamp_batch_densities: the one- and two-body densities from one launch equal the
    separate launches', and the driver writes both files from it."""
    from sccm_gb300.driver import rank_pairs, rho1b_name, rho2b_name, run_pairs
    from sccm_gb300.formats import read_rho1b_dens, read_rho2b_dat
    w = make_workload("sd", 2, Mesh(1, 2, 2, 3), seed=66)
    pairs = [(*w.vacua[0], *w.vacua[1]), (*w.vacua[1], *w.vacua[1])]
    with ctx_for(w, "df64") as ctx:
        z, st, r1, r2 = ctx.batch_densities(pairs)
        z1, st1, r1s = ctx.batch_rho1b(pairs)
        z2, st2, r2s = ctx.batch_rho2b(pairs)
        run_pairs(ctx, w.vacua, rank_pairs([(1, 2)], 0, 1), str(tmp_path), batch=1, rho1b=True, rho2b=True)
    assert np.array_equal(z, z1) and np.array_equal(z, z2) and np.array_equal(st, st1)
    assert np.array_equal(r1, r1s)
    assert np.abs(r2 - r2s).max() <= 1e-13 * np.abs(r2s).max()   # atomic adds: order may differ
    assert len(read_rho1b_dens(tmp_path / rho1b_name(1, 2))) > 0
    assert len(read_rho2b_dat(tmp_path / rho2b_name(1, 2))) > 0


@pytest.mark.parametrize("form", ["fp64", "df64"])
def test_densities_device_entry_with_one_output(form):
    """pnamp_batch_densities_device on the pf species-split path in both forms: with both
    outputs it equals the single-density launches, with d_rho1b = NULL it writes only the
    two-body sums and with d_rho2b = NULL only the one-body blocks; norm-only outputs are
    refused."""
    import ctypes as C
    import torch
    from sccm_gb300.pnamp import load_library
    lib = load_library()
    w = make_workload("pf", 2, Mesh(1, 2, 1, 3), seed=67)
    pairs = [(*w.vacua[0], *w.vacua[1]), (*w.vacua[1], *w.vacua[1])]
    dev = torch.device("cuda")
    with ctx_for(w, form) as ctx:
        _, _, r1s = ctx.batch_rho1b(pairs)
        _, _, r2s = ctx.batch_rho2b(pairs)
        nb, nq, P = r1s.shape[1], r2s.shape[1], ctx.n_euler
        uv = torch.from_numpy(ctx.pack_pairs(pairs)).to(dev)
        z = torch.zeros((2, 19 * P * 2), dtype=torch.float64, device=dev)
        st = torch.zeros((2, P), dtype=torch.int32, device=dev)
        out = {}
        for which in ("both", "rho2b", "rho1b"):
            r1 = torch.zeros((2, nb * P * 2), dtype=torch.float64, device=dev)
            r2 = torch.zeros((2, nq * 2), dtype=torch.float64, device=dev)
            p1 = None if which == "rho2b" else C.c_void_p(r1.data_ptr())
            p2 = None if which == "rho1b" else C.c_void_p(r2.data_ptr())
            rc = lib.pnamp_batch_densities_device(ctx.handle, 2, C.c_void_p(uv.data_ptr()), C.c_void_p(z.data_ptr()),
                                                  C.c_void_p(st.data_ptr()), p1, p2, C.c_void_p(0))
            torch.cuda.synchronize()
            assert rc == 0, rc
            out[which] = (r1.cpu().numpy().view(np.complex128).reshape(2, nb, P),
                          r2.cpu().numpy().view(np.complex128).reshape(2, nq))
        ctx.set_outputs("norm")
        rc = lib.pnamp_batch_densities_device(ctx.handle, 2, C.c_void_p(uv.data_ptr()), C.c_void_p(z.data_ptr()),
                                              C.c_void_p(st.data_ptr()), C.c_void_p(r1.data_ptr()), None,
                                              C.c_void_p(0))
        assert rc == PNAMP_ERR_STATE
    scale2 = np.abs(r2s).max()
    assert np.array_equal(out["both"][0], r1s) and np.abs(out["both"][1] - r2s).max() <= 1e-13 * scale2
    assert np.abs(out["rho2b"][1] - r2s).max() <= 1e-13 * scale2 and not out["rho2b"][0].any()
    assert np.array_equal(out["rho1b"][0], r1s) and not out["rho1b"][1].any()
