"""GPU (C-ABI) vs oracle parity on seeded inputs, and the Ge76 kernel files through the GPU.

Tolerances (FP64 throughout):
  * norm kernel N(Omega) = ZRES(:,1): 1e-10 relative to max |N| over the mesh
  * the other observables ZRES(:,2..18): 1e-9 relative to max |column|
  * projected fields vs the reference's Ge76 kernel files: 2e-7 relative
    (the files print 8 significant digits)
"""
import os

import numpy as np
import pytest

from sccm_gb300.basis import JJMAX, Mesh
from sccm_gb300.pnamp import PnampContext, PnampError, PNAMP_ERR_SINGULAR_U
from sccm_gb300.synth import make_workload
from oracle.pnamp_oracle import Hamiltonian, kernel_triaxial, project

pytestmark = pytest.mark.gpu

NORM_TOL = 1e-10
OBS_TOL = 1e-9


FORMS = ["fp64", "df64"]


def ctx_for(w, mesh, iE2=True, form="fp64"):
    return PnampContext(w.sp, w.e0, w.t1b, w.recs, w.vbar, mesh, q2=w.q2 if iE2 else None, form=form)


def oracle_zres(w, mesh, i, j, iE2=True):
    ham = Hamiltonian(w.e0, w.t1b, w.recs, w.vbar, w.q2, w.jops)
    (U0, V0), (U1, V1) = w.vacua[i], w.vacua[j]
    return kernel_triaxial(w.sp, ham, mesh, U0, V0, U1, V1, iE2=iE2)


def assert_zres_close(z_gpu, z_ref):
    nref = np.abs(z_ref[:, 0]).max()
    err = np.abs(z_gpu[:, 0] - z_ref[:, 0]).max() / nref
    assert err <= NORM_TOL, f"norm kernel rel err {err:.2e}"
    for io in range(1, z_ref.shape[1]):
        scale = np.abs(z_ref[:, io]).max()
        if scale == 0.0:
            assert np.abs(z_gpu[:, io]).max() == 0.0, io
            continue
        e = np.abs(z_gpu[:, io] - z_ref[:, io]).max() / scale
        assert e <= OBS_TOL, f"observable {io + 1}: rel err {e:.2e}"


@pytest.fixture(scope="module")
def sd():
    return make_workload("sd", 2, Mesh(3, 4, 3, 3), seed=101, deformed=False)


@pytest.fixture(scope="module")
def pf():
    return make_workload("pf", 2, Mesh(2, 3, 2, 3), seed=202)


@pytest.mark.parametrize("form", FORMS)
def test_sd_pair_matches_oracle(sd, form):
    with ctx_for(sd, sd.mesh, form=form) as ctx:
        r = ctx.pair(*sd.vacua[0], *sd.vacua[1])
    assert (r.status & ~1).max() == 0
    assert_zres_close(r.zres, oracle_zres(sd, sd.mesh, 0, 1))


@pytest.mark.parametrize("form", FORMS)
def test_sd_diagonal_pair_matches_oracle(sd, form):
    with ctx_for(sd, sd.mesh, form=form) as ctx:
        z, st = ctx.batch([(*sd.vacua[1], *sd.vacua[1])])
    assert_zres_close(z[0], oracle_zres(sd, sd.mesh, 1, 1))


@pytest.mark.parametrize("form", FORMS)
def test_pf_pair_matches_oracle(pf, form):
    with ctx_for(pf, pf.mesh, form=form) as ctx:
        r = ctx.pair(*pf.vacua[0], *pf.vacua[1])
    assert_zres_close(r.zres, oracle_zres(pf, pf.mesh, 0, 1))


@pytest.mark.parametrize("form", FORMS)
def test_sdpf_n64_global_workspace_matches_oracle(form):
    w = make_workload("sdpf", 2, Mesh(1, 2, 1, 2), seed=303)
    with ctx_for(w, w.mesh, form=form) as ctx:
        r = ctx.pair(*w.vacua[0], *w.vacua[1])
    assert_zres_close(r.zres, oracle_zres(w, w.mesh, 0, 1))


def test_norm_is_one_at_identity(sd):
    mesh = Mesh(1, 1, 1, 1)
    with ctx_for(sd, mesh) as ctx:
        r = ctx.pair(*sd.vacua[0], *sd.vacua[0])
    assert abs(r.zres[0, 0] - 1.0) < 1e-12
    assert abs(r.zres[0, 1] - sd.sp.nprot) < 1e-10 and abs(r.zres[0, 2] - sd.sp.nneut) < 1e-10


def test_batch_equals_single_pairs(sd):
    with ctx_for(sd, sd.mesh) as ctx:
        z, _ = ctx.batch([(*sd.vacua[0], *sd.vacua[1]), (*sd.vacua[1], *sd.vacua[0])])
        a = ctx.pair(*sd.vacua[0], *sd.vacua[1]).zres
        b = ctx.pair(*sd.vacua[1], *sd.vacua[0]).zres
    assert np.array_equal(z[0], a) and np.array_equal(z[1], b)


def test_projection_matches_oracle(sd):
    z = oracle_zres(sd, sd.mesh, 0, 1)
    ref = project(z, sd.mesh, chop=1e-8)
    with ctx_for(sd, sd.mesh) as ctx:
        got = ctx.project(z, chop=True)
    # sums: 1e-12; ratio fields (<N>, <Z>, <J^2> divide by N^J): 1e-10
    for f, tol in (("njkk", 1e-12), ("hjkk", 1e-12), ("nn", 1e-10), ("zz", 1e-10), ("J2", 1e-10)):
        scale = max(np.abs(ref[f]).max(), 1e-30)
        assert np.abs(got[f] - ref[f]).max() <= tol * scale + 1e-14, f


def test_singular_u_is_reported(sd):
    U, V = sd.vacua[0]
    Us = U.copy()
    Us[:, 3] = 0.0
    with ctx_for(sd, Mesh(1, 1, 1, 1)) as ctx:
        with pytest.raises(PnampError) as e:
            ctx.pair(Us, V, U, V)
    assert e.value.code == PNAMP_ERR_SINGULAR_U


@pytest.mark.parametrize("form", FORMS)
def test_ge76_kernel_files_through_gpu(ge76, form):
    """All 16 intact Ge76 pairs in one batch reproduce the reference's kernel files."""
    g = ge76
    mesh = Mesh(1, g["nbet"], 1, g["nfom"], ncosbet=g["ncosbet"])
    idx = [(i, j) for i in range(4) for j in range(4)]
    with PnampContext(g["sp"], g["e0"], g["t1b"], g["recs"], g["vbar"], mesh, q2=g["q2"], form=form) as ctx:
        z, st = ctx.batch([(g["U"][i], g["V"][i], g["U"][j], g["V"][j]) for i, j in idx])
        for k, (i, j) in enumerate(idx):
            kern = ctx.project(z[k], chop=False)
            gold = g["gold"][i, j]
            n0 = abs(gold[0, 0])
            for jj, J in enumerate(g["jvals"]):
                if abs(gold[jj, 0]) < 1e-6 * n0:
                    continue
                for f, name in enumerate(("njkk", "hjkk", "nn", "zz", "J2")):
                    mine = kern[name][J, JJMAX, JJMAX].real
                    ref = gold[jj, f].real
                    assert abs(mine - ref) <= 2e-7 * abs(ref) + 1e-12, ((i, j), J, name, mine, ref)


def test_df64_form_energies_within_1kev_of_fp64():
    """Every form must keep E_J and GCM levels within 1 keV of FP64."""
    from sccm_gb300.forms import compare
    w = make_workload("pf", 4, Mesh(4, 8, 4, 5), seed=606)
    r = compare(w, "df64")
    assert r["max_rel_err_norm_kernel"] <= NORM_TOL
    assert r["max_abs_err_gcm_levels_keV"] < 1.0
    assert r["max_abs_err_EJ_per_vacuum_keV"] < 1.0


def test_ge76_gcm_levels_match_reference_kernel_files(ge76):
    """Hill-Wheeler on the GPU kernels reproduces the levels from the reference's kernel files."""
    from sccm_gb300.gcm import gcm_levels, compare_levels
    g = ge76
    mesh = Mesh(1, g["nbet"], 1, g["nfom"], ncosbet=g["ncosbet"])
    pairs = [(i, j) for i in range(4) for j in range(i, 4)]
    with PnampContext(g["sp"], g["e0"], g["t1b"], g["recs"], g["vbar"], mesh, q2=g["q2"]) as ctx:
        z, _ = ctx.batch([(g["U"][i], g["V"][i], g["U"][j], g["V"][j]) for i, j in pairs])
        mine = [ctx.project(z[k], chop=False) for k in range(len(pairs))]
    ref = []
    for (i, j) in pairs:
        k = {f: np.zeros((7, 13, 13), complex) for f in ("njkk", "hjkk")}
        for jj, J in enumerate(g["jvals"]):
            k["njkk"][J, JJMAX, JJMAX] = g["gold"][i, j, jj, 0]
            k["hjkk"][J, JJMAX, JJMAX] = g["gold"][i, j, jj, 1]
        ref.append(k)
    a = gcm_levels(mine, pairs, 4, jvals=(0, 2, 4), axial=True)
    b = gcm_levels(ref, pairs, 4, jvals=(0, 2, 4), axial=True)
    dl, dq = compare_levels(a, b, nlev=2)
    assert dl < 1e-3 and dq < 1e-3, (dl, dq)   # MeV: within 1 keV


@pytest.mark.parametrize("form", FORMS)
def test_nfom1_uses_onishi_norm_like_the_reference(sd, form):
    """NFOM = 1: Kernel3D.f90:286-290 switches to the Onishi norm (principal square root)."""
    mesh = Mesh(2, 3, 2, 1)
    with ctx_for(sd, mesh, form=form) as ctx:
        r = ctx.pair(*sd.vacua[0], *sd.vacua[1])
    assert_zres_close(r.zres, oracle_zres(sd, mesh, 0, 1))


def test_quadrupole_projection_matches_oracle(sd):
    """<J1 K1||Q2||J2 K2>, dJ = 0, 1, 2, direct and exchanged (PNAMP_Kernel3D_v2.f90:515-600)."""
    from oracle.pnamp_oracle import project_q
    mesh = Mesh(2, 3, 2, 2)
    z = oracle_zres(sd, mesh, 0, 1)
    qp_ref, qc_ref = project_q(z, mesh, exchange=True, jmax=4)
    with ctx_for(sd, mesh) as ctx:
        qp, qc = ctx.project_q(z, exchange=True)
    for got, ref in ((qp, qp_ref), (qc, qc_ref)):
        scale = np.abs(ref).max()
        assert scale > 0
        assert np.abs(got[:5] - ref[:5]).max() <= 1e-12 * scale


def test_driver_writes_kernel_files_and_resumes(sd, tmp_path):
    """PNAMP_Main's loop for one rank: kernel files written atomically, manifest resumes."""
    from sccm_gb300.driver import pair_list, rank_pairs, run_pairs, elem_name
    from sccm_gb300.formats import read_elem_general
    pairs = pair_list(1, 2, 1, 2, icons=0)
    from sccm_gb300.driver import rho1b_name
    from sccm_gb300.formats import read_rho1b_dens
    with ctx_for(sd, sd.mesh) as ctx:
        done = run_pairs(ctx, sd.vacua, rank_pairs(pairs, 0, 1), str(tmp_path), batch=2, rho1b=True)
        assert done == pairs
        z, _, r1 = ctx.batch_rho1b([(*sd.vacua[0], *sd.vacua[1])])
        kern = ctx.project(z[0])
        dens = ctx.project_rho1b(z[0], r1[0])
        blocks = ctx.rho1b_blocks()
    got = read_rho1b_dens(tmp_path / rho1b_name(1, 2))
    for b, v in zip(blocks, dens):
        if b[:4] in got:
            assert abs(got[b[:4]] - v) <= 1e-10
    with ctx_for(sd, sd.mesh) as ctx:
        before = os.path.getmtime(tmp_path / elem_name("kern", 1, 2))
        run_pairs(ctx, sd.vacua, pairs, str(tmp_path))          # nothing left to do
        assert os.path.getmtime(tmp_path / elem_name("kern", 1, 2)) == before
    r, _ = read_elem_general(tmp_path / elem_name("kern", 1, 2))
    for f in ("njkk", "hjkk"):
        sc = np.abs(kern[f]).max()
        assert np.abs(r[f][::2] - kern[f][::2]).max() <= 1e-7 * sc


RHO1B_TOL = 2e-9   # the reference's .dens files print 10 decimals


@pytest.mark.parametrize("form", FORMS)
def test_ge76_rho1b_files_through_gpu(ge76, form):
    """The J = 0 one-body densities of the 16 Ge76 pairs reproduce data/Ge/Rho1B.*.dens."""
    g = ge76
    mesh = Mesh(1, g["nbet"], 1, g["nfom"], ncosbet=g["ncosbet"])
    idx = [(i, j) for i in range(4) for j in range(4)]
    with PnampContext(g["sp"], g["e0"], g["t1b"], g["recs"], g["vbar"], mesh, q2=None, form=form) as ctx:
        assert [b[:4] for b in ctx.rho1b_blocks()] == g["rho1b_keys"]
        z, _, r = ctx.batch_rho1b([(g["U"][i], g["V"][i], g["U"][j], g["V"][j]) for i, j in idx])
        for k, (i, j) in enumerate(idx):
            vals = ctx.project_rho1b(z[k], r[k])
            assert np.abs(vals - g["rho1b_gold"][i, j]).max() <= RHO1B_TOL, ((i, j), vals)


def test_rho1b_blocks_with_two_radial_orbits_match_oracle():
    """A space with 0p1/2 and 1p1/2: off-diagonal (n1 != n2) blocks against the oracle."""
    from oracle.pnamp_oracle import rho1b_table
    w = make_workload("p2", 3, Mesh(2, 3, 2, 3), seed=909)
    ham = Hamiltonian(w.e0, w.t1b, w.recs, w.vbar, w.q2, w.jops)
    table = rho1b_table(w.sp)
    assert any(k[2] != k[3] for k, _ in table)
    with ctx_for(w, w.mesh) as ctx:
        assert ctx.rho1b_blocks() == [k for k, _ in table]
        pairs = [(0, 1), (2, 2)]
        z, _, r = ctx.batch_rho1b([(*w.vacua[i], *w.vacua[j]) for i, j in pairs])
    for k, (i, j) in enumerate(pairs):
        zo, ro = kernel_triaxial(w.sp, ham, w.mesh, *w.vacua[i], *w.vacua[j], rho1b=table)
        sc = np.abs(ro).max()
        assert np.abs(r[k] - ro.T).max() <= OBS_TOL * sc


def test_quasiparticle_basis_change_takes_general_path():
    """(U C, V C) with C orthogonal is the same vacuum. A C that mixes proton and neutron
    quasiparticle columns gives U, V with proton-neutron blocks, so the kernels leave the
    species-split form for the general one; the results must not change."""
    from scipy.linalg import expm
    w = make_workload("pf", 2, Mesh(2, 3, 2, 3), seed=515)
    n = w.sp.nlev
    rng = np.random.default_rng(9)
    G = rng.normal(0.0, 0.3, (n, n))
    C = expm(G - G.T)
    mixed = [(U @ C, V @ C) for U, V in w.vacua]
    assert np.abs(mixed[0][0][: n // 2, n // 2:]).max() > 1e-3
    pairs = [(0, 1), (1, 1)]
    with ctx_for(w, w.mesh) as ctx:
        z_ref, _ = ctx.batch([(*w.vacua[i], *w.vacua[j]) for i, j in pairs])
        z_mix, _ = ctx.batch([(*mixed[i], *mixed[j]) for i, j in pairs])
    for k in range(len(pairs)):
        for io in range(19):
            sc = np.abs(z_ref[k][:, io]).max()
            tol = NORM_TOL if io == 0 else OBS_TOL
            assert np.abs(z_mix[k][:, io] - z_ref[k][:, io]).max() <= tol * max(sc, 1e-300), io
