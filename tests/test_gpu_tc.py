"""Tensor-core forms vs the oracle: the two-body contraction of HFB_Energy_COMPLEX
(Codes/PNAMP/PNAMP_Energy_OpenMP.f90:31-90) as block GEMMs on tcgen05 with bf16 inputs and
FP32 accumulation (sccm_gb300/csrc/contract_tc.cu), the rest of the point in the double-float
form.

Tolerances (relative to max |column| over the mesh):
  * norm kernel N(Omega): 1e-10, the other observables except the energy: 1e-9 (unchanged
    from the double-float form: the contraction touches only the energy);
  * energy kernel H(Omega) = ZRES(:, 7): 1e-4 for BF16x3 (two bf16 terms per value, three
    products; ~4e-6 of the two-body energy per point when the arithmetic is simulated on
    CPU), 1e-6 for BF16x6 (three terms, six products; ~5e-8 simulated).
"""
import numpy as np
import pytest

from sccm_gb300.basis import NOBS, Mesh
from sccm_gb300.pnamp import ST_CONTRACTION, ST_PIVOT_UNDERFLOW, PnampContext, PnampError
from sccm_gb300.synth import make_workload, ti48_workload
from oracle.pnamp_oracle import Hamiltonian, kernel_triaxial

pytestmark = pytest.mark.gpu

TOL_H = {"tc3": 1e-4, "tc6": 1e-6}
TC_FORMS = ["tc3", "tc6"]


def ctx_for(w, form, mesh=None):
    return PnampContext(w.sp, w.e0, w.t1b, w.recs, w.vbar, mesh or w.mesh, q2=w.q2, form=form)


def oracle(w, i, j, mesh=None):
    ham = Hamiltonian(w.e0, w.t1b, w.recs, w.vbar, w.q2, w.jops)
    return kernel_triaxial(w.sp, ham, mesh or w.mesh, *w.vacua[i], *w.vacua[j])


def assert_tc_close(z, ref, form):
    for io in range(NOBS):
        scale = np.abs(ref[:, io]).max()
        if scale == 0.0:
            assert np.abs(z[:, io]).max() == 0.0, io
            continue
        tol = 1e-10 if io == 0 else (TOL_H[form] if io == 6 else 1e-9)
        e = np.abs(z[:, io] - ref[:, io]).max() / scale
        assert e <= tol, f"observable {io + 1}: rel err {e:.2e} (tol {tol:.0e})"


@pytest.fixture(scope="module")
def sd():
    return make_workload("sd", 2, Mesh(3, 4, 3, 3), seed=101, deformed=False)


@pytest.fixture(scope="module")
def pf():
    return make_workload("pf", 2, Mesh(2, 3, 2, 3), seed=202)


@pytest.fixture(scope="module")
def pfmix():
    return make_workload("pf", 2, Mesh(2, 3, 2, 3), seed=404, pn_mix=True)


@pytest.mark.parametrize("form", TC_FORMS)
def test_sd_pair_matches_oracle(sd, form):
    with ctx_for(sd, form) as ctx:
        r = ctx.pair(*sd.vacua[0], *sd.vacua[1])
    assert (r.status & ~ST_PIVOT_UNDERFLOW).max() == 0
    assert_tc_close(r.zres, oracle(sd, 0, 1), form)


@pytest.mark.parametrize("form", TC_FORMS)
def test_pf_split_and_general_pairs_match_oracle(pf, pfmix, form):
    for w in (pf, pfmix):
        with ctx_for(w, form) as ctx:
            z, st = ctx.batch([(*w.vacua[0], *w.vacua[1]), (*w.vacua[1], *w.vacua[1])])
        assert not (st & ST_CONTRACTION).any()
        assert_tc_close(z[0], oracle(w, 0, 1), form)
        assert_tc_close(z[1], oracle(w, 1, 1), form)


@pytest.mark.parametrize("form", TC_FORMS)
def test_sdpf_n64_matches_oracle(form):
    """n = 64: ph groups larger than one UMMA N chunk (up to 324 entries) are split into
    chunks that share their K range."""
    w = make_workload("sdpf", 2, Mesh(1, 2, 1, 2), seed=303)
    with ctx_for(w, form) as ctx:
        r = ctx.pair(*w.vacua[0], *w.vacua[1])
    assert_tc_close(r.zres, oracle(w, 0, 1), form)


@pytest.mark.parametrize("form", TC_FORMS)
def test_ti48_kb3g_pair_matches_oracle(form):
    """The reference's own interaction (KB3G m-scheme file) and vacua."""
    w = ti48_workload(Mesh(2, 3, 2, 5))
    with ctx_for(w, form) as ctx:
        r = ctx.pair(*w.vacua[3], *w.vacua[5])
    assert_tc_close(r.zres, oracle(w, 3, 5), form)


@pytest.mark.parametrize("form", TC_FORMS)
def test_tc_forms_agree_with_double_float_on_a_batch(pf, form):
    """Several pairs in one launch (tiles of 64 points straddle Euler and pair boundaries)."""
    pairs = [(*pf.vacua[i], *pf.vacua[j]) for i, j in ((0, 1), (1, 0), (0, 0), (1, 1))]
    with ctx_for(pf, "df64") as ctx:
        zd, _ = ctx.batch(pairs)
        ctx.set_form(form)
        zt, st = ctx.batch(pairs)
        zt1 = ctx.pair(*pairs[2][:2], *pairs[2][2:]).zres
    assert not (st & ST_CONTRACTION).any()
    for k in range(len(pairs)):
        assert_tc_close(zt[k], zd[k], form)
    assert np.allclose(zt[2], zt1, rtol=0, atol=1e-12 * np.abs(zt1).max())


def test_items_path_matches_full_mesh(pf):
    """pnamp_batch_items_device under a tensor-core form: listed Euler points only, same values."""
    import torch
    w = pf
    dev = torch.device("cuda")
    with ctx_for(w, "tc6") as ctx:
        full = ctx.pair(*w.vacua[0], *w.vacua[1]).zres
        P = ctx.n_euler
        idx = [0, 3, P - 1]
        uv = torch.from_numpy(PnampContext.pack_pairs([(*w.vacua[0], *w.vacua[1])])).to(dev)
        items = torch.tensor([[0, e] for e in idx] + [[5, 0], [0, P + 7]], dtype=torch.int32, device=dev)
        z = torch.zeros((1, NOBS, P, 2), dtype=torch.float64, device=dev)
        st = torch.zeros((1, P), dtype=torch.int32, device=dev)
        ctx.batch_items_device(1, uv.data_ptr(), items.shape[0], items.data_ptr(), z.data_ptr(), st.data_ptr(), 0,
                               torch.cuda.current_stream().cuda_stream)
        torch.cuda.synchronize()
        with pytest.raises(PnampError):   # per-gauge output is not served by the tensor-core forms
            g = torch.zeros((1, P, w.mesh.n_gauge, 4), dtype=torch.float64, device=dev)
            ctx.batch_items_device(1, uv.data_ptr(), 1, items.data_ptr(), z.data_ptr(), st.data_ptr(),
                                   g.data_ptr(), torch.cuda.current_stream().cuda_stream)
    zz = z.cpu().numpy()[0]
    zi = (zz[..., 0] + 1j * zz[..., 1]).T
    assert np.allclose(zi[idx], full[idx], rtol=0, atol=1e-12 * np.abs(full).max())
    others = np.setdiff1d(np.arange(P), idx)
    assert np.abs(zi[others]).max() == 0.0


def test_form_switches_on_one_context(pf):
    """BF16x3 -> BF16x6 -> BF16x3 -> double-float on one context: the staging grows to the
    third bf16 term when BF16x6 follows BF16x3, and each form gives its own result."""
    pairs = [(*pf.vacua[0], *pf.vacua[1])]
    got = {}
    with ctx_for(pf, "tc3") as ctx:
        for form in ("tc3", "tc6", "tc3", "df64"):
            ctx.set_form(form)
            z, st = ctx.batch(pairs)
            assert not (st & ST_CONTRACTION).any()
            got.setdefault(form, []).append(z[0])
    ref = got["df64"][0]
    for form in ("tc3", "tc6"):
        for z in got[form]:
            assert_tc_close(z, ref, form)
    assert np.array_equal(got["tc3"][0], got["tc3"][1])
