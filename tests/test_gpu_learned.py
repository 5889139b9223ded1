"""Learned mode on a small sd-shell set (fine 8 x 12 x 8 Euler x 5 x 5 gauge, coarse 4 x 6 x 4).

What the mode guarantees, checked against the full-mesh quadrature:
  * N^J is exact (the norm is computed at every fine point);
  * every pair's energy kernel H^J is within 1 keV in the basis of normalised
    states (the held-out gate sends a pair to the full mesh above 0.5 keV);
and what the trained network gains over the same method without it: a
smaller |N|-weighted H/N error at fresh exactly computed points than the
coarse-mesh interpolation alone (measured: about 10 %; the network generalises
poorly from a few thousand exact points to the rest of the mesh).
"""
import numpy as np
import pytest

from sccm_gb300.basis import Mesh
from sccm_gb300.learned import LearnedConfig, LearnedPNAMP, energy_errors_kev
from sccm_gb300.synth import make_workload

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def trained():
    wl = make_workload("sd", 6, Mesh(8, 12, 8, 5), seed=515)
    cfg = LearnedConfig(coarse=(4, 6, 4), width=128, depth=4, train_euler=192, epochs=40, batch=4096,
                        lr=2e-3, chunk=4, min_heldout=24, heldout=0.04, seed=3)
    lm = LearnedPNAMP(wl, cfg)
    rec = lm.train(wl.pairs[:10])
    yield wl, lm, rec
    lm.close()


def test_training_reduces_loss(trained):
    _, _, rec = trained
    assert rec["loss_last"] < rec["loss_first"] - 0.5


def test_norm_exact_and_energy_kernel_within_1kev(trained):
    wl, lm, _ = trained
    learned = lm.run(wl.pairs)
    exact = lm.exact(wl.pairs)
    for a, b in zip(learned, exact):
        sc = np.abs(b["njkk"]).max()
        assert np.abs(a["njkk"] - b["njkk"]).max() <= 1e-12 * sc
        assert a["fallback"] or a["est_err_keV"] <= lm.cfg.tol_kev
    err = energy_errors_kev(learned, exact)
    assert err["max_kernel_EJ_err_keV"] <= 1.0


def test_hill_wheeler_gate_meets_the_level_gates(trained):
    """run_gcm over the complete pair set: the coarse precheck, the learned run and the gate
    leave the lowest GCM levels and every vacuum's E_J within gcm_kev (1 keV) of the full
    quadrature, whichever way the precheck decides."""
    wl, lm, _ = trained
    nvac = len(wl.vacua)
    res, rec = lm.run_gcm(wl.pairs, nvac)
    exact = lm.exact(wl.pairs)
    err = energy_errors_kev(res, exact, nvac=nvac, pairs=wl.pairs)
    print(rec["decision"], rec["precheck_bound_keV"], err["gcm_levels_err_keV"], err["EJ_per_vacuum_err_keV"])
    assert err["gcm_levels_err_keV"] <= lm.cfg.gcm_kev
    assert err["EJ_per_vacuum_err_keV"] <= lm.cfg.gcm_kev
    for a, b in zip(res, exact):
        assert np.abs(a["njkk"] - b["njkk"]).max() <= 1e-12 * np.abs(b["njkk"]).max()


def test_network_gains_over_interpolation_alone(trained):
    wl, lm, _ = trained
    rms_interp, rms_net = lm.validation_rms(wl.pairs[:10], n_euler=32)   # fresh Euler points
    print(f"H/N error at fresh points: interpolation {rms_interp:.4f} MeV, with the network {rms_net:.4f} MeV")
    assert rms_net < rms_interp


def test_separable_interpolation_kernel_matches_dense_product():
    """pnamp_learned_interp (three 1-D passes) against the dense [P_fine x P_coarse] product of
    the same weights (np.kron), on random coarse per-gauge kernels."""
    import torch
    from sccm_gb300.learned import interp_factors, interp_matrix
    from sccm_gb300.mlp import _ck, _lib, _p
    coarse, fine, G, npairs = Mesh(4, 6, 4, 3), Mesh(8, 12, 8, 3), 9, 3
    wb, wa, wg = interp_factors(coarse, fine)
    I = interp_matrix(coarse, fine)
    Pc, P = I.shape[1], I.shape[0]
    rng = np.random.default_rng(5)
    gc = rng.normal(size=(npairs, Pc, G, 4))
    dev = torch.device("cuda")
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    h = torch.empty((npairs, P, G, 2), dtype=torch.float64, device=dev)
    nn = torch.empty_like(h)
    gcd, wbd, wad, wgd = t(gc), t(wb), t(wa), t(wg)
    _ck(_lib().pnamp_learned_interp(npairs, wb.shape[1], wa.shape[1], wg.shape[1], wb.shape[0], wa.shape[0],
                                    wg.shape[0], G, _p(wbd), _p(wad), _p(wgd), _p(gcd), _p(h), _p(nn),
                                    torch.cuda.current_stream().cuda_stream), "pnamp_learned_interp")
    torch.cuda.synchronize()
    want = np.einsum("fc,pcgq->pfgq", I, gc)
    scale = np.abs(want).max()
    assert np.abs(nn.cpu().numpy() - want[..., 0:2]).max() <= 1e-12 * scale
    assert np.abs(h.cpu().numpy() - want[..., 2:4]).max() <= 1e-12 * scale
