"""The C++/OpenMP CPU baseline (oracle/cpu/pnamp_cpu.cpp) against the numpy oracle (no GPU).

bench.py times this restatement as the CPU baseline, so it must compute what the oracle
computes: both forms ("as implemented", the reference's per-point ZGEMM/LU sequence, and
"minimal", the GPU library's algebra) within 1e-12 of the oracle on every observable, on the
species-split, the proton-neutron-mixing and the sd paths, on all threads and on one.
"""
import numpy as np
import pytest

from sccm_gb300.basis import NOBS, Mesh
from sccm_gb300.synth import make_workload
from oracle import cpu_baseline as cb
from oracle.pnamp_oracle import Hamiltonian, kernel_triaxial

CASES = {
    "sd": lambda: make_workload("sd", 2, Mesh(3, 4, 3, 3), seed=101, deformed=False),
    "pf": lambda: make_workload("pf", 2, Mesh(2, 3, 2, 3), seed=202),
    "pf-pnmix": lambda: make_workload("pf", 2, Mesh(2, 3, 2, 3), seed=404, pn_mix=True),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("form", ["as_implemented", "minimal"])
def test_cpu_baseline_matches_oracle(case, form):
    w = CASES[case]()
    ham = Hamiltonian(w.e0, w.t1b, w.recs, w.vbar, w.q2, w.jops)
    ref = kernel_triaxial(w.sp, ham, w.mesh, *w.vacua[0], *w.vacua[1])
    z = cb.zres(w, w.mesh, 0, 1, form)
    for io in range(NOBS):
        scale = np.abs(ref[:, io]).max()
        if scale == 0.0:
            assert np.abs(z[:, io]).max() == 0.0
            continue
        assert np.abs(z[:, io] - ref[:, io]).max() <= 1e-12 * scale, (case, form, io)


def test_cpu_baseline_thread_count_and_subset_do_not_change_results():
    w = CASES["pf"]()
    full = cb.zres(w, w.mesh, 0, 1, "minimal")
    one = cb.zres(w, w.mesh, 0, 1, "minimal", threads=1)
    assert np.array_equal(full, one)
    sub = cb.zres(w, w.mesh, 0, 1, "minimal", euler=[1, 5])
    assert np.array_equal(sub[[1, 5]], full[[1, 5]])
    assert np.abs(np.delete(sub, [1, 5], axis=0)).max() == 0.0
