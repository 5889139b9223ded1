import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built library")


@pytest.fixture(scope="session")
def ge76():
    """Ge76 / GCN2850 / pf5g9 inputs and the reference's kernel-file values."""
    from sccm_gb300.basis import ModelSpace, j_operators, q2_operators
    from sccm_gb300.formats import mscheme_pairs, onebody_matrix
    d = np.load(os.path.join(GOLDEN, "ge76_fixture.npz"))
    sp = ModelSpace([tuple(int(x) for x in o) for o in d["orbits"]], int(d["nprot"]), int(d["nneut"]),
                    int(d["core"]), int(d["core"]))
    spe = {tuple(int(x) for x in k): float(v) for k, v in zip(d["spe_keys"], d["spe_vals"])}
    recs = mscheme_pairs(sp)
    return dict(sp=sp, e0=float(d["e0"]), t1b=onebody_matrix(sp, spe), recs=recs, vbar=d["vbar"],
                U=d["U"], V=d["V"], gold=d["gold"], betas=d["betas"], jvals=d["jvals"],
                nfom=int(d["nfom"]), nbet=int(d["nbet"]), ncosbet=int(d["ncosbet"]),
                q2=q2_operators(sp), jops=j_operators(sp),
                rho1b_keys=[tuple(int(x) for x in k) for k in d["rho1b_keys"]], rho1b_gold=d["rho1b_gold"])
