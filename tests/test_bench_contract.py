"""bench.py without a GPU: the roofline's algorithmic flop count and the reference arm's
JSON line (the oracle port on the host cores)."""
import json
import os
import subprocess
import sys

import numpy as np

from conftest import ROOT

sys.path.insert(0, ROOT)


def test_flop_count_follows_the_species_split():
    import bench
    from sccm_gb300.synth import config
    wl = config(1, small=True)
    n, G = wl.sp.nlev, wl.mesh.n_gauge
    split = bench.algorithmic_flops_per_point(wl, G)
    # the same vacua with a proton-neutron rotation of the quasiparticle columns: general path
    rng = np.random.default_rng(0)
    g = rng.normal(0.0, 0.1, (n, n))
    from scipy.linalg import expm
    C = expm(g - g.T)
    wl.vacua = [(U @ C, V @ C) for U, V in wl.vacua]
    full = bench.algorithmic_flops_per_point(wl, G)
    dense = (4 / 3 + 8 / 3 + 16 + 12) * n ** 3
    assert abs((full - split) - 0.75 * dense) < 0.15 * dense   # dense part x4, records longer
    assert full > split > 0.25 * dense


def test_reference_arm_prints_its_line():
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "points/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
