"""The two CPU Monte Carlo oracles agree in distribution: the replay
harness (the product's step functions and Philox streams, compiled for the
host) and the independent FP64 transport (oracle/mc_ref64.c, no shared
code), on eight views of the 65^3 cylinder-with-Ca-inserts workload at
60 keV.  This pins the step functions' physics on the CPU; the GPU test
(test_gpu_mc_independent.py) does the same for the kernels."""
import numpy as np

import oracle
from helpers import block_sum, chi2_binomial_two_sample, chi2_two_sample, golden
from monte_gb300 import abi, phantoms


import pytest


@pytest.mark.parametrize("local", [False, True])
def test_replay_and_fp64_transport_agree(local):
    x = golden("xcom")
    lab, vox, org = phantoms.cylinder_inserts_labels()
    inp = abi.McInputs(lab, vox, org, [-1, 0, 1, 1, 1], [0.0, 1.0, 1.2, 1.5, 1.9],
                       [x["water"], x["ca"]], [60.0])
    g = abi.mc_geom(8, 64, 64, 0.1, 50.0, 100.0, 3.5,
                    flags=abi.MONTE_MC_STALE_SIN_PHI | (abi.MONTE_MC_LOCAL_MAJORANT if local else 0))
    p64, s64, st64 = oracle.mc_ref64(g, inp, 5, 49, (0, 8))
    pr, sr, st = oracle.mc_run(g, inp, abi.mc_request(6, 49, (0, 8), (0, 64), (0, 64)))
    x2, dof, pv = chi2_binomial_two_sample(p64[:8], pr[:8], 49)
    assert pv > 1e-3, (x2, dof, pv)
    x2, dof, pv = chi2_two_sample(block_sum(s64[:8].sum(0), 2), block_sum(sr[:8].sum(0), 2))
    assert pv > 1e-3, (x2, dof, pv)
    for key in ("interactions", "rayleigh", "compton", "photoelectric"):
        a, b = st64[key], st[key]
        assert abs(a - b) < 4 * np.sqrt(a + b), (key, a, b)
