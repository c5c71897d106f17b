"""The GPU Monte Carlo against an independent FP64 transport (oracle/
mc_ref64.c: written from monte_cu/CBCT_real325im.cu in double, its own
random streams, no code shared with the product) on the CPU-runnable
workload: the 65^3 water cylinder with three Ca-water inserts (1.2, 1.5,
1.9 g/cm^3), SOD 500 mm, SDD 1000 mm, a 64 x 64 detector of 1 mm, 90 views,
2e5 histories per view (49 aimed at each pixel).

Different streams, the same physics: per-pixel tallies must agree in
distribution --
* primary: binomial two-sample chi-square over every pixel of every view
  (each of the 49 histories aimed at a pixel arrives uncollided or not);
* scatter: Poisson two-sample chi-square on 2 x 2 pixel blocks of the
  scatter image summed over the views;
* totals: interactions per history and the Rayleigh / Compton /
  photoelectric split by two-sample tests on the counts.
The 60 keV source runs all 90 views, the 20-80 keV source (lines weighted
80 - E) 24 of them, each with the reference's single majorant and with the
local majorants of MONTE_MC_LOCAL_MAJORANT (the FP64 transport always uses
the single majorant: the two must not be told apart).
"""
import numpy as np
import pytest
import torch
from scipy.stats import chi2, norm

import oracle
from helpers import block_sum, chi2_binomial_two_sample, chi2_two_sample, golden
from monte_gb300 import abi, phantoms

pytestmark = pytest.mark.gpu

PER = 49


def _inputs(device, spectrum):
    x = golden("xcom")
    lab, vox, org = phantoms.cylinder_inserts_labels()
    if device is not None:
        lab = torch.from_numpy(lab).to(device)
    E, W = ([60.0], None) if spectrum == "mono" else (np.arange(20.0, 81.0), 80.0 - np.arange(20.0, 81.0))
    return abi.McInputs(lab, vox, org, [-1, 0, 1, 1, 1], [0.0, 1.0, 1.2, 1.5, 1.9],
                        [x["water"], x["ca"]], E, W)


def _two_counts(a, na, b, nb):
    """p-value of equal rates for Poisson-like totals a / na and b / nb."""
    ra, rb = a / na, b / nb
    se = np.sqrt(a / na ** 2 + b / nb ** 2)
    return float(2 * norm.sf(abs(ra - rb) / se))


@pytest.mark.parametrize("local", [False, True])
@pytest.mark.parametrize("spectrum,n_views", [("mono", 90), ("poly", 24)])
def test_gpu_tallies_match_independent_fp64_transport(ctx, spectrum, n_views, local):
    flags = abi.MONTE_MC_STALE_SIN_PHI | (abi.MONTE_MC_LOCAL_MAJORANT if local else 0)
    g = abi.mc_geom(90, 64, 64, 0.1, 50.0, 100.0, 3.5, flags=flags)
    prim = torch.zeros((g.n_views, g.nu, g.nv), dtype=torch.int64, device="cuda")
    scat = torch.zeros_like(prim)
    st = ctx.mc_run(g, _inputs("cuda", spectrum), abi.mc_request(2024 + local, PER, (0, n_views),
                                                                (0, 64), (0, 64)), prim, scat)
    torch.cuda.synchronize()
    pg, sg = prim.cpu().numpy()[:n_views], scat.cpu().numpy()[:n_views]
    pr, sr, sr_st = oracle.mc_ref64(g, _inputs(None, spectrum), 4202, PER, (0, n_views))
    pr, sr = pr[:n_views], sr[:n_views]
    assert st["histories"] == sr_st["histories"] == n_views * 64 * 64 * PER
    x2, dof, pv = chi2_binomial_two_sample(pg, pr, PER)
    assert pv > 1e-3, ("primary", x2, dof, pv)
    x2, dof, pv = chi2_two_sample(block_sum(sg.sum(0), 2), block_sum(sr.sum(0), 2))
    assert pv > 1e-3, ("scatter", x2, dof, pv)
    n = st["histories"]
    for key in ("interactions", "rayleigh", "compton", "photoelectric", "scatter_counts"):
        pv = _two_counts(st[key], n, sr_st[key], n)
        assert pv > 1e-3, (key, st[key], sr_st[key], pv)
