"""The Monte Carlo's physics against expectations that do not come from its
own step code (monte_gb300/csrc/mc_physics.h).

* Interaction mix: at 20, 40, 60 and 80 keV, in water (1.0 g/cm^3) and in
  Ca (1.9 g/cm^3), the kinds of first interactions (max_interactions = 1:
  each history interacts at most once, at the source energy, in one
  material) follow the XCOM ratios of that row -- photoelectric
  photo/total, Rayleigh coh/total, Compton the rest -- as the reference
  selects them (monte_cu/CBCT_real325im.cu:649-660); multinomial chi-square
  with the expected fractions computed here from the XCOM fixture.
* Source spectrum: energies drawn by the kernels' own sampler
  (monte_mc_sample_energies) follow the line weights proportional to
  (80 - E) keV of the 325^3 workload, and the weights of a cumulative
  half-keV table in the reference's format (CBCT_real325.cu:479-486, read
  by monte_spectrum_from_cumulative), by chi-square; lines of zero weight
  are never drawn, and an all-zero table gives the 140 keV fallback only.
"""
import numpy as np
import pytest
import torch
from scipy.stats import chi2

from helpers import golden
from monte_gb300 import abi, lib

pytestmark = pytest.mark.gpu


def _slab_inputs(material, density, energy_kev):
    x = golden("xcom")
    lab = torch.ones((32, 32, 32), dtype=torch.uint8, device="cuda")
    # a 3.2 cm cube of one material, centred on the rotation axis
    return abi.McInputs(lab, 0.1, (-1.6, -1.6, -1.6), [-1, material], [0.0, density],
                        [x["water"], x["ca"]], [energy_kev])


@pytest.mark.parametrize("energy", [20.0, 40.0, 60.0, 80.0])
@pytest.mark.parametrize("material,density", [(0, 1.0), (1, 1.9)])
def test_first_interaction_mix_matches_xcom(ctx, energy, material, density):
    x = golden("xcom")
    tab = (x["water"], x["ca"])[material].astype(np.float64)  # [coh, incoh, photo, total][keV]
    k = int(energy + 0.5)
    coh, photo, tot = tab[0, k], tab[2, k], tab[3, k]
    p = np.array([coh / tot, 1.0 - (photo + coh) / tot, photo / tot])  # Rayleigh, Compton, photo
    g = abi.mc_geom(1, 32, 32, 0.1, 50.0, 100.0, 5.0, max_interactions=1)
    inp = _slab_inputs(material, density, energy)
    prim = torch.zeros((1, 32, 32), dtype=torch.int64, device="cuda")
    scat = torch.zeros_like(prim)
    st = ctx.mc_run(g, inp, abi.mc_request(1000 + k + 7 * material, 1000, (0, 1), (0, 32),
                                           (0, 32)), prim, scat)
    counts = np.array([st["rayleigh"], st["compton"], st["photoelectric"]], np.float64)
    n = counts.sum()
    assert n == st["interactions"] and n > 3e5
    expected = n * p
    m = expected > 5
    x2 = float(np.sum((counts[m] - expected[m]) ** 2 / expected[m]))
    pv = float(chi2.sf(x2, int(m.sum()) - 1))
    assert pv > 1e-3, (energy, material, counts, expected, pv)
    # no history interacted twice
    assert st["histories"] == 1000 * 32 * 32


def _energy_counts(ctx, E, W, n, seed):
    spec = abi.McInputs(np.zeros((1, 1, 1), np.uint8), 1.0, (0, 0, 0), [-1], [0.0],
                        [golden("xcom")["water"]], E, W).spectrum
    out = torch.empty(n, dtype=torch.float32, device="cuda")
    ctx.mc_sample_energies(spec, seed, out)
    torch.cuda.synchronize()
    e = out.cpu().numpy().astype(np.float64)
    idx = np.searchsorted(np.asarray(E, np.float64), e)
    assert np.all(np.asarray(E)[np.clip(idx, 0, len(E) - 1)] == e), "energy not a line"
    return np.bincount(idx, minlength=len(E)).astype(np.float64)


def _chi2_lines(counts, weights):
    w = np.asarray(weights, np.float64)
    assert np.all(counts[w == 0] == 0), "a zero-weight line was drawn"
    expected = counts.sum() * w / w.sum()
    m = expected > 5
    x2 = float(np.sum((counts[m] - expected[m]) ** 2 / expected[m]))
    return float(chi2.sf(x2, int(m.sum()) - 1))


def test_source_energies_follow_the_line_weights(ctx):
    E = np.arange(20.0, 81.0)
    W = 80.0 - E
    counts = _energy_counts(ctx, E, W, 4_000_000, 11)
    pv = _chi2_lines(counts, W)
    assert pv > 1e-3, pv


def test_source_energies_from_a_cumulative_table(ctx):
    # a 250-bin half-keV table: bins 20-80 keV weighted (80 - E), as the
    # reference's readxray tables lay them out
    e_bins = 0.5 * np.arange(1, 251)
    w_bins = np.where((e_bins >= 20) & (e_bins <= 80), 80.0 - e_bins, 0.0)
    cum = np.concatenate([[0.0], np.cumsum(w_bins) / w_bins.sum()]).astype(np.float32)
    E, W = lib.spectrum_from_cumulative(cum, 0.5, 140.0)
    assert len(E) == 251 and E[-1] == 140.0
    # the weights are the table's increments (the fallback takes what
    # rounding leaves of 1)
    assert np.allclose(W[:250], np.diff(cum.astype(np.float64)), atol=1e-12)
    counts = _energy_counts(ctx, E, W, 4_000_000, 12)
    pv = _chi2_lines(counts, np.diff(cum.astype(np.float64)).tolist() + [W[-1]])
    assert pv > 1e-3, pv
    # the reference's reader leaves its table at zero: 140 keV only
    E0, W0 = lib.spectrum_from_cumulative(np.zeros(251, np.float32), 0.5, 140.0)
    counts0 = _energy_counts(ctx, E0, W0, 100_000, 13)
    assert counts0[-1] == 100_000
