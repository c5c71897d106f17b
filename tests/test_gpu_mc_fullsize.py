"""The Monte Carlo at the benchmark's full size: the 325^3 label phantom at
0.8 mm (water, Ca-water bone 1.5-1.9 g/cm^3, air; 20 seeded ellipsoids),
20-80 keV lines weighted (80 - E), a 512 x 384 detector at 0.8 mm, SOD 500,
SDD 1000 mm, 509 histories per pixel (1.0e8 per view).  The CPU replay
cannot run a whole view in seconds, so:

* a window of 32 x 32 central pixels and a window at the detector's edge
  replay bit for bit on the CPU;
* a whole view gives the same int64 tallies from the persistent and the
  plain kernel, and from four pixel bands run one after another (the tallies
  do not depend on the order of the histories or on the split)."""
import numpy as np
import pytest
import torch

import oracle
from helpers import golden
from monte_gb300 import abi, phantoms

pytestmark = pytest.mark.gpu

PER = 509


@pytest.fixture(scope="module")
def workload():
    x = golden("xcom")
    lab, vox, org, dens, mats = phantoms.ellipsoid_labels()
    E = np.arange(20.0, 81.0)

    def make(labels):
        return abi.McInputs(labels, vox, org, mats, dens, [x["water"], x["ca"]], E, 80.0 - E)

    g = abi.mc_geom(360, 512, 384, 0.08, 50.0, 100.0, 14.0, flags=abi.MONTE_MC_STALE_SIN_PHI)
    return g, make(lab), make(torch.from_numpy(lab).cuda())


def _run(ctx, g, inp, req, prim=None, scat=None):
    if prim is None:
        prim = torch.zeros((g.n_views, g.nu, g.nv), dtype=torch.int64, device="cuda")
        scat = torch.zeros_like(prim)
    st = ctx.mc_run(g, inp, req, prim, scat)
    ctx.synchronize()
    return prim, scat, st


@pytest.mark.parametrize("window", [(240, 272, 176, 208), (0, 24, 360, 384)])
def test_full_size_windows_replay_on_cpu(ctx, workload, window):
    g, host, dev = workload
    u0, u1, v0, v1 = window
    req = abi.mc_request(2024, PER, (7, 8), (u0, u1), (v0, v1), abi.MONTE_MC_PERSISTENT)
    prim, scat, st = _run(ctx, g, dev, req)
    p_cpu, s_cpu, st_cpu = oracle.mc_run(g, host, req)
    assert st["histories"] == st_cpu["histories"] == (u1 - u0) * (v1 - v0) * PER
    assert np.array_equal(prim.cpu().numpy(), p_cpu)
    assert np.array_equal(scat.cpu().numpy(), s_cpu)
    assert int(p_cpu.sum()) > 0


def test_full_size_view_kernels_and_splits_agree(ctx, workload):
    g, _, dev = workload
    whole = {}
    for kernel in (abi.MONTE_MC_PERSISTENT, abi.MONTE_MC_PLAIN):
        req = abi.mc_request(99, PER, (123, 124), (0, g.nu), (0, g.nv), kernel)
        prim, scat, st = _run(ctx, g, dev, req)
        assert st["histories"] == g.nu * g.nv * PER
        whole[kernel] = (prim[123].clone(), scat[123].clone())
    p_pers, s_pers = whole[abi.MONTE_MC_PERSISTENT]
    assert torch.equal(p_pers, whole[abi.MONTE_MC_PLAIN][0])
    assert torch.equal(s_pers, whole[abi.MONTE_MC_PLAIN][1])
    assert int(s_pers.sum()) > 0
    prim = torch.zeros((g.n_views, g.nu, g.nv), dtype=torch.int64, device="cuda")
    scat = torch.zeros_like(prim)
    for us in ((0, 100), (100, 256), (256, 300), (300, 512)):
        req = abi.mc_request(99, PER, (123, 124), us, (0, g.nv), abi.MONTE_MC_PERSISTENT)
        _run(ctx, g, dev, req, prim, scat)
    assert torch.equal(prim[123], p_pers) and torch.equal(scat[123], s_pers)
