"""Batched scans through monte_batch_* (C ABI).

A batch of scans of uneven phantom size, view count and detector shape runs
as one persistent Monte Carlo launch plus per-scan FDK captured in a CUDA
graph (FUSED), or scan by scan with the plain kernels (SEQUENTIAL).  Checks:

* every scan's int64 tallies are bit-equal to monte_mc_run of that scan
  alone (same history streams: job = the scan's index), in both forms;
* the -log map is the reference post-processing of those tallies
  (monte_cu/CBCT_real325im.cu:261-294);
* every reconstruction equals, bit for bit, monte_fdk of the same map with
  the same filter and backprojector (the plan adds no arithmetic of its
  own), and is within 1e-5 relative RMS of the FP64 oracle FDK of that map;
* replaying the graph reproduces the run bit for bit.

These maps are Monte Carlo noise on a 0.3-0.8 mm detector grid, so any
error of the backprojector's detector coordinates becomes a value error one
for one: the coordinates come from exact float pairs (BpView in fdk.cuh),
which a walk in plain float arithmetic missed here by up to three-fold.
"""
import numpy as np
import pytest
import torch

import oracle
from helpers import golden, rel_rms
from monte_gb300 import abi, batchscan
from monte_gb300.lib import MonteError

pytestmark = pytest.mark.gpu


def _specs():
    sp = batchscan.specs(seed=77, n_jobs=4, side=(17, 41), views=(8, 24), nu_steps=(1, 2),
                         nv_steps=(1, 1), hist_per_view=(2e5, 6e5))
    # a detector outside the tensor-core filter's tile (FP32 filter fallback)
    sp[2]["nu"], sp[2]["nv"] = 96, 80
    sp[2]["hpp"] = max(1, int(round(sp[2]["hist_per_view"] / (96 * 80))))
    return sp


@pytest.fixture(scope="module")
def scans():
    x = golden("xcom")
    return batchscan.Batch(_specs(), x["water"], x["ca"])


def _snapshot(b):
    torch.cuda.synchronize()
    return ([p.cpu().numpy() for p in b.primary], [s.cpu().numpy() for s in b.scatter],
            [m.cpu().numpy() for m in b.maps], [v.cpu().numpy() for v in b.vols])


def _single_runs(ctx, b):
    out = []
    for j, (job, inp) in enumerate(zip(b.jobs, b.inputs)):
        g = job.mc
        prim = torch.zeros((g.n_views, g.nu, g.nv), dtype=torch.int64, device="cuda")
        scat = torch.zeros_like(prim)
        req = abi.mc_request(job.seed, job.histories_per_pixel, (0, g.n_views), (0, g.nu),
                             (0, g.nv), job=j)
        ctx.mc_run(g, inp, req, prim, scat)
        ctx.synchronize()
        out.append((prim.cpu().numpy(), scat.cpu().numpy()))
    return out


def _check_fdk(ctx, b, maps, vols, mode, variants):
    for j, job in enumerate(b.jobs):
        g = job.fdk
        # the same map through the single-scan entry point, same kernels
        if mode == abi.MONTE_BATCH_FUSED:
            fm = (abi.MONTE_FILTER_BF16X3 if g.nu % 64 == 0 and g.nv % 128 == 0
                  else abi.MONTE_FILTER_FP32)
            bm = abi.MONTE_BP_TILED if variants[j] >= 0 else abi.MONTE_BP_PLAIN
            ctx.set_bp_variant(max(variants[j], -1))
        else:
            fm, bm = abi.MONTE_FILTER_FP32, abi.MONTE_BP_PLAIN
        vol = torch.zeros((g.nz, g.ny, g.nx), device="cuda")
        ctx.fdk(g, torch.from_numpy(maps[j]).cuda(), vol, filter_mode=fm, bp_mode=bm)
        ctx.check_status()
        assert np.array_equal(vol.cpu().numpy(), vols[j]), j
        f64 = oracle.fdk_filter(g, maps[j], precise=True)
        v64 = oracle.fdk_backproject(g, f64)
        err = rel_rms(vols[j], v64)
        assert err < 1e-5, (j, err)
    ctx.set_bp_variant(-1)


@pytest.mark.parametrize("mode", [abi.MONTE_BATCH_FUSED, abi.MONTE_BATCH_SEQUENTIAL])
def test_batch_matches_single_scans_and_oracle(ctx, scans, mode):
    single = _single_runs(ctx, scans)
    with ctx.batch(scans.xcom, scans.jobs, mode=mode) as plan:
        plan.run()
        st = plan.stats()
        prim, scat, maps, vols = _snapshot(scans)
        ctx.check_status()
        variants = [plan.bp_variant(j) for j in range(len(scans.jobs))]
    assert st["histories"] == scans.histories()
    for j, s in enumerate(scans.specs):
        assert np.array_equal(prim[j], single[j][0]), j
        assert np.array_equal(scat[j], single[j][1]), j
        n = np.clip(prim[j] + scat[j], 1, s["hpp"]).astype(np.float64)
        ref = (-np.log(n) + np.float64(np.float32(np.log(s["hpp"])))).astype(np.float32)
        assert np.array_equal(maps[j], ref), j
    _check_fdk(ctx, scans, maps, vols, mode, variants)


def test_batch_with_local_majorants_matches_single_scans(ctx, scans):
    """MONTE_MC_LOCAL_MAJORANT in a fused plan: each job's tables and class
    grid are built at creation; the tallies equal monte_mc_run of the job
    alone with the same flag, bit for bit."""
    saved = [j.mc.flags for j in scans.jobs]
    try:
        for j in scans.jobs:
            j.mc.flags |= abi.MONTE_MC_LOCAL_MAJORANT
        single = _single_runs(ctx, scans)
        with ctx.batch(scans.xcom, scans.jobs, mode=abi.MONTE_BATCH_FUSED) as plan:
            plan.run()
            st = plan.stats()
            prim, scat, _, _ = _snapshot(scans)
            ctx.check_status()
        assert st["majorant_legs"] > 0
        for j in range(len(scans.jobs)):
            assert np.array_equal(prim[j], single[j][0]), j
            assert np.array_equal(scat[j], single[j][1]), j
    finally:
        for j, f in zip(scans.jobs, saved):
            j.mc.flags = f


def test_graph_replay_is_bit_exact(ctx, scans):
    with ctx.batch(scans.xcom, scans.jobs, options=abi.MONTE_BATCH_AUTOTUNE) as plan:
        variants = [plan.bp_variant(j) for j in range(len(scans.jobs))]
        assert all(v >= -1 for v in variants)
        plan.run()
        first = _snapshot(scans)
        for v in scans.vols:
            v.fill_(0.0)
        plan.run()
        second = _snapshot(scans)
        ctx.check_status()
    for a, b in zip(first, second):
        for x, y in zip(a, b):
            assert np.array_equal(x, y)
    _check_fdk(ctx, scans, first[2], first[3], abi.MONTE_BATCH_FUSED, variants)


def test_batch_rejects_bad_jobs(ctx, scans):
    bad = abi.BatchJob.from_buffer_copy(scans.jobs[0])
    bad.fdk.nu = bad.mc.nu + 1
    with pytest.raises(MonteError) as e:
        ctx.batch(scans.xcom, [scans.jobs[1], bad])
    assert e.value.code == abi.MONTE_EINVAL
    assert "job 1" in str(e.value)
    bad = abi.BatchJob.from_buffer_copy(scans.jobs[0])
    bad.histories_per_pixel = 0
    with pytest.raises(MonteError):
        ctx.batch(scans.xcom, [bad])
    with pytest.raises(MonteError):
        ctx.batch(scans.xcom, scans.jobs, mode=7)
