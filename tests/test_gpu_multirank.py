"""The multi-GPU partition through the library: two ranks as two processes
on the one GPU, exchanging over gloo on the host.  Their kernels never wait
on one another; every exchange happens between launches, on CPU tensors.

* Monte Carlo: each rank runs monte_mc_run on its share of the views; the
  all-reduced int64 tallies equal one process running every view, bit for
  bit (every history owns its random stream).
* FDK: each rank filters its share of the views (monte_fdk_filter), the
  filtered projections are all-gathered, each rank backprojects its z-slab
  (monte_fdk_backproject with a slab geometry) and the slabs are
  all-gathered.  The filtered projections equal one process's bit for bit;
  the slabs, split at a multiple of the tile's z-group, equal its volume.
"""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from monte_gb300 import abi, shard

pytestmark = pytest.mark.gpu

TILE = 39  # 56 voxels per lane, anchors every 28: the slabs below split at 56


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _mc_setup(device):
    from helpers import golden
    from monte_gb300 import phantoms
    x = golden("xcom")
    lab, vox, org = phantoms.cylinder_inserts_labels()
    if device is not None:
        lab = torch.from_numpy(lab).to(device)
    inp = abi.McInputs(lab, vox, org, [-1, 0, 1, 1, 1], [0.0, 1.0, 1.2, 1.5, 1.9],
                       [x["water"], x["ca"]], [60.0])
    g = abi.mc_geom(90, 64, 64, 0.1, 50.0, 100.0, 3.5,
                    flags=abi.MONTE_MC_STALE_SIN_PHI | abi.MONTE_MC_LOCAL_MAJORANT)
    req = abi.mc_request(777, 4, (20, 27), (0, 64), (0, 64))
    return g, inp, req


def _fdk_setup():
    from inputs import fdk_projections
    g = abi.fdk_geom_recon325(n_views=90, nu=256, nv=128, pitch_mm=1.6, n=112, voxel_mm=0.8)
    return g, fdk_projections(g.n_views, g.nu, g.nv, 23)


def _worker(rank, world, port, out_dir):
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (repo, os.path.join(repo, "tests"), os.path.join(repo, "tests", "golden")):
        sys.path.insert(0, p)
    import torch.distributed as dist
    from monte_gb300.lib import Context
    from test_multirank import all_gather_rows
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    torch.cuda.set_device(0)
    ctx = Context(0, stream=torch.cuda.current_stream())
    try:
        # Monte Carlo: this rank's views, then the sum-reduce of the tallies
        g, inp, req = _mc_setup("cuda")
        mine = shard.mc_request_for_rank(req, g.n_views, rank, world)
        prim = torch.zeros((g.n_views, g.nu, g.nv), dtype=torch.int64, device="cuda")
        scat = torch.zeros_like(prim)
        ctx.mc_run(g, inp, mine, prim, scat)
        ctx.synchronize()
        tp, ts = prim.cpu(), scat.cpu()
        dist.all_reduce(tp)
        dist.all_reduce(ts)
        # FDK: this rank's views filtered, all-gathered; its z-slab, all-gathered
        fg, proj = _fdk_setup()
        v0, v1 = shard.fdk_views_for_rank(fg.n_views, rank, world)
        p = torch.from_numpy(proj[v0:v1]).cuda()
        f = torch.empty((v1 - v0, fg.nv, fg.nu), device="cuda")
        ctx.fdk_filter(shard.fdk_geom_views(fg, v0, v1), p, f, abi.MONTE_FILTER_BF16X3)
        ctx.synchronize()
        filt = all_gather_rows(f.cpu(), fg.n_views, world)
        z0, z1 = shard.fdk_zslab_for_rank(fg.nz, rank, world)
        sg = shard.fdk_geom_zslab(fg, z0, z1)
        slab = torch.empty((z1 - z0, fg.ny, fg.nx), device="cuda")
        ctx.set_bp_variant(TILE)
        ctx.fdk_backproject(sg, filt.cuda(), slab, mode=abi.MONTE_BP_TILED)
        ctx.synchronize()
        assert ctx.last_bp_variant() == TILE
        ctx.check_status()
        vol = all_gather_rows(slab.cpu(), fg.nz, world)
        if rank == 0:
            np.save(os.path.join(out_dir, "prim.npy"), tp.numpy())
            np.save(os.path.join(out_dir, "scat.npy"), ts.numpy())
            np.save(os.path.join(out_dir, "filt.npy"), filt.numpy())
            np.save(os.path.join(out_dir, "vol.npy"), vol.numpy())
        dist.barrier()
    finally:
        ctx.close()
        dist.destroy_process_group()


def test_two_ranks_on_the_gpu_reproduce_one(ctx, tmp_path):
    fg, proj = _fdk_setup()
    assert shard.fdk_zslab_for_rank(fg.nz, 0, 2) == (0, 56)
    ctx_spawn = mp.get_context("spawn")
    port = _free_port()
    procs = [ctx_spawn.Process(target=_worker, args=(r, 2, port, str(tmp_path)))
             for r in range(2)]
    for pr in procs:
        pr.start()
    for pr in procs:
        pr.join(timeout=600)
    assert all(pr.exitcode == 0 for pr in procs), [pr.exitcode for pr in procs]

    g, inp, req = _mc_setup("cuda")
    prim = torch.zeros((g.n_views, g.nu, g.nv), dtype=torch.int64, device="cuda")
    scat = torch.zeros_like(prim)
    ctx.mc_run(g, inp, req, prim, scat)
    ctx.synchronize()
    assert prim.sum().item() > 0 and scat.sum().item() > 0
    assert np.array_equal(np.load(tmp_path / "prim.npy"), prim.cpu().numpy())
    assert np.array_equal(np.load(tmp_path / "scat.npy"), scat.cpu().numpy())

    p = torch.from_numpy(proj).cuda()
    f = torch.empty((fg.n_views, fg.nv, fg.nu), device="cuda")
    ctx.fdk_filter(fg, p, f, abi.MONTE_FILTER_BF16X3)
    vol = torch.empty((fg.nz, fg.ny, fg.nx), device="cuda")
    try:
        ctx.set_bp_variant(TILE)
        ctx.fdk_backproject(fg, f, vol, mode=abi.MONTE_BP_TILED)
        ctx.synchronize()
        assert ctx.last_bp_variant() == TILE
    finally:
        ctx.set_bp_variant(-1)
    assert np.array_equal(np.load(tmp_path / "filt.npy"), f.cpu().numpy())
    got, want = np.load(tmp_path / "vol.npy"), vol.cpu().numpy()
    assert np.abs(want).max() > 0
    # the slab geometry moves the origin: its float-pair z terms may round
    # differently in the last bit from the whole volume's
    np.testing.assert_allclose(got, want, rtol=0, atol=1e-6 * np.abs(want).max())
