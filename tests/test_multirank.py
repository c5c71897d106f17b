"""The multi-GPU contract on CPU ranks (gloo, world size 2): Monte Carlo
ranks split the views and sum their int64 tallies; FDK ranks filter their
share of the views, all-gather the filtered projections and backproject
their z-slab of the volume.  Both reproduce the single-rank result bit for
bit.  The per-rank work here runs on the CPU oracle;
tests/test_gpu_multirank.py runs the same partition through the library
on the GPU."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from monte_gb300 import abi, phantoms, shard


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _mc_setup():
    from helpers import golden
    x = golden("xcom")
    lab, vox, org = phantoms.cylinder_inserts_labels()
    inp = abi.McInputs(lab, vox, org, [-1, 0, 1, 1, 1], [0.0, 1.0, 1.2, 1.5, 1.9],
                       [x["water"], x["ca"]], [60.0])
    g = abi.mc_geom(90, 64, 64, 0.1, 50.0, 100.0, 3.5, flags=abi.MONTE_MC_STALE_SIN_PHI)
    req = abi.mc_request(2024, 4, (0, 6), (0, 64), (0, 64))
    return g, inp, req


def all_gather_rows(mine, n, world):
    """All ranks' row ranges split_range(n, world, r) of an array, gathered
    in rank order (padded to the largest share for the collective)."""
    spans = [shard.split_range(n, world, r) for r in range(world)]
    rows = max(e - b for b, e in spans)
    pad = torch.zeros((rows,) + tuple(mine.shape[1:]), dtype=mine.dtype)
    pad[:mine.shape[0]] = mine
    parts = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad)
    return torch.cat([p[:e - b] for p, (b, e) in zip(parts, spans)])


def _worker(rank, world, port, out_dir):
    import sys
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (repo, os.path.join(repo, "tests"), os.path.join(repo, "tests", "golden")):
        sys.path.insert(0, p)
    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # Monte Carlo: this rank's views, then the sum-reduce of the tallies
    g, inp, req = _mc_setup()
    mine = shard.mc_request_for_rank(req, g.n_views, rank, world)
    prim, scat, _ = oracle.mc_run(g, inp, mine)
    tp, ts = torch.from_numpy(prim), torch.from_numpy(scat)
    dist.all_reduce(tp)
    dist.all_reduce(ts)
    # FDK: this rank's views filtered, the filtered projections all-gathered,
    # then this rank's z-slab, and an all-gather of the slabs
    from inputs import fdk_projections
    fg = abi.fdk_geom_recon325(n_views=31, nu=48, nv=32, pitch_mm=8.0, n=21, voxel_mm=4.0)
    proj = fdk_projections(fg.n_views, fg.nu, fg.nv, 17)
    v0, v1 = shard.fdk_views_for_rank(fg.n_views, rank, world)
    mine = oracle.fdk_filter(shard.fdk_geom_views(fg, v0, v1), proj[v0:v1])
    filt = all_gather_rows(torch.from_numpy(mine), fg.n_views, world).numpy()
    z0, z1 = shard.fdk_zslab_for_rank(fg.nz, rank, world)
    vol = torch.from_numpy(oracle.fdk_backproject(fg, filt, z_range=(z0, z1)))
    parts = [torch.zeros_like(vol) for _ in range(world)]
    dist.all_gather(parts, vol)
    full = sum(parts)
    if rank == 0:
        np.save(os.path.join(out_dir, "prim.npy"), tp.numpy())
        np.save(os.path.join(out_dir, "scat.npy"), ts.numpy())
        np.save(os.path.join(out_dir, "vol.npy"), full.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_reproduce_one(tmp_path):
    import oracle
    from inputs import fdk_projections
    mp.spawn(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2, join=True)
    g, inp, req = _mc_setup()
    prim, scat, _ = oracle.mc_run(g, inp, req)
    assert np.array_equal(np.load(tmp_path / "prim.npy"), prim)
    assert np.array_equal(np.load(tmp_path / "scat.npy"), scat)
    fg = abi.fdk_geom_recon325(n_views=31, nu=48, nv=32, pitch_mm=8.0, n=21, voxel_mm=4.0)
    proj = fdk_projections(fg.n_views, fg.nu, fg.nv, 17)
    vol = oracle.fdk_backproject(fg, oracle.fdk_filter(fg, proj))
    assert np.array_equal(np.load(tmp_path / "vol.npy"), vol)


def test_geometry_shards_describe_the_same_reconstruction():
    """A view share filters like those views of the whole scan, and a z-slab
    geometry backprojects like those slices of the whole volume."""
    import oracle
    from inputs import fdk_projections
    fg = abi.fdk_geom_recon325(n_views=24, nu=48, nv=32, pitch_mm=8.0, n=21, voxel_mm=4.0)
    proj = fdk_projections(fg.n_views, fg.nu, fg.nv, 5)
    filt = oracle.fdk_filter(fg, proj)
    assert np.array_equal(oracle.fdk_filter(shard.fdk_geom_views(fg, 7, 19), proj[7:19]),
                          filt[7:19])
    vol = oracle.fdk_backproject(fg, filt)
    for b, e in ((0, 8), (8, 21), (5, 6)):
        slab = oracle.fdk_backproject(shard.fdk_geom_zslab(fg, b, e), filt)
        assert slab.shape == (e - b, fg.ny, fg.nx)
        np.testing.assert_allclose(slab, vol[b:e], rtol=0, atol=1e-6 * np.abs(vol).max())
    masked = abi.fdk_geom_reference65()
    with pytest.raises(ValueError):
        shard.fdk_geom_zslab(masked, 0, 10)
    with pytest.raises(ValueError):
        shard.fdk_geom_zslab(fg, 3, 3)


def test_split_range_covers_exactly():
    for n in (0, 1, 7, 325, 360):
        for parts in (1, 2, 3, 8):
            spans = [shard.split_range(n, parts, i) for i in range(parts)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
    with pytest.raises(ValueError):
        shard.split_range(10, 2, 2)
