"""monte_fdk from pinned host memory runs pipelined (view ranges uploaded on
a copy stream, filtered as they land, backprojected into running sums, the
last range stored straight into the pinned volume).  Its results must equal
the device-memory call bit for bit: the filter is per view and every voxel
sums its views in index order however they are split."""
import numpy as np
import pytest
import torch

from inputs import fdk_projections
from monte_gb300 import abi

pytestmark = pytest.mark.gpu


def _device(ctx, g, proj, fmode, zy):
    p = torch.from_numpy(proj).cuda()
    f = torch.empty((g.n_views, g.nv, g.nu), device="cuda")
    xy = torch.empty((g.nz, g.ny, g.nx), device="cuda")
    vzy = torch.empty((g.nx, g.ny, g.nz), device="cuda") if zy else None
    ctx.fdk(g, p, xy, filtered=f, vol_zy=vzy, filter_mode=fmode, bp_mode=abi.MONTE_BP_TILED)
    ctx.synchronize()
    return f.cpu().numpy(), xy.cpu().numpy(), (vzy.cpu().numpy() if zy else None)


def _host(ctx, g, proj, fmode, zy, pinned=True, with_filtered=True):
    def buf(shape):
        # NaN first: every element must be written by the call
        return torch.full(shape, float("nan"), pin_memory=pinned)
    p = torch.from_numpy(proj).pin_memory() if pinned else torch.from_numpy(proj)
    f = buf((g.n_views, g.nv, g.nu)) if with_filtered else None
    xy = buf((g.nz, g.ny, g.nx))
    vzy = buf((g.nx, g.ny, g.nz)) if zy else None
    ctx.fdk(g, p, xy, filtered=f, vol_zy=vzy, filter_mode=fmode, bp_mode=abi.MONTE_BP_TILED)
    return (f.numpy() if with_filtered else None), xy.numpy(), (vzy.numpy() if zy else None)


def _geom(n_views, mask=0):
    g = abi.fdk_geom_recon325(n_views=n_views, nu=128, nv=96, pitch_mm=3.2, n=49, voxel_mm=2.4)
    g.mask_radius = mask
    return g


@pytest.mark.parametrize("n_views,mask", [(360, 0), (90, 20), (5, 0), (1, 0)])
def test_pinned_pipeline_equals_device_path(ctx, n_views, mask):
    g = _geom(n_views, mask)
    proj = fdk_projections(g.n_views, g.nu, g.nv, 7 + n_views)
    fd, xyd, zyd = _device(ctx, g, proj, abi.MONTE_FILTER_FP32, True)
    fh, xyh, zyh = _host(ctx, g, proj, abi.MONTE_FILTER_FP32, True)
    assert ctx.last_host_ranges() == (2 if n_views > 1 else 1)
    assert np.array_equal(fh, fd)
    assert np.array_equal(xyh, xyd)
    assert np.array_equal(zyh, zyd)


def test_pipeline_with_each_tiled_kernel(ctx):
    """the CTA-ring kernel (shape 0) and a per-warp-ring shape (24)"""
    g = _geom(180)
    proj = fdk_projections(g.n_views, g.nu, g.nv, 31)
    try:
        for variant in (0, 24):
            ctx.set_bp_variant(variant)
            _, xyd, _ = _device(ctx, g, proj, abi.MONTE_FILTER_FP32, False)
            assert ctx.last_bp_variant() == variant
            _, xyh, _ = _host(ctx, g, proj, abi.MONTE_FILTER_FP32, False, with_filtered=False)
            assert ctx.last_host_ranges() == 2 and ctx.last_bp_variant() == variant
            assert np.array_equal(xyh, xyd), variant
    finally:
        ctx.set_bp_variant(-1)


def test_pipeline_with_tensor_core_filter(ctx):
    g = abi.fdk_geom_recon325(n_views=90, nu=256, nv=128, pitch_mm=1.6, n=65, voxel_mm=1.6)
    proj = fdk_projections(g.n_views, g.nu, g.nv, 5)
    fd, xyd, _ = _device(ctx, g, proj, abi.MONTE_FILTER_BF16X3, False)
    fh, xyh, _ = _host(ctx, g, proj, abi.MONTE_FILTER_BF16X3, False)
    ctx.check_status()
    assert ctx.last_host_ranges() == 2
    assert np.array_equal(fh, fd) and np.array_equal(xyh, xyd)


@pytest.mark.parametrize("nu", [129, 126])
def test_pipeline_with_odd_detector_widths(ctx, nu):
    """widths whose rows are not a multiple of 16 bytes: each range pads its
    views' rows before its backprojection (the tiles load from the padded
    copy, the exact per-voxel path reads the filtered views themselves)"""
    g = abi.fdk_geom_recon325(n_views=120, nu=nu, nv=96, pitch_mm=3.2, n=49, voxel_mm=2.4)
    proj = fdk_projections(g.n_views, g.nu, g.nv, 40 + nu)
    try:
        for variant in (33, 0):
            ctx.set_bp_variant(variant)
            fd, xyd, zyd = _device(ctx, g, proj, abi.MONTE_FILTER_FP32, True)
            assert ctx.last_bp_variant() == variant
            fh, xyh, zyh = _host(ctx, g, proj, abi.MONTE_FILTER_FP32, True)
            assert ctx.last_host_ranges() == 2 and ctx.last_bp_variant() == variant
            assert np.array_equal(fh, fd) and np.array_equal(xyh, xyd) and np.array_equal(zyh, zyd)
            # the backprojection alone, from pinned filtered projections
            f = torch.from_numpy(fd).pin_memory()
            xy = torch.full((g.nz, g.ny, g.nx), float("nan"), pin_memory=True)
            ctx.fdk_backproject(g, f, xy, mode=abi.MONTE_BP_TILED)
            assert ctx.last_host_ranges() == 2
            assert np.array_equal(xy.numpy(), xyd)
    finally:
        ctx.set_bp_variant(-1)


def test_pageable_buffers_run_unpipelined(ctx):
    g = _geom(24)
    proj = fdk_projections(g.n_views, g.nu, g.nv, 3)
    _, xyd, _ = _device(ctx, g, proj, abi.MONTE_FILTER_FP32, False)
    _, xyh, _ = _host(ctx, g, proj, abi.MONTE_FILTER_FP32, False, pinned=False)
    assert ctx.last_host_ranges() == 0
    assert np.array_equal(xyh, xyd)


def test_pinned_filter_alone_equals_device_path(ctx):
    g = _geom(180)
    proj = fdk_projections(g.n_views, g.nu, g.nv, 12)
    fd, _, _ = _device(ctx, g, proj, abi.MONTE_FILTER_FP32, False)
    p = torch.from_numpy(proj).pin_memory()
    fh = torch.full((g.n_views, g.nv, g.nu), float("nan"), pin_memory=True)
    ctx.fdk_filter(g, p, fh, mode=abi.MONTE_FILTER_FP32)
    assert ctx.last_host_ranges() == 2
    assert np.array_equal(fh.numpy(), fd)


def test_pinned_backprojection_alone_equals_device_path(ctx):
    g = _geom(180, mask=20)
    proj = fdk_projections(g.n_views, g.nu, g.nv, 13)
    fd, xyd, zyd = _device(ctx, g, proj, abi.MONTE_FILTER_FP32, True)
    f = torch.from_numpy(fd).pin_memory()
    xy = torch.full((g.nz, g.ny, g.nx), float("nan"), pin_memory=True)
    zy = torch.full((g.nx, g.ny, g.nz), float("nan"), pin_memory=True)
    ctx.fdk_backproject(g, f, xy, vol_zy=zy, mode=abi.MONTE_BP_TILED)
    assert ctx.last_host_ranges() == 2
    assert np.array_equal(xy.numpy(), xyd) and np.array_equal(zy.numpy(), zyd)
