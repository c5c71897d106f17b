"""FDK at the benchmark's full size (360 views of 512 x 384 at 0.8 mm into
325^3 at 0.4 mm, ellipsoid line integrals with noise, seed 1002), where the
CPU oracle cannot run whole in seconds: the properties that do not depend on
the size.

* the oracle's backprojection (the reference's arithmetic, FP64 over FP32
  data) on nine z-slices at the top, middle and bottom of the volume, from
  the same filtered projections: 1e-5 relative RMS;
* the FP64 oracle filter on four views: 1e-5 for the FP32 and the
  tensor-core filter;
* the benchmark's own chain -- the tensor-core filter, the autotuned tile
  shape, the volume -- against the FP64 oracle (FP64 filter of all 360
  views, FP64 backprojection) on those nine slices: 1e-5;
* tile shapes that anchor their row walks every 16 voxels give the same
  volume bit for bit (the anchors sit at the same multiples of 16 in z),
  per-warp and shared-ring kernels alike, whatever the voxels per lane
  (16, 32, 48, 64); the shapes with anchors every 32 voxels agree with one
  another bit for bit; shapes with other anchor spacings (8, 20, 24, 28,
  32) agree with the rest to FP32 rounding;
* the pinned host pipeline (two view ranges) equals the device path bit
  for bit;
* linearity, FDK(a p + b q) = a FDK(p) + b FDK(q): 1e-5 (FP32 rounding)."""
import numpy as np
import pytest
import torch

import oracle
from helpers import rel_rms
from monte_gb300 import abi
from monte_gb300.phantoms import ellipsoid_line_integrals, random_ellipsoids

pytestmark = pytest.mark.gpu

SLABS = [(0, 3), (161, 164), (322, 325)]


@pytest.fixture(scope="module")
def scan():
    g = abi.fdk_geom_recon325()
    proj = ellipsoid_line_integrals(g, random_ellipsoids(1002), noise_sigma=0.01, seed=1002,
                                    device="cuda")
    return g, proj


def _fdk(ctx, g, proj, fmode=abi.MONTE_FILTER_BF16X3):
    f = torch.empty((g.n_views, g.nv, g.nu), device="cuda")
    xy = torch.empty((g.nz, g.ny, g.nx), device="cuda")
    ctx.fdk(g, proj, xy, filtered=f, filter_mode=fmode, bp_mode=abi.MONTE_BP_TILED)
    ctx.synchronize()
    return f, xy


def test_full_size_slices_against_oracle(ctx, scan):
    g, proj = scan
    ctx.fdk_autotune(g)
    f, xy = _fdk(ctx, g, proj, abi.MONTE_FILTER_FP32)
    assert ctx.last_bp_variant() >= 0
    fh, xyh = f.cpu().numpy(), xy.cpu().numpy()
    for z0, z1 in SLABS:
        ref = oracle.fdk_backproject(g, fh, z_range=(z0, z1))
        err = rel_rms(xyh[z0:z1], ref[z0:z1])
        assert err < 1e-5, (z0, err)


def test_full_size_benchmark_chain_against_fp64_oracle(ctx, scan):
    g, proj = scan
    best = ctx.fdk_autotune(g)
    _, xy = _fdk(ctx, g, proj, abi.MONTE_FILTER_BF16X3)
    assert ctx.last_bp_variant() == best
    f64 = oracle.fdk_filter(g, proj.cpu().numpy(), precise=True)
    xyh = xy.cpu().numpy()
    for z0, z1 in SLABS:
        ref = oracle.fdk_backproject(g, f64, z_range=(z0, z1))
        err = rel_rms(xyh[z0:z1], ref[z0:z1])
        assert err < 1e-5, (z0, err)


def test_full_size_filters_against_fp64_oracle(ctx, scan):
    g, proj = scan
    views = [0, 97, 211, 359]
    gs = g.copy()
    gs.n_views = len(views)
    f64 = oracle.fdk_filter(gs, proj[views].cpu().numpy(), precise=True)
    for fmode in (abi.MONTE_FILTER_FP32, abi.MONTE_FILTER_BF16X3):
        f, _ = _fdk(ctx, g, proj, fmode)
        err = rel_rms(f[views].cpu().numpy(), f64)
        assert err < 1e-5, (fmode, err)


def test_full_size_tile_shapes_agree(ctx, scan):
    g, proj = scan
    f, _ = _fdk(ctx, g, proj)
    ref = None
    try:
        ref32 = None
        for variant in (33, 29, 30, 24, 0, 22, 31, 37, 20, 34, 35, 36, 38, 39, 40):
            ctx.set_bp_variant(variant)
            xy = torch.empty((g.nz, g.ny, g.nx), device="cuda")
            ctx.fdk_backproject(g, f, xy, mode=abi.MONTE_BP_TILED)
            ctx.synchronize()
            assert ctx.last_bp_variant() == variant
            if ref is None:
                ref = xy
            if variant in (34, 35):  # anchors every 32 voxels
                if ref32 is None:
                    ref32 = xy
                assert torch.equal(xy, ref32), variant
            if variant in (20, 34, 35, 36, 38, 39, 40):
                err = rel_rms(xy.cpu().numpy(), ref.cpu().numpy())
                assert err < 2e-6, (variant, err)
            else:
                assert torch.equal(xy, ref), variant
    finally:
        ctx.set_bp_variant(-1)


def test_full_size_pinned_pipeline_equals_device_path(ctx, scan):
    g, proj = scan
    ctx.fdk_autotune(g)
    _, xyd = _fdk(ctx, g, proj)
    p = proj.cpu().pin_memory()
    xy = torch.full((g.nz, g.ny, g.nx), float("nan"), pin_memory=True)
    ctx.fdk(g, p, xy, filter_mode=abi.MONTE_FILTER_BF16X3, bp_mode=abi.MONTE_BP_TILED)
    assert ctx.last_host_ranges() == 2
    assert torch.equal(xy, xyd.cpu())


def test_full_size_linearity(ctx, scan):
    g, p = scan
    q = torch.flip(p, dims=[1]).contiguous()  # another scan: the detector mirrored in u
    a, b = 0.75, -1.5
    _, vp = _fdk(ctx, g, p)
    _, vq = _fdk(ctx, g, q)
    _, vpq = _fdk(ctx, g, (a * p + b * q).contiguous())
    lin = (a * vp.double() + b * vq.double()).cpu().numpy()
    err = rel_rms(vpq.cpu().numpy(), lin)
    assert err < 1e-5, err
