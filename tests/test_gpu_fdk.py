"""FDK on the GPU through the C ABI against the reference programs' output
(golden fixtures) and the FP64 oracle.  Tolerance: 1e-5 relative RMS for
the filtered projections and the volume (FP32 accumulation over up to 512
taps and 360 views)."""
import numpy as np
import pytest
import torch

import oracle
from helpers import golden, past_end_voxels, rel_rms
from inputs import fdk_projections
from monte_gb300 import abi
from monte_gb300.lib import MonteError

pytestmark = pytest.mark.gpu

FILTERS = [abi.MONTE_FILTER_FP32, abi.MONTE_FILTER_BF16X3]
BPS = [abi.MONTE_BP_PLAIN, abi.MONTE_BP_TILED]


def _run(ctx, g, proj, filter_mode=abi.MONTE_FILTER_FP32, bp_mode=abi.MONTE_BP_PLAIN, zy=False):
    p = torch.from_numpy(proj).cuda()
    f = torch.empty((g.n_views, g.nv, g.nu), dtype=torch.float32, device="cuda")
    xy = torch.empty((g.nz, g.ny, g.nx), dtype=torch.float32, device="cuda")
    vzy = torch.empty((g.nx, g.ny, g.nz), dtype=torch.float32, device="cuda") if zy else None
    ctx.fdk(g, p, xy, filtered=f, vol_zy=vzy, filter_mode=filter_mode, bp_mode=bp_mode)
    ctx.synchronize()
    out = [f.cpu().numpy(), xy.cpu().numpy()]
    if zy:
        out.append(vzy.cpu().numpy())
    return out


@pytest.mark.parametrize("bp_mode", BPS)
def test_fdk65_matches_reference_program(ctx, bp_mode):
    g = abi.fdk_geom_reference65()
    gold = golden("fdk65")
    proj = fdk_projections(360, 65, 65, int(gold["seed"]))
    f, xy, zy = _run(ctx, g, proj, bp_mode=bp_mode, zy=True)
    assert rel_rms(f[gold["view_ids"]], gold["filtered_views"]) < 1e-5
    keep = ~past_end_voxels(g)[:, :, 125:130]
    slab = xy[:, :, 125:130]
    assert rel_rms(slab[keep], gold["xy_slab"][keep]) < 1e-5
    assert not np.any(xy[:, :, :125]) and not np.any(xy[:, :, 130:])
    assert np.array_equal(zy, xy.transpose(2, 1, 0))


@pytest.mark.parametrize("bp_mode", BPS)
def test_fdk325_matches_reference_program(ctx, bp_mode):
    g = abi.fdk_geom_reference325()
    gold = golden("fdk325")
    proj = fdk_projections(360, 325, 325, int(gold["seed"]))
    f, xy = _run(ctx, g, proj, bp_mode=bp_mode)
    got = f[gold["view_ids"]][:, gold["row_ids"], :]
    assert rel_rms(got, gold["filtered_rows"]) < 1e-5
    keep = ~past_end_voxels(g)[:, :, 125:130]
    assert rel_rms(xy[:, :, 125:130][keep], gold["xy_slab"][keep]) < 1e-5


def _small_recon_geom():
    # the recon-325 conventions at a size the FP64 oracle finishes quickly
    return abi.fdk_geom_recon325(n_views=360, nu=128, nv=96, pitch_mm=3.2, n=81,
                                 voxel_mm=1.6)


@pytest.mark.parametrize("bp_mode", BPS)
def test_full_volume_against_fp64_oracle(ctx, bp_mode):
    g = _small_recon_geom()
    proj = fdk_projections(g.n_views, g.nu, g.nv, 2024)
    f, xy = _run(ctx, g, proj, bp_mode=bp_mode)
    f64 = oracle.fdk_filter(g, proj, precise=True)
    assert rel_rms(f, f64) < 1e-5
    v64 = oracle.fdk_backproject(g, f64)
    err = rel_rms(xy, v64)
    assert err < 1e-5, err


@pytest.mark.parametrize("variant", [-1, 33, 29, 0, 22, 20, 2])
def test_noisy_maps_against_fp64_oracle(ctx, variant):
    """Monte Carlo-like -log maps (Poisson noise, 30 histories per pixel)
    on the batched workload's geometry for a 97^3 cube and a 256 x 256
    detector: pixel-to-pixel noise turns any detector-coordinate error into
    a value error one for one, so this is where the float pairs of the
    coordinate path count (a float walk of the coordinates missed 1e-5
    three-fold here).  Plain (-1) and tiled shapes with 32, 16, 24 and 8
    voxels per lane, FP32 filter, 1e-5 relative RMS against the FP64
    oracle."""
    from inputs import noisy_counts_map
    from monte_gb300 import batchscan
    spec = dict(side=97, n_views=30, nu=256, nv=256)
    g = batchscan.fdk_geom_for(spec, batchscan.mc_geom_for(spec))
    proj = noisy_counts_map(g.n_views, g.nu, g.nv, 30, 97)
    f64 = oracle.fdk_filter(g, proj, precise=True)
    v64 = oracle.fdk_backproject(g, f64)
    p = torch.from_numpy(proj).cuda()
    xy = torch.empty((g.nz, g.ny, g.nx), device="cuda")
    try:
        if variant >= 0:
            ctx.set_bp_variant(variant)
        bm = abi.MONTE_BP_PLAIN if variant < 0 else abi.MONTE_BP_TILED
        ctx.fdk(g, p, xy, filter_mode=abi.MONTE_FILTER_FP32, bp_mode=bm)
        ctx.check_status()
        if variant >= 0:
            assert ctx.last_bp_variant() == variant
    finally:
        ctx.set_bp_variant(-1)
    err = rel_rms(xy.cpu().numpy(), v64)
    assert err < 1e-5, (variant, err)


@pytest.mark.parametrize("variant", [33, 34, 35, 36, 38, 39, 40])
def test_noisy_maps_wide_anchor_shapes(ctx, variant):
    """The same check for the shapes that anchor every 20 to 56 voxels,
    which need the rows to advance slowly along z: the benchmark's
    magnification (SOD 500,
    SDD 1000 mm, 0.8 mm pixels, 0.4 mm voxels; ~1.1 rows per voxel) on a
    129^3 volume, 90 views of 256 x 192, 30 histories per pixel."""
    from inputs import noisy_counts_map
    g = abi.fdk_geom_recon325(n_views=90, nu=256, nv=192, pitch_mm=0.8, n=129, voxel_mm=0.4)
    proj = noisy_counts_map(g.n_views, g.nu, g.nv, 30, 129)
    f64 = oracle.fdk_filter(g, proj, precise=True)
    v64 = oracle.fdk_backproject(g, f64)
    p = torch.from_numpy(proj).cuda()
    xy = torch.empty((g.nz, g.ny, g.nx), device="cuda")
    try:
        ctx.set_bp_variant(variant)
        ctx.fdk(g, p, xy, filter_mode=abi.MONTE_FILTER_FP32, bp_mode=abi.MONTE_BP_TILED)
        ctx.check_status()
        assert ctx.last_bp_variant() == variant
    finally:
        ctx.set_bp_variant(-1)
    err = rel_rms(xy.cpu().numpy(), v64)
    assert err < 1e-5, (variant, err)


def test_host_memory_path_equals_device_path(ctx):
    g = abi.fdk_geom_reference65()
    proj = fdk_projections(360, 65, 65, 11)
    f_d, xy_d = _run(ctx, g, proj)
    f_h = np.zeros((g.n_views, g.nv, g.nu), np.float32)
    xy_h = np.zeros((g.nz, g.ny, g.nx), np.float32)
    ctx.fdk(g, proj, xy_h, filtered=f_h)
    assert np.array_equal(f_h, f_d) and np.array_equal(xy_h, xy_d)


def test_bad_arguments_are_rejected(ctx):
    from monte_gb300.lib import MonteError
    g = abi.fdk_geom_reference65()
    g.nu = 0
    p = torch.zeros(10, device="cuda")
    with pytest.raises(MonteError) as e:
        ctx.fdk(g, p, p, filtered=p)
    assert e.value.code == abi.MONTE_EINVAL
    g = abi.fdk_geom_reference65()
    g.s_end = 300
    with pytest.raises(MonteError) as e:
        ctx.fdk(g, p, p, filtered=p)
    assert e.value.code == abi.MONTE_EINVAL
    g = abi.fdk_geom_reference65()
    with pytest.raises(MonteError) as e:
        ctx.fdk(g, p, p, filtered=p, filter_mode=7)
    assert e.value.code == abi.MONTE_EINVAL


def test_tiled_kernel_runs_for_test_geometries(ctx):
    """MONTE_BP_TILED must run the shared-memory kernel (not the plain
    fallback) on the reference and recon geometries."""
    for g in (abi.fdk_geom_reference65(), abi.fdk_geom_reference325(), _small_recon_geom()):
        f = torch.zeros((g.n_views, g.nv, g.nu), device="cuda")
        xy = torch.empty((g.nz, g.ny, g.nx), device="cuda")
        ctx.fdk_backproject(g, f, xy, mode=abi.MONTE_BP_TILED)
        ctx.synchronize()
        assert ctx.last_bp_variant() >= 0


def _tc_geom():
    # nu % 64 == 0 and nv % 128 == 0: the tensor-core filter's tile shape
    return abi.fdk_geom_recon325(n_views=90, nu=256, nv=128, pitch_mm=1.6, n=65, voxel_mm=1.6)


def test_bf16x3_filter_against_fp64_oracle(ctx):
    g = _tc_geom()
    from monte_gb300.phantoms import ellipsoid_line_integrals, random_ellipsoids
    proj = ellipsoid_line_integrals(g, random_ellipsoids(1002), noise_sigma=0.01, seed=3).numpy()
    f_tc, xy_tc = _run(ctx, g, proj, filter_mode=abi.MONTE_FILTER_BF16X3,
                       bp_mode=abi.MONTE_BP_TILED)
    ctx.check_status()
    f_32, xy_32 = _run(ctx, g, proj, filter_mode=abi.MONTE_FILTER_FP32,
                       bp_mode=abi.MONTE_BP_TILED)
    f64 = oracle.fdk_filter(g, proj, precise=True)
    e_tc, e_32 = rel_rms(f_tc, f64), rel_rms(f_32, f64)
    assert e_tc < 1e-5, (e_tc, e_32)
    v64 = oracle.fdk_backproject(g, f64)
    assert rel_rms(xy_tc, v64) < 1e-5
    assert rel_rms(xy_tc, xy_32) < 1e-5


def test_bf16x3_filter_multi_tile_shapes(ctx):
    """nu = 192 (N tile 64), 384 (128), 512 (256) and several row tiles."""
    for nu, nv in ((192, 128), (384, 256), (512, 128)):
        g = abi.fdk_geom_recon325(n_views=6, nu=nu, nv=nv, pitch_mm=1.0, n=33, voxel_mm=2.0)
        proj = fdk_projections(g.n_views, g.nu, g.nv, nu)
        p = torch.from_numpy(proj).cuda()
        f = torch.empty((g.n_views, g.nv, g.nu), device="cuda")
        ctx.fdk_filter(g, p, f, mode=abi.MONTE_FILTER_BF16X3)
        ctx.check_status()
        f64 = oracle.fdk_filter(g, proj, precise=True)
        assert rel_rms(f.cpu().numpy(), f64) < 1e-5, nu


def test_autotune_picks_a_tile_and_all_tiles_agree(ctx):
    g = _small_recon_geom()
    proj = fdk_projections(g.n_views, g.nu, g.nv, 99)
    best = ctx.fdk_autotune(g)
    assert best >= 0
    _, ref = _run(ctx, g, proj, bp_mode=abi.MONTE_BP_PLAIN)
    _, got = _run(ctx, g, proj, bp_mode=abi.MONTE_BP_TILED)
    assert ctx.last_bp_variant() == best
    assert rel_rms(got, ref) < 2e-6
    # every tile shape (pipeline depth, register budget, block shape)
    v = 0
    while True:
        try:
            ctx.set_bp_variant(v)
        except MonteError:
            break
        _, got = _run(ctx, g, proj, bp_mode=abi.MONTE_BP_TILED)
        ctx.check_status()
        assert ctx.last_bp_variant() == v
        assert rel_rms(got, ref) < 2e-6, v
        v += 1
    assert v >= 12
    ctx.set_bp_variant(best)


@pytest.mark.parametrize("bp_mode", BPS)
def test_even_grid_axis_column_against_fp64_oracle(ctx, bp_mode):
    """n even: voxel column n/2 lies on the rotation axis, where the
    distance weight's sign term ts is ~0 in every view (decided in double,
    as the reference computes it)."""
    g = abi.fdk_geom_recon325(n_views=360, nu=128, nv=96, pitch_mm=3.2, n=80, voxel_mm=1.6)
    proj = fdk_projections(g.n_views, g.nu, g.nv, 80)
    _, xy = _run(ctx, g, proj, bp_mode=bp_mode)
    v64 = oracle.fdk_backproject(g, oracle.fdk_filter(g, proj, precise=True))
    assert rel_rms(xy, v64) < 1e-5
    c = g.nx // 2
    assert rel_rms(xy[:, c, c], v64[:, c, c]) < 1e-5


def test_even_grid_backprojects_as_fast_as_odd(ctx):
    """The axis column of an even grid once took the per-voxel double path
    in every view; its warp then held the kernel for ~45 ms whatever the
    volume size.  Even and odd grids of equal size must now take equal time."""
    ms = {}
    for n in (96, 97):
        g = abi.fdk_geom_recon325(n_views=360, nu=128, nv=96, pitch_mm=3.2, n=n,
                                  voxel_mm=1.6 * 80 / n)
        filt = torch.rand((g.n_views, g.nv, g.nu), device="cuda") - 0.5
        vol = torch.empty((g.nz, g.ny, g.nx), device="cuda")
        ctx.fdk_backproject(g, filt, vol, mode=abi.MONTE_BP_TILED)
        torch.cuda.synchronize()
        t = []
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            ctx.fdk_backproject(g, filt, vol, mode=abi.MONTE_BP_TILED)
            e1.record()
            torch.cuda.synchronize()
            t.append(e0.elapsed_time(e1))
        ctx.check_status()
        ms[n] = sorted(t)[1]
    assert ms[96] < 2.0 * ms[97], ms


def test_volume_taller_than_the_field_of_view(ctx):
    """A volume whose top and bottom slices project past the detector's
    first and last rows: per view some voxel blocks lie inside the detector
    (the per-lane edge tests are skipped for them), some straddle its row
    edges (voxel-by-voxel classification, exact decisions near the edges)
    and some project off it.  Every tile shape against the FP64 oracle."""
    g = abi.fdk_geom_recon325(n_views=90, nu=128, nv=64, pitch_mm=3.2, n=65, voxel_mm=2.4)
    proj = fdk_projections(g.n_views, g.nu, g.nv, 65)
    v64 = oracle.fdk_backproject(g, oracle.fdk_filter(g, proj, precise=True))
    _, ref = _run(ctx, g, proj, bp_mode=abi.MONTE_BP_PLAIN)
    assert rel_rms(ref, v64) < 1e-5
    v, ran = 0, 0
    while True:
        try:
            ctx.set_bp_variant(v)
        except MonteError:
            break
        _, got = _run(ctx, g, proj, bp_mode=abi.MONTE_BP_TILED)
        ctx.check_status()
        if ctx.last_bp_variant() == v:
            ran += 1
            assert rel_rms(got, v64) < 1e-5, v
            assert rel_rms(got, ref) < 2e-6, v
        v += 1
    ctx.set_bp_variant(-1)
    assert ran >= 12


@pytest.mark.parametrize("nu", [130, 129])
def test_detector_width_not_a_multiple_of_4(ctx, nu):
    """Rows of nu floats are not a multiple of 16 bytes (as on the
    reference's 65- and 325-wide detectors): the tiles come from a copy with
    padded rows, the exact per-voxel path reads the original.  Every tile
    shape, including the per-warp ones that need TMA, against the FP64
    oracle."""
    g = abi.fdk_geom_recon325(n_views=90, nu=nu, nv=96, pitch_mm=3.2, n=65, voxel_mm=1.6)
    proj = fdk_projections(g.n_views, g.nu, g.nv, nu)
    v64 = oracle.fdk_backproject(g, oracle.fdk_filter(g, proj, precise=True))
    _, ref = _run(ctx, g, proj, bp_mode=abi.MONTE_BP_PLAIN)
    v, ran = 0, 0
    while True:
        try:
            ctx.set_bp_variant(v)
        except MonteError:
            break
        _, got = _run(ctx, g, proj, bp_mode=abi.MONTE_BP_TILED)
        ctx.check_status()
        if ctx.last_bp_variant() == v:
            ran += 1
            assert rel_rms(got, v64) < 1e-5, v
            assert rel_rms(got, ref) < 2e-6, v
        v += 1
    ctx.set_bp_variant(-1)
    assert ran == v  # every shape ran, the per-warp ones on the padded copy
