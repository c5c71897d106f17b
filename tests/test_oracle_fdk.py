"""The FDK oracle against the reference programs' own output.

tests/golden/fdk65.npz and fdk325.npz hold the output of recon/bp3d20.cpp
and recon/bp3d20_325.cpp, compiled unmodified and run on seeded inputs
(tests/golden/make_golden.py).  On x86-64 the oracle's faithful mode is
bit-equal to them; elsewhere libm may differ in the last ulp.
"""
import platform

import numpy as np
import pytest

import oracle
from helpers import golden, past_end_voxels, rel_rms
from inputs import fdk_projections
from monte_gb300.abi import fdk_geom_reference65, fdk_geom_reference325

EXACT = platform.machine() in ("x86_64", "AMD64")


def _check(got, want):
    if EXACT:
        assert np.array_equal(got, want), np.abs(got - want).max()
    else:
        assert rel_rms(got, want) < 1e-6


def test_taps_match_reference_definition():
    taps = oracle.fdk_taps(65)
    assert taps[64] == np.float32(0.25)
    assert taps[64 + 2] == 0 and taps[64 - 4] == 0
    assert taps[64 + 1] == np.float32(-1.0 / np.pi ** 2)
    assert taps[64 - 3] == np.float32(-1.0 / (3 * np.pi) ** 2)


def test_fdk65_matches_bp3d20():
    g = fdk_geom_reference65()
    gold = golden("fdk65")
    proj = fdk_projections(360, 65, 65, int(gold["seed"]))
    f = oracle.fdk_filter(g, proj)
    _check(f[gold["view_ids"]], gold["filtered_views"])
    vol = oracle.fdk_backproject(g, f)
    slab = vol[:, :, 125:130]
    keep = ~past_end_voxels(g)[:, :, 125:130]
    _check(slab[keep], gold["xy_slab"][keep])
    # outside the slab the reference writes zeros
    assert not np.any(vol[:, :, :125]) and not np.any(vol[:, :, 130:])


@pytest.mark.slow
def test_fdk325_matches_bp3d20_325():
    g = fdk_geom_reference325()
    gold = golden("fdk325")
    proj = fdk_projections(360, 325, 325, int(gold["seed"]))
    f = oracle.fdk_filter(g, proj)
    _check(f[gold["view_ids"]][:, gold["row_ids"], :], gold["filtered_rows"])
    vol = oracle.fdk_backproject(g, f)
    slab = vol[:, :, 125:130]
    excl = past_end_voxels(g)[:, :, 125:130]
    assert 0 < excl.sum() < 1000
    _check(slab[~excl], gold["xy_slab"][~excl])


def test_precise_mode_close_to_faithful():
    g = fdk_geom_reference65()
    proj = fdk_projections(360, 65, 65, 7)
    f32 = oracle.fdk_filter(g, proj)
    f64 = oracle.fdk_filter(g, proj, precise=True)
    assert rel_rms(f32, f64) < 1e-6
    v32 = oracle.fdk_backproject(g, f32, z_range=(100, 140))
    v64 = oracle.fdk_backproject(g, f64, z_range=(100, 140))
    assert rel_rms(v32, v64) < 1e-5
