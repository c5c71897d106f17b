"""The 2-D fan-beam FBP (recon/fbp2.cpp) on the GPU through monte_fbp2: the
kernels keep the reference's double arithmetic and float accumulation, so
the filtered projections and the image equal the oracle's -- which equals
the compiled reference program's (tests/golden/fbp2.npz) -- bit for bit."""
import numpy as np
import pytest
import torch

import oracle
from helpers import golden
from inputs import fdk_projections
from monte_gb300 import abi
from monte_gb300.lib import MonteError

pytestmark = pytest.mark.gpu


def test_fbp2_matches_reference_program(ctx):
    gold = golden("fbp2")
    g = abi.fbp2_geom_reference()
    proj = fdk_projections(360, 65, 1, int(gold["seed"])).reshape(360, 65)
    p = torch.from_numpy(proj).cuda()
    img = torch.empty((g.ny, g.nx), device="cuda")
    filt = torch.empty_like(p)
    ctx.fbp2(g, p, img, filtered=filt)
    ctx.synchronize()
    assert np.array_equal(filt.cpu().numpy(), gold["filtered"])
    assert np.array_equal(img.cpu().numpy(), gold["image"])


def test_fbp2_other_geometries_and_host_memory(ctx):
    g = abi.fbp2_geom_reference()
    g.n_views, g.view_begin, g.view_end = 180, 0, 180
    g.flags = 0
    g.nx, g.ny = 200, 120
    proj = fdk_projections(180, 65, 1, 7).reshape(180, 65)
    f_ref, i_ref = oracle.fbp2(g, proj)
    img = np.zeros((g.ny, g.nx), np.float32)
    filt = np.zeros_like(proj)
    ctx.fbp2(g, proj, img, filtered=filt)  # host arrays: staged through the device
    assert np.array_equal(filt, f_ref)
    assert np.array_equal(img, i_ref)


def test_fbp2_rejects_bad_geometry(ctx):
    g = abi.fbp2_geom_reference()
    g.view_end = 400
    p = np.zeros((360, 65), np.float32)
    with pytest.raises(MonteError) as e:
        ctx.fbp2(g, p, np.zeros((256, 256), np.float32))
    assert e.value.code == abi.MONTE_EINVAL
