"""Differentiable FDK on the GPU: the forward projector is the exact adjoint
of the backprojector, and the FDK backward pass gives the gradient of
||FDK(p) - x*||^2 -- checked by dot-product tests, against the FP64 oracle
gradient, and by central finite differences."""
import numpy as np
import pytest
import torch

import oracle
from helpers import rel_rms
from inputs import fdk_projections
from monte_gb300 import abi
from monte_gb300.lib import MonteError

pytestmark = pytest.mark.gpu


def _geom():
    g = abi.fdk_geom_recon325(n_views=60, nu=96, nv=64, pitch_mm=4.8, n=41, voxel_mm=2.4)
    g.flags = 0  # textbook operator: no flat-edge wrap, tan of radians
    return g


def test_forward_projector_is_adjoint_of_backprojector(ctx):
    g = _geom()
    rng = np.random.default_rng(0)
    F = torch.from_numpy(rng.standard_normal((g.n_views, g.nv, g.nu)).astype(np.float32)).cuda()
    R = torch.from_numpy(rng.standard_normal((g.nz, g.ny, g.nx)).astype(np.float32)).cuda()
    BF = torch.empty_like(R)
    ctx.fdk_backproject(g, F, BF, mode=abi.MONTE_BP_PLAIN)
    FR = torch.empty_like(F)
    ctx.fdk_forward_project(g, R, FR)
    ctx.synchronize()
    lhs = float(torch.sum(BF.double() * R.double()))
    rhs = float(torch.sum(F.double() * FR.double()))
    assert abs(lhs - rhs) < 1e-5 * abs(lhs), (lhs, rhs)
    # and the forward projector matches the FP64 transpose
    ref = oracle.fdk_forward_project(g, R.cpu().numpy().astype(np.float64))
    assert rel_rms(FR.cpu().numpy(), ref) < 1e-5


def test_fdk_backward_is_adjoint_and_matches_fp64_gradient(ctx):
    g = _geom()
    proj = fdk_projections(g.n_views, g.nu, g.nv, 8)
    xstar = np.random.default_rng(1).random((g.nz, g.ny, g.nx)).astype(np.float32)
    p = torch.from_numpy(proj).cuda()
    vol = torch.empty((g.nz, g.ny, g.nx), device="cuda")
    ctx.fdk(g, p, vol)
    resid = 2.0 * (vol - torch.from_numpy(xstar).cuda())
    grad = torch.empty_like(p)
    ctx.fdk_backward(g, resid.contiguous(), grad)
    ctx.synchronize()
    # dot test <FDK(p), r> = <p, FDK^T r>
    lhs = float(torch.sum(vol.double() * resid.double()))
    rhs = float(torch.sum(p.double() * grad.double()))
    assert abs(lhs - rhs) < 1e-5 * abs(lhs)
    # FP64 gradient: 2 FDK^T (FDK(p) - x*) with the oracle's operators
    f64 = oracle.fdk_filter(g, proj, precise=True)
    v64 = oracle.fdk_backproject(g, f64)
    g64 = oracle.fdk_backward(g, 2.0 * (v64 - xstar.astype(np.float64)))
    # FP32 arithmetic; the ramp filter's cancellation amplifies rounding
    assert rel_rms(grad.cpu().numpy(), g64) < 1e-4


def test_fdk_gradient_central_differences(ctx):
    g = _geom()
    proj = fdk_projections(g.n_views, g.nu, g.nv, 9).astype(np.float64)
    xstar = np.random.default_rng(2).random((g.nz, g.ny, g.nx))

    def loss(pp):
        v = oracle.fdk_backproject(g, oracle.fdk_filter(g, pp.astype(np.float32), precise=True))
        return float(np.sum((v - xstar) ** 2))

    p = torch.from_numpy(proj.astype(np.float32)).cuda()
    vol = torch.empty((g.nz, g.ny, g.nx), device="cuda")
    ctx.fdk(g, p, vol)
    resid = (2.0 * (vol.double() - torch.from_numpy(xstar).cuda())).float().contiguous()
    grad = torch.empty_like(p)
    ctx.fdk_backward(g, resid, grad)
    ctx.synchronize()
    gr = grad.cpu().numpy()
    for idx in [(5, 40, 30), (30, 50, 10), (45, 20, 33)]:
        h = 0.5
        pp, pm = proj.copy(), proj.copy()
        pp[idx] += h
        pm[idx] -= h
        fd = (loss(pp) - loss(pm)) / (2 * h)
        assert abs(fd - gr[idx]) < 1e-3 * abs(fd) + 1e-6, (idx, fd, gr[idx])


def test_adjoint_requires_textbook_edges(ctx):
    g = abi.fdk_geom_reference65()
    v = torch.zeros((g.nz, g.ny, g.nx), device="cuda")
    out = torch.zeros((g.n_views, g.nv, g.nu), device="cuda")
    with pytest.raises(MonteError) as e:
        ctx.fdk_forward_project(g, v, out)
    assert e.value.code == abi.MONTE_EUNSUPPORTED


def test_forward_projector_on_a_sparse_volume(ctx):
    """Empty voxels and empty voxel columns are skipped (a column occupancy
    map from the z-major copy): a volume that is zero outside a few blocks
    and along whole columns still matches the FP64 transpose."""
    g = _geom()
    rng = np.random.default_rng(3)
    R = np.zeros((g.nz, g.ny, g.nx), np.float32)
    R[5:30, 8:20, 10:33] = rng.standard_normal((25, 12, 23))
    R[:, 25:28, 2:6] = rng.standard_normal((g.nz, 3, 4))
    R[::3] = 0.0  # empty z-slices inside the blocks
    FR = torch.empty((g.n_views, g.nv, g.nu), device="cuda")
    ctx.fdk_forward_project(g, torch.from_numpy(R).cuda(), FR)
    ctx.synchronize()
    ref = oracle.fdk_forward_project(g, R.astype(np.float64))
    assert np.abs(ref).max() > 0
    assert rel_rms(FR.cpu().numpy(), ref) < 1e-5
