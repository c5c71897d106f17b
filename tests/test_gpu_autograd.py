"""The differentiable mode through torch.autograd (tests/autograd_ops.py:
thin Functions over the C ABI's forward and backward entry points).
Gradients that autograd assembles from the library's adjoints are checked
against the FP64 oracle's gradients and against central finite differences
of the FP64 oracle loss; the recomputing least-squares op equals the plain
composition to rounding."""
import numpy as np
import pytest
import torch

import oracle
from autograd_ops import Fdk, ForwardProject, LeastSquares, Transmission
from helpers import rel_rms
from inputs import fdk_projections
from monte_gb300 import abi

pytestmark = pytest.mark.gpu


def _geom():
    g = abi.fdk_geom_recon325(n_views=60, nu=96, nv=64, pitch_mm=4.8, n=41, voxel_mm=2.4)
    g.flags = 0  # the textbook operator: the adjoints need no flat-edge wrap
    return g


def test_least_squares_gradient_through_autograd(ctx):
    g = _geom()
    rng = np.random.default_rng(11)
    x64 = rng.random((g.nz, g.ny, g.nx))
    p64 = oracle.fdk_forward_project(g, rng.random((g.nz, g.ny, g.nx)))  # [view][v][u]
    x = torch.from_numpy(x64.astype(np.float32)).cuda().requires_grad_(True)
    p = torch.from_numpy(p64.astype(np.float32)).cuda()
    loss = ((ForwardProject.apply(x, ctx, g).double() - p.double()) ** 2).sum()
    loss.backward()
    g_auto = x.grad.clone()
    # FP64 gradient 2 A^T (A x - p) with the oracle's operators
    g64 = 2.0 * oracle.fdk_backproject(
        g, oracle.fdk_forward_project(g, x64.astype(np.float32).astype(np.float64)) - p64)
    assert rel_rms(g_auto.cpu().numpy(), g64) < 1e-4
    # the recomputing op: the same gradient, nothing projection-sized kept
    # between forward and backward.  Equal to rounding, not bit for bit: its
    # residual is formed in float rather than double, and the forward
    # projector accumulates detector pixels with atomics, so two runs of A x
    # differ in summation order.
    x.grad = None
    loss2 = LeastSquares.apply(x, p, ctx, g)
    loss2.backward()
    assert rel_rms(x.grad.cpu().numpy(), g_auto.cpu().numpy()) < 1e-6
    assert abs(float(loss2) - float(loss)) <= 1e-7 * abs(float(loss))


def test_least_squares_central_differences(ctx):
    g = _geom()
    rng = np.random.default_rng(12)
    x64 = rng.random((g.nz, g.ny, g.nx))
    p64 = oracle.fdk_forward_project(g, rng.random((g.nz, g.ny, g.nx)))
    x = torch.from_numpy(x64.astype(np.float32)).cuda().requires_grad_(True)
    LeastSquares.apply(x, torch.from_numpy(p64.astype(np.float32)).cuda(), ctx, g).backward()
    gr = x.grad.cpu().numpy()

    def loss(v):
        return float(np.sum((oracle.fdk_forward_project(g, v) - p64) ** 2))

    for idx in [(20, 20, 20), (10, 25, 30), (30, 12, 8)]:
        h = 1e-3
        xp, xm = x64.copy(), x64.copy()
        xp[idx] += h
        xm[idx] -= h
        fd = (loss(xp) - loss(xm)) / (2 * h)
        assert abs(fd - gr[idx]) < 1e-3 * abs(fd) + 1e-6, (idx, fd, gr[idx])


def test_fdk_gradient_through_autograd(ctx):
    g = _geom()
    proj = fdk_projections(g.n_views, g.nu, g.nv, 13)
    xstar = np.random.default_rng(14).random((g.nz, g.ny, g.nx))
    p = torch.from_numpy(proj).cuda().requires_grad_(True)
    loss = ((Fdk.apply(p, ctx, g).double() - torch.from_numpy(xstar).cuda()) ** 2).sum()
    loss.backward()
    v64 = oracle.fdk_backproject(g, oracle.fdk_filter(g, proj, precise=True))
    g64 = oracle.fdk_backward(g, 2.0 * (v64 - xstar))
    # FP32 arithmetic; the ramp filter's cancellation amplifies rounding
    assert rel_rms(p.grad.cpu().numpy(), g64) < 1e-4


def test_transmission_gradient_through_autograd(ctx):
    g = abi.mc_geom(36, 48, 40, 0.25, 50.0, 100.0, 8.0)
    shape = (30, 34, 32)
    rng = np.random.default_rng(15)
    mu64 = 0.2 * rng.random(shape)
    mu32 = mu64.astype(np.float32)
    grid = abi.siddon_grid(shape, 0.2, (-3.2, -3.4, -3.0))
    views = (0, 12)
    w = rng.random((g.n_views, g.nu, g.nv))
    mu = torch.from_numpy(mu32).cuda().requires_grad_(True)
    t = Transmission.apply(mu, ctx, g, grid, views)
    (t.double() * torch.from_numpy(w).cuda()).sum().backward()
    # FP64: d/dmu sum(w exp(-L)) = -A^T (w exp(-L)) with the oracle's walk
    L = oracle.siddon_forward(g, grid, mu32, views)
    gt = np.zeros_like(w)
    gt[views[0]:views[1]] = w[views[0]:views[1]]
    g64 = oracle.siddon_backward(g, grid, mu32, views, grad_trans=gt)
    assert rel_rms(mu.grad.cpu().numpy(), g64) < 1e-5
    assert np.allclose(t.detach().cpu().numpy()[views[0]:views[1]], np.exp(-L[views[0]:views[1]]),
                       rtol=1e-5, atol=1e-7)
