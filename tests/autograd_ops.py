"""Thin torch.autograd.Function wrappers over the C ABI's forward and
backward entry points -- test harness only (the product is the C ABI; the
tests drive its adjoints through autograd as a caller would).

* ForwardProject: A x, the cone-beam forward projector
  (monte_fdk_forward_project, [z][y][x] -> [view][v][u]); backward A^T g
  with the plain backprojector (monte_fdk_backproject), its exact adjoint.
* LeastSquares: ||A x - p||^2 in one op that keeps only x: backward
  recomputes A x rather than storing the projections (the pattern for
  volumes whose projections would not fit beside them).
* Fdk: the whole FDK, proj[view][u][v] -> vol (monte_fdk); backward
  monte_fdk_backward.
* Transmission: exp(-integral mu) along the Monte Carlo's emission rays
  (monte_siddon_forward); backward monte_siddon_backward.
Every backward stays on the GPU: the library queues on torch's stream.
"""
import torch

from monte_gb300 import abi


class ForwardProject(torch.autograd.Function):
    @staticmethod
    def forward(fctx, x, ctx, g):
        fctx.ctx, fctx.g = ctx, g
        out = torch.empty((g.n_views, g.nv, g.nu), device=x.device)
        ctx.fdk_forward_project(g, x.contiguous(), out)
        return out

    @staticmethod
    def backward(fctx, grad):
        gx = torch.empty((fctx.g.nz, fctx.g.ny, fctx.g.nx), device=grad.device)
        fctx.ctx.fdk_backproject(fctx.g, grad.contiguous(), gx, mode=abi.MONTE_BP_PLAIN)
        return gx, None, None


class LeastSquares(torch.autograd.Function):
    @staticmethod
    def forward(fctx, x, p, ctx, g):
        fctx.ctx, fctx.g = ctx, g
        fctx.save_for_backward(x, p)
        ax = torch.empty((g.n_views, g.nv, g.nu), device=x.device)
        ctx.fdk_forward_project(g, x.contiguous(), ax)
        return ((ax.double() - p.double()) ** 2).sum()

    @staticmethod
    def backward(fctx, grad):
        x, p = fctx.saved_tensors
        g = fctx.g
        # recompute A x: nothing of the size of the projections was kept
        r = torch.empty((g.n_views, g.nv, g.nu), device=x.device)
        fctx.ctx.fdk_forward_project(g, x.contiguous(), r)
        r.sub_(p).mul_(2.0 * float(grad))
        gx = torch.empty_like(x)
        fctx.ctx.fdk_backproject(g, r, gx, mode=abi.MONTE_BP_PLAIN)
        return gx, None, None, None


class Fdk(torch.autograd.Function):
    @staticmethod
    def forward(fctx, p, ctx, g):
        fctx.ctx, fctx.g = ctx, g
        vol = torch.empty((g.nz, g.ny, g.nx), device=p.device)
        ctx.fdk(g, p.contiguous(), vol)
        return vol

    @staticmethod
    def backward(fctx, grad):
        gp = torch.empty((fctx.g.n_views, fctx.g.nu, fctx.g.nv), device=grad.device)
        fctx.ctx.fdk_backward(fctx.g, grad.contiguous(), gp)
        return gp, None, None


class Transmission(torch.autograd.Function):
    @staticmethod
    def forward(fctx, mu, ctx, g, grid, views):
        fctx.ctx, fctx.g, fctx.grid, fctx.views = ctx, g, grid, views
        fctx.save_for_backward(mu)
        t = torch.zeros((g.n_views, g.nu, g.nv), device=mu.device)
        ctx.siddon_forward(g, grid, mu.contiguous(), views, transmission=t)
        return t

    @staticmethod
    def backward(fctx, grad):
        (mu,) = fctx.saved_tensors
        gm = torch.zeros_like(mu)
        fctx.ctx.siddon_backward(fctx.g, fctx.grid, mu.contiguous(), fctx.views, gm,
                                 grad_transmission=grad.contiguous())
        return gm, None, None, None, None
