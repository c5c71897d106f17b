"""FP64 Siddon oracle: exact chord lengths through a uniform box, and its
adjoint is the transpose of its forward (no GPU)."""
import numpy as np

import oracle
from monte_gb300 import abi


def _geom():
    return abi.mc_geom(8, 24, 16, 0.4, 50.0, 100.0, 10.0)


def test_uniform_box_line_integrals_are_chords():
    g = _geom()
    n, vox = 20, 0.25
    org = (-2.5, -2.0, -2.4)
    grid = abi.siddon_grid((n, n, n), vox, org)
    mu = np.full((n, n, n), 0.37, np.float32)
    L = oracle.siddon_forward(g, grid, mu, (0, g.n_views))
    # analytic chord of each ray through the box
    lo = np.array(org)
    hi = lo + n * vox
    for view in (0, 3, 7):
        a = np.pi * view * 360.0 / g.n_views / 180.0
        c, s = np.float32(np.cos(a)), np.float32(np.sin(a))
        for iu in range(g.nu):
            for iv in range(g.nv):
                yl = g.half_u - g.du * (iu + 0.5)
                zl = g.half_v - g.dv * (iv + 0.5)
                pa, th = np.arctan(yl / g.sdd), 0.5 * np.pi - np.arctan(zl / g.sdd)
                sa, ca = np.float32(np.sin(pa)), np.float32(np.cos(pa))
                st, ct = np.float32(np.sin(th)), np.float32(np.cos(th))
                cp = np.float32(ca * c - sa * s)
                sp = np.float32(sa * c + ca * s)
                o = np.array([np.float32(-np.float32(g.sod) * c), np.float32(-np.float32(g.sod) * s), 0.0])
                d = np.array([np.float32(st * cp), np.float32(st * sp), ct], np.float64)
                with np.errstate(divide="ignore"):
                    ta, tb = (lo - o) / d, (hi - o) / d
                t0 = np.max(np.minimum(ta, tb))
                t1 = np.min(np.maximum(ta, tb))
                want = 0.37 * max(0.0, t1 - t0) * np.linalg.norm(d) / np.linalg.norm(d)
                assert abs(L[view, iu, iv] - np.float32(0.37) * max(0.0, t1 - t0)) < 1e-9 * max(1, want)


def test_backward_is_transpose():
    g = _geom()
    rng = np.random.default_rng(0)
    grid = abi.siddon_grid((12, 14, 10), 0.4, (-2.0, -2.8, -2.4))
    mu = rng.random((12, 14, 10)).astype(np.float32)
    y = rng.standard_normal((g.n_views, g.nu, g.nv))
    views = (1, 6)
    L = oracle.siddon_forward(g, grid, mu, views)
    At_y = oracle.siddon_backward(g, grid, mu, views, grad_line=y)
    lhs = float(np.sum(L[1:6] * y[1:6]))
    rhs = float(np.sum(mu.astype(np.float64) * At_y))
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)
