"""Shared test helpers: golden fixtures, error metrics, geometric masks."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def rel_rms(a, ref):
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    return float(np.linalg.norm(a - ref) / max(np.linalg.norm(ref), 1e-300))


def past_end_voxels(g):
    """Boolean [nz][ny][nx] mask of slab voxels whose bilinear stencil, in
    the last view, reaches past the end of the filtered array.  The
    reference reads whatever memory follows its map_out allocation there
    (recon/bp3d20.cpp:152-158 with the flat index of :154-156); the GPU path
    and the oracle read zeros, so those voxels are excluded from exact
    comparisons against the reference programs' output."""
    k = g.n_views - 1
    beta = k * 360.0 / g.n_views
    a = np.pi * beta / 180
    c, s_ = np.cos(a), np.sin(a)
    px, py = float(np.float32(-g.sod)) * c, float(np.float32(-g.sod)) * s_
    z, t, s = np.meshgrid(np.arange(g.nz), np.arange(g.ny), np.arange(g.s_begin, g.s_end),
                          indexing="ij")
    X = g.x0 + s * g.dvox
    Y = g.y0 - t * g.dvox
    Z = g.z0 - z * g.dvox
    p0, p1 = X - px, Y - py
    V0 = p0 * c + p1 * s_
    V1 = -p0 * s_ + p1 * c
    kk = g.sdd / V0
    up, vp = V1 * kk, Z * kk
    ok = (np.abs(up) <= g.half_u) & (np.abs(vp) <= g.half_v)
    y = -(up / g.du - g.half_u / g.du)
    x = -(vp / g.dv - g.half_v / g.dv)
    xi, yi = x.astype(np.int64), y.astype(np.int64)
    total = g.n_views * g.nu * g.nv
    i11 = k * g.nu * g.nv + (xi + 1) * g.nu + yi + 1
    hit = ok & (i11 >= total)
    mask = np.zeros((g.nz, g.ny, g.nx), bool)
    mask[:, :, g.s_begin:g.s_end] = hit
    return mask


def chi2_two_sample(a, b, na=1.0, nb=1.0, min_count=20):
    """Two-sample chi-square for Poisson counts a (exposure na) and b
    (exposure nb) over bins with a + b >= min_count:
    sum (a*sqrt(nb/na) - b*sqrt(na/nb))^2 / (a + b).  Returns (chi2, dof,
    p-value)."""
    from scipy.stats import chi2 as _chi2
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    m = (a + b) >= min_count
    k1, k2 = np.sqrt(nb / na), np.sqrt(na / nb)
    x2 = float(np.sum((k1 * a[m] - k2 * b[m]) ** 2 / (a[m] + b[m])))
    dof = int(m.sum())
    return x2, dof, float(_chi2.sf(x2, dof))


def block_sum(img, k):
    """Sum k x k blocks of a 2-D image (cropped to a multiple of k)."""
    h, w = (img.shape[0] // k) * k, (img.shape[1] // k) * k
    return img[:h, :w].reshape(h // k, k, w // k, k).sum(axis=(1, 3))


def chi2_binomial_two_sample(a, b, n):
    """Two-sample chi-square for binomial counts a, b out of n trials each
    (primary tallies: of n histories aimed at a pixel, each reaches it
    uncollided or not): sum (a - b)^2 / var with the pooled p = (a + b) / 2n
    and var = 2n p (1 - p) * 2n / (2n - 1) -- the unbiased estimate of the
    difference's variance (p (1 - p) alone is low by 1/2n: at n = 49 that
    inflates chi-square by 1 %, which millions of degrees of freedom see),
    over cells with 0 < p < 1.  Returns (chi2, dof, p-value)."""
    from scipy.stats import chi2 as _chi2
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    p = (a + b) / (2.0 * n)
    m = (p > 0) & (p < 1)
    var = 2.0 * n * p[m] * (1.0 - p[m]) * (2.0 * n) / (2.0 * n - 1.0)
    x2 = float(np.sum((a[m] - b[m]) ** 2 / var))
    dof = int(m.sum())
    return x2, dof, float(_chi2.sf(x2, dof))
