"""Seeded synthetic phantoms and exact projections for the benchmark
workloads (the reference ships no phantom files: cyu8_2.raw, spher01.raw
are generated or missing, monte_cpp/make_image01.cpp:15-30).

* random_ellipsoids(): the 20-ellipsoid phantoms of the FDK / differentiable
  workloads -- semi-axes U(5,60) mm, centres U(-40,40) mm, uniformly random
  rotation, mu U(0,0.04)/mm, additive.
* ellipsoid_line_integrals(): exact ray-ellipsoid chord integrals for the
  FDK detector convention (sample a at u = half_u - du*a, b at
  v = half_v - dv*b; source at distance sod, detector plane at sdd, view k
  at k*360/n_views degrees), optionally with Gaussian noise.
* cylinder_inserts_labels(): the 65^3 Monte Carlo phantom -- water cylinder
  r = 28 mm along z with three Ca-water inserts r = 5 mm at seeded positions.
* ellipsoid_labels(): the 325^3 Monte Carlo phantom -- water / bone (Ca-water)
  / air regions from 20 seeded ellipsoids.

All lengths here are centimetres (the reference's unit).
"""
import math

import numpy as np
import torch


def _rotation(rng):
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([
        [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
        [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
        [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
    ])


def random_ellipsoids(seed, n=20, axes_mm=(5.0, 60.0), centre_mm=40.0, mu_per_mm=(0.0, 0.04)):
    """List of (centre[3] cm, semi_axes[3] cm, R[3x3], mu 1/cm)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for _ in range(n):
        axes = rng.uniform(*axes_mm, size=3) / 10.0
        centre = rng.uniform(-centre_mm, centre_mm, size=3) / 10.0
        R = _rotation(rng)
        mu = rng.uniform(*mu_per_mm) * 10.0
        out.append((centre, axes, R, mu))
    return out


def ellipsoid_line_integrals(g, ellipsoids, noise_sigma=0.0, seed=0, device="cpu"):
    """proj[view][u][v] float32 of exact line integrals through `ellipsoids`
    for FDK geometry `g` (monte_fdk_geom), plus N(0, noise_sigma^2)."""
    dt = torch.float64
    k = torch.arange(g.n_views, dtype=dt, device=device)
    beta = k * (2 * math.pi / g.n_views)
    cb, sb = torch.cos(beta), torch.sin(beta)
    a = torch.arange(g.nu, dtype=dt, device=device)
    b = torch.arange(g.nv, dtype=dt, device=device)
    up = g.half_u - g.du * a  # view-frame y of column a
    vp = g.half_v - g.dv * b  # z of row b
    xd = g.sdd - g.sod
    # source (world)
    S = torch.stack([-g.sod * cb, -g.sod * sb, torch.zeros_like(cb)], -1)  # [V,3]
    # detector point (world) [V,U,Vv,3]
    Px = (xd * cb)[:, None] - up[None, :] * sb[:, None]
    Py = (xd * sb)[:, None] + up[None, :] * cb[:, None]
    out = torch.zeros((g.n_views, g.nu, g.nv), dtype=dt, device=device)
    for centre, axes, R, mu in ellipsoids:
        Rt = torch.tensor(R.T, dtype=dt, device=device)
        c = torch.tensor(centre, dtype=dt, device=device)
        ax = torch.tensor(axes, dtype=dt, device=device)
        q = ((S - c) @ Rt.T) / ax  # [V,3]
        # direction d = P - S, per (view, u, v); split by components for memory
        dx = (Px - S[:, 0:1])[:, :, None].expand(-1, -1, g.nv)
        dy = (Py - S[:, 1:2])[:, :, None].expand(-1, -1, g.nv)
        dz = vp[None, None, :].expand(g.n_views, g.nu, -1)
        e0 = (Rt[0, 0] * dx + Rt[0, 1] * dy + Rt[0, 2] * dz) / ax[0]
        e1 = (Rt[1, 0] * dx + Rt[1, 1] * dy + Rt[1, 2] * dz) / ax[1]
        e2 = (Rt[2, 0] * dx + Rt[2, 1] * dy + Rt[2, 2] * dz) / ax[2]
        A = e0 * e0 + e1 * e1 + e2 * e2
        B = q[:, 0, None, None] * e0 + q[:, 1, None, None] * e1 + q[:, 2, None, None] * e2
        Cc = (q * q).sum(-1)[:, None, None] - 1.0
        disc = torch.clamp(B * B - A * Cc, min=0.0)
        length = torch.sqrt(dx * dx + dy * dy + dz * dz)
        out += mu * 2.0 * torch.sqrt(disc) / A * length
        del dx, dy, dz, e0, e1, e2, A, B, disc, length
    if noise_sigma > 0:
        gen = torch.Generator(device=device)
        gen.manual_seed(seed)
        out += noise_sigma * torch.randn(out.shape, dtype=dt, device=device, generator=gen)
    return out.to(torch.float32)


def ellipsoid_density(ellipsoids, X, Y, Z):
    """Sum of mu over ellipsoids containing the points (numpy/torch arrays)."""
    out = 0.0 * X
    for centre, axes, R, mu in ellipsoids:
        p = [X - centre[0], Y - centre[1], Z - centre[2]]
        r2 = 0.0
        for i in range(3):
            qi = (R[0, i] * p[0] + R[1, i] * p[1] + R[2, i] * p[2]) / axes[i]
            r2 = r2 + qi * qi
        out = out + mu * (r2 <= 1.0)
    return out
