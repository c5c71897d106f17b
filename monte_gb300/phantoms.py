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


def sphere_labels_185():
    """The label volume monte_cpp/make_image01.cpp:15-30 writes (spher01.raw):
    185 x 185 x 325 voxels, label 1 inside the sphere of radius 50 voxels
    centred on voxel (90, 90, 160), 0 elsewhere; layout [z][y][x].  With the
    CPU program's lookup (monte_cpp/CBCT_real2.cpp:771) voxel (ix,iy,iz) covers
    x in [(ix-90.5)/10, (ix-89.5)/10) cm, y likewise, z around (iz-160)/10."""
    k, j, i = np.ogrid[0:325, 0:185, 0:185]
    inside = (i - 90) ** 2 + (j - 90) ** 2 + (k - 160) ** 2 <= 2500
    return inside.astype(np.uint8)


# voxel size and low corner (cm) of sphere_labels_185() under CBCT_real2's lookup
SPHERE185_VOXEL = 0.1
SPHERE185_ORIGIN = (-9.05, -9.05, -16.05)


def cylinder_inserts_labels(seed=1001, n=65, voxel_mm=1.0, radius_mm=28.0, insert_mm=5.0,
                            place_mm=18.0):
    """The 65^3 phantom of the CPU-runnable workload: water cylinder of radius
    28 mm along z (label 1), three Ca-water inserts of radius 5 mm (labels 2,
    3, 4 for densities 1.2 / 1.5 / 1.9) centred at seeded uniform positions
    within 18 mm of the axis, not overlapping; air (label 0) outside.
    Returns (labels[z][y][x] uint8, voxel cm, origin cm)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    centres = []
    while len(centres) < 3:
        r = place_mm * np.sqrt(rng.random())
        a = 2 * np.pi * rng.random()
        c = (r * np.cos(a), r * np.sin(a))
        if all((c[0] - d[0]) ** 2 + (c[1] - d[1]) ** 2 > (2 * insert_mm + 1) ** 2 for d in centres):
            centres.append(c)
    ax = (np.arange(n) + 0.5 - n / 2.0) * voxel_mm
    Z, Y, X = np.meshgrid(ax, ax, ax, indexing="ij")
    lab = np.zeros((n, n, n), np.uint8)
    lab[X * X + Y * Y <= radius_mm ** 2] = 1
    for i, (cx, cy) in enumerate(centres):
        lab[(X - cx) ** 2 + (Y - cy) ** 2 <= insert_mm ** 2] = 2 + i
    h = n * voxel_mm / 2.0 / 10.0
    return lab, voxel_mm / 10.0, (-h, -h, -h)


# densities (g/cm^3) of the analytic phantom of monte_cu/CBCT_real325.cu:122-123
CA_ROD_DENSITY = (1.0, 1.55)


def ca_rod_labels(voxel_cm=0.1):
    """Voxelised form of the analytic phantom that monte_cu/CBCT_real325.cu
    tests in its Woodcock loop (:916-928): a water cylinder of radius 10 cm
    along x, |x| <= 10 cm, holding eight Ca rods of radius 1.5 cm whose axes
    sit 5 cm from the cylinder's, every 45 degrees in the y-z plane; air
    outside.  A voxel takes the label of its centre: 0 air, 1 water, 2 Ca
    (materials [-1, 0, 1] with densities [0, 1.0, 1.55]).  Covers the box
    [-10, 10]^3 cm.  Returns (labels[z][y][x] uint8, voxel cm, origin cm,
    densities, materials)."""
    n = int(round(20.0 / voxel_cm))
    ax = (np.arange(n) + 0.5) * voxel_cm - 10.0
    Z, Y, X = np.meshgrid(ax, ax, ax, indexing="ij")
    lab = np.zeros((n, n, n), np.uint8)
    lab[(Y * Y + Z * Z <= 100.0) & (np.abs(X) <= 10.0)] = 1
    for k in range(8):
        a = k * np.pi / 4.0
        cy, cz = 5.0 * np.sin(a), 5.0 * np.cos(a)
        lab[((Y - cy) ** 2 + (Z - cz) ** 2 <= 1.5 ** 2) & (lab == 1)] = 2
    return lab, voxel_cm, (-10.0, -10.0, -10.0), [0.0, *CA_ROD_DENSITY], [-1, 0, 1]


def ellipsoid_labels(seed=1003, n=325, voxel_mm=0.8, n_ell=20):
    """The 325^3 phantom of the full Monte Carlo workload: 20 seeded
    ellipsoids (centres U(-80,80) mm, semi-axes U(10,70) mm, random
    rotation) painted in order -- the first four are water (label 1), the
    rest bone (Ca-water) with densities U(1.5, 1.9) g/cm^3, one label each --
    air elsewhere.  Returns (labels uint8, voxel cm, origin cm, densities of
    labels 0..n_labels-1, material of each label)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ax = ((np.arange(n) + 0.5 - n / 2.0) * voxel_mm / 10.0).astype(np.float32)
    lab = np.zeros((n, n, n), np.uint8)
    dens = [0.0, 1.0]
    mats = [-1, 0]
    for e in range(n_ell):
        c = rng.uniform(-8.0, 8.0, 3)
        a = rng.uniform(1.0, 7.0, 3)
        R = _rotation(rng)
        if e < 4:
            label = 1
        else:
            dens.append(float(rng.uniform(1.5, 1.9)))
            mats.append(1)
            label = len(dens) - 1
        for z in range(n):
            Y, X = np.meshgrid(ax, ax, indexing="ij")
            p = (X - c[0], Y - c[1], ax[z] - c[2])
            r2 = 0.0
            for i in range(3):
                q = (R[0, i] * p[0] + R[1, i] * p[1] + R[2, i] * p[2]) / a[i]
                r2 = r2 + q * q
            lab[z][r2 <= 1.0] = label
    h = n * voxel_mm / 2.0 / 10.0
    return lab, voxel_mm / 10.0, (-h, -h, -h), dens, mats


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
