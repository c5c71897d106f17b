"""Seeded batches of simulated scans for monte_batch_* (abi.BatchJob).

Each scan: a cube phantom of `side` voxels at 0.8 mm holding seeded random
ellipsoids (water and Ca-water bone at 1.5-1.9 g/cm^3 in air, the content of
the 325^3 Monte Carlo phantom scaled to the cube), a polychromatic source of
1-keV lines from 20 to 80 keV weighted (80 - E), SOD 500 mm, SDD 1000 mm,
`n_views` views over 360 degrees on an nu x nv detector, histories per view
split evenly over the pixels, then FDK of the -log map into a side^3 volume
at the phantom's voxel pitch.

The default draw is the batched serving workload: 64 scans, side
U{65..257}, views U{60..360}, detector nu in {128, 192, ..., 512} by
nv in {128, 256, 384} (multiples of the tensor-core filter's tile), 1e6-1e7
histories per view.
"""
import math

import numpy as np
import torch

from . import abi
from .phantoms import _rotation

VOXEL_CM = 0.08
SOD_CM, SDD_CM = 50.0, 100.0


def specs(seed=1004, n_jobs=64, side=(65, 257), views=(60, 360), nu_steps=(2, 8),
          nv_steps=(1, 3), hist_per_view=(1e6, 1e7), hist_scale=1.0):
    """List of dicts (side, n_views, nu, nv, hist_per_view, hpp, seed)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for j in range(n_jobs):
        s = int(rng.integers(side[0], side[1] + 1))
        nviews = int(rng.integers(views[0], views[1] + 1))
        nu = 64 * int(rng.integers(nu_steps[0], nu_steps[1] + 1))
        nv = 128 * int(rng.integers(nv_steps[0], nv_steps[1] + 1))
        hpv = float(rng.uniform(*hist_per_view)) * hist_scale
        hpp = max(1, int(round(hpv / (nu * nv))))
        out.append(dict(side=s, n_views=nviews, nu=nu, nv=nv, hist_per_view=hpv, hpp=hpp,
                        seed=int(rng.integers(1, 2**62)), phantom_seed=int(rng.integers(1, 2**31))))
    return out


def cube_labels(seed, side, device):
    """uint8 labels[side]^3 (0 air, 1 water, 2.. bone) and per-label
    (density, material): 20 ellipsoids with the 325^3 phantom's draws scaled
    by the cube's edge / 26 cm, painted in order, the first four water."""
    rng = np.random.Generator(np.random.PCG64(seed))
    L = side * VOXEL_CM
    k = L / 26.0
    ax = (torch.arange(side, dtype=torch.float32, device=device) + 0.5 - side / 2.0) * VOXEL_CM
    Z, Y, X = torch.meshgrid(ax, ax, ax, indexing="ij")
    lab = torch.zeros((side, side, side), dtype=torch.uint8, device=device)
    dens, mats = [0.0, 1.0], [-1, 0]
    for e in range(20):
        c = rng.uniform(-8.0, 8.0, 3) * k
        a = rng.uniform(1.0, 7.0, 3) * k
        R = _rotation(rng)
        if e < 4:
            label = 1
        else:
            dens.append(float(rng.uniform(1.5, 1.9)))
            mats.append(1)
            label = len(dens) - 1
        p = (X - float(c[0]), Y - float(c[1]), Z - float(c[2]))
        r2 = torch.zeros_like(X)
        for i in range(3):
            q = (float(R[0, i]) * p[0] + float(R[1, i]) * p[1] + float(R[2, i]) * p[2]) / float(a[i])
            r2 += q * q
        lab[r2 <= 1.0] = label
    return lab, dens, mats


def mc_geom_for(spec):
    L = spec["side"] * VOXEL_CM
    du = 2.5 * L / spec["nu"]
    dv = 2.5 * L / spec["nv"]
    g = abi.McGeom()
    g.n_views, g.nu, g.nv = spec["n_views"], spec["nu"], spec["nv"]
    g.max_interactions = 5
    g.flags = abi.MONTE_MC_STALE_SIN_PHI
    g.du, g.dv = du, dv
    g.half_u, g.half_v = spec["nu"] * du / 2.0, spec["nv"] * dv / 2.0
    g.sod, g.sdd = SOD_CM, SDD_CM
    g.start_plane = 0.75 * L + 0.2
    return g


def fdk_geom_for(spec, mcg):
    """FDK of the scan's map: detector index a at the centre of Monte Carlo
    pixel a (half extents shifted by half a pixel), the phantom's grid."""
    g = abi.FdkGeom()
    g.n_views, g.nu, g.nv = mcg.n_views, mcg.nu, mcg.nv
    g.flags = abi.MONTE_FDK_TAN_DEGREES | abi.MONTE_FDK_FLAT_EDGE
    g.du, g.dv = mcg.du, mcg.dv
    g.half_u = mcg.half_u - mcg.du / 2.0
    g.half_v = mcg.half_v - mcg.dv / 2.0
    g.sod, g.sdd = mcg.sod, mcg.sdd
    g.wdist = g.sdd - g.sod
    n = spec["side"]
    g.nx = g.ny = g.nz = n
    g.s_begin, g.s_end = 0, n
    g.dvox = VOXEL_CM
    c = n * g.dvox / 2.0
    g.x0, g.y0, g.z0 = -c, c, c
    g.mask_radius = 0
    g.scale, g.scale2 = 2.7, 1.0
    return g


class Batch:
    """Device buffers and abi.BatchJob structs of a list of specs (kept
    alive here)."""

    def __init__(self, spec_list, xcom_water, xcom_ca, device="cuda", recon_total=1):
        self.specs = spec_list
        self.E = np.arange(20.0, 81.0)
        self.W = 80.0 - self.E
        self.inputs, self.jobs, self.labels = [], [], []
        self.primary, self.scatter, self.maps, self.vols = [], [], [], []
        tabs = [xcom_water, xcom_ca]
        for j, s in enumerate(spec_list):
            lab, dens, mats = cube_labels(s["phantom_seed"], s["side"], device)
            L = s["side"] * VOXEL_CM
            inp = abi.McInputs(lab, VOXEL_CM, (-L / 2, -L / 2, -L / 2), mats, dens, tabs,
                               self.E, self.W)
            mcg = mc_geom_for(s)
            fg = fdk_geom_for(s, mcg)
            cells = (s["n_views"], s["nu"], s["nv"])
            prim = torch.zeros(cells, dtype=torch.int64, device=device)
            scat = torch.zeros_like(prim)
            mp = torch.zeros(cells, dtype=torch.float32, device=device)
            vol = torch.zeros((s["side"],) * 3, dtype=torch.float32, device=device)
            job = abi.BatchJob()
            job.mc = mcg
            job.phantom = inp.phantom
            job.spectrum = inp.spectrum
            job.seed = s["seed"]
            job.histories_per_pixel = s["hpp"]
            job.fdk = fg
            job.recon_total = recon_total
            job.primary, job.scatter = prim.data_ptr(), scat.data_ptr()
            job.map, job.vol_xy = mp.data_ptr(), vol.data_ptr()
            self.inputs.append(inp)
            self.jobs.append(job)
            self.primary.append(prim)
            self.scatter.append(scat)
            self.maps.append(mp)
            self.vols.append(vol)
        self.xcom = self.inputs[0].xcom

    def histories(self):
        return sum(s["n_views"] * s["nu"] * s["nv"] * s["hpp"] for s in self.specs)

    def updates(self):
        return sum(s["side"] ** 3 * s["n_views"] for s in self.specs)
