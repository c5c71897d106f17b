"""Seeded synthetic inputs shared by the golden-fixture generator and the
tests.  Only IEEE-exact operations (+ - * / sqrt) and numpy's PCG64 stream
are used, so every platform regenerates the same float32 arrays."""
import numpy as np


def fdk_projections(n_views, nu, nv, seed):
    """A projection stack proj[view][u][v]: a few smooth rational bumps whose
    centres drift with the view index, plus uniform noise."""
    rng = np.random.Generator(np.random.PCG64(seed))
    k = np.arange(n_views, dtype=np.float64)[:, None, None]
    a = np.arange(nu, dtype=np.float64)[None, :, None]
    b = np.arange(nv, dtype=np.float64)[None, None, :]
    out = np.zeros((n_views, nu, nv), np.float64)
    for _ in range(4):
        amp, cu, cv, su, sv, drift = rng.random(6)
        cu = (0.25 + 0.5 * cu) * nu
        cv = (0.25 + 0.5 * cv) * nv
        su = (0.05 + 0.2 * su) * nu
        sv = (0.05 + 0.2 * sv) * nv
        # triangle-wave drift of the centre with the view index
        ph = (k * (0.5 + drift) / n_views) % 1.0
        tri = 4.0 * np.abs(ph - 0.5) - 1.0
        du = (a - cu - 0.15 * nu * tri) / su
        dv = (b - cv) / sv
        out += (0.5 + 2.0 * amp) / (1.0 + du * du + dv * dv)
    out += 0.01 * rng.random((n_views, nu, nv))
    return out.astype(np.float32)


def noisy_counts_map(n_views, nu, nv, histories_per_pixel, seed):
    """A -log map like the Monte Carlo's, map[view][u][v] = ln(hpp) - ln N
    with N Poisson counts (clamped to [1, hpp]) of hpp histories through a
    smooth attenuation bump: pixel-to-pixel noise of ~1/sqrt(N), the case
    where the backprojector's coordinate rounding shows in the volume.
    Uses exp and log (libm), so it is for comparisons made on one host,
    not for fixtures."""
    rng = np.random.Generator(np.random.PCG64(seed))
    a = (np.arange(nu, dtype=np.float64) - nu / 2) / (nu / 2)
    b = (np.arange(nv, dtype=np.float64) - nv / 2) / (nv / 2)
    mu = 2.0 * np.clip(1.0 - a[:, None] ** 2 - 0.5 * b[None, :] ** 2, 0.0, None)
    n = rng.poisson(histories_per_pixel * np.exp(-mu), (n_views, nu, nv))
    n = np.clip(n, 1, histories_per_pixel).astype(np.float64)
    return (np.log(float(histories_per_pixel)) - np.log(n)).astype(np.float32)
