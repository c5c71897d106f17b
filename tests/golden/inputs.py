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
