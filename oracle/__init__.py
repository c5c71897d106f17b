"""CPU oracle for the Monte hot paths -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package, and only to check or to time the reference algorithm on the
host; the product (monte_gb300, libmonte.so) never calls it.

liboracle.so is built from the C restatements in this directory
(fdk_oracle.c, ...) by oracle/Makefile.
"""
import ctypes as C
import os
import subprocess

import numpy as np

from monte_gb300.abi import FdkGeom

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None


def build():
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(_HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        _LIB = C.CDLL(path)
        f = C.POINTER(C.c_float)
        d = C.POINTER(C.c_double)
        g = C.POINTER(FdkGeom)
        _LIB.oracle_fdk_taps.argtypes = [C.c_int, f]
        _LIB.oracle_fdk_filter.argtypes = [g, f, f]
        _LIB.oracle_fdk_filter_f64.argtypes = [g, f, d]
        _LIB.oracle_fdk_backproject.argtypes = [g, f, f, f, C.c_int, C.c_int]
        _LIB.oracle_fdk_backproject_f64.argtypes = [g, d, d, C.c_int, C.c_int]
        from monte_gb300 import abi
        _LIB.oracle_mc_run.argtypes = [C.POINTER(abi.McGeom), C.POINTER(abi.McPhantom),
                                       C.POINTER(abi.McXcom), C.POINTER(abi.McSpectrum),
                                       C.POINTER(abi.McRequest), C.c_void_p, C.c_void_p,
                                       C.POINTER(C.c_uint64)]
        _LIB.oracle_stream.argtypes = [C.c_uint64, C.c_uint64, C.c_uint32, C.c_int, f]
        u32 = C.POINTER(C.c_uint32)
        _LIB.oracle_philox.argtypes = [u32, C.c_uint32, C.c_uint32, u32]
        _LIB.oracle_logf.argtypes = [f, f, C.c_int]
        _LIB.oracle_sincos_2pi.argtypes = [f, f, f, C.c_int]
        _LIB.oracle_compton.argtypes = [C.c_float, C.c_uint64, C.c_int, f, f]
        sg = C.POINTER(abi.SiddonGrid)
        _LIB.oracle_siddon_forward.argtypes = [C.POINTER(abi.McGeom), sg, f, C.c_int, C.c_int, d]
        _LIB.oracle_siddon_backward.argtypes = [C.POINTER(abi.McGeom), sg, f, C.c_int, C.c_int,
                                                d, d, d]
        _LIB.oracle_fbp2.argtypes = [C.POINTER(abi.Fbp2Geom), f, f, f]
        _LIB.oracle_fbp2.restype = None
    return _LIB


def fbp2(g, proj):
    """recon/fbp2.cpp restated: proj[view][det] float32 -> (filtered
    [view][det], image[ny][nx]) float32."""
    proj = np.ascontiguousarray(proj, np.float32)
    assert proj.shape == (g.n_views, g.n_det)
    filt = np.zeros_like(proj)
    img = np.zeros((g.ny, g.nx), np.float32)
    lib().oracle_fbp2(C.byref(g), _fp(proj), _fp(filt), _fp(img))
    return filt, img


def siddon_forward(g, grid, mu, views):
    """FP64 line integrals [n_views][nu][nv] along the Monte Carlo's
    emission rays (views outside the range stay 0)."""
    mu = np.ascontiguousarray(mu, np.float32)
    out = np.zeros((g.n_views, g.nu, g.nv), np.float64)
    rc = lib().oracle_siddon_forward(C.byref(g), C.byref(grid), _fp(mu), views[0], views[1],
                                     _dp(out))
    if rc != 0:
        raise ValueError("oracle_siddon_forward rejected the inputs")
    return out


def siddon_backward(g, grid, mu, views, grad_line=None, grad_trans=None):
    mu = np.ascontiguousarray(mu, np.float32)
    gm = np.zeros(mu.shape, np.float64)
    gl = None if grad_line is None else np.ascontiguousarray(grad_line, np.float64)
    gt = None if grad_trans is None else np.ascontiguousarray(grad_trans, np.float64)
    rc = lib().oracle_siddon_backward(C.byref(g), C.byref(grid), _fp(mu), views[0], views[1],
                                      _dp(gl) if gl is not None else None,
                                      _dp(gt) if gt is not None else None, _dp(gm))
    if rc != 0:
        raise ValueError("oracle_siddon_backward rejected the inputs")
    return gm


def mc_run(g, inputs, request):
    """Replay of monte_mc_run on the CPU: (primary, scatter, stats) for a
    request, tallies int64 [n_views][nu][nv] (labels must be host numpy)."""
    prim = np.zeros((g.n_views, g.nu, g.nv), np.int64)
    scat = np.zeros_like(prim)
    st = (C.c_uint64 * 10)()
    rc = lib().oracle_mc_run(C.byref(g), C.byref(inputs.phantom), C.byref(inputs.xcom),
                             C.byref(inputs.spectrum), C.byref(request), prim.ctypes.data,
                             scat.ctypes.data, st)
    if rc != 0:
        raise ValueError("oracle_mc_run rejected the inputs (%d)" % rc)
    names = ("histories", "woodcock_steps", "interactions", "primary_counts",
             "scatter_counts", "dropped", "rayleigh", "compton", "photoelectric",
             "majorant_legs")
    return prim, scat, dict(zip(names, [int(x) for x in st]))


def mc_ref64(g, inputs, seed, per, views):
    """The independent FP64 transport (mc_ref64.c): its own streams and
    double arithmetic, no product code.  Returns (primary, scatter, stats)
    for per histories at every pixel of views [views[0], views[1])."""
    L = lib()
    from monte_gb300 import abi
    L.oracle_mc_ref64.argtypes = [C.POINTER(abi.McGeom), C.POINTER(abi.McPhantom),
                                  C.POINTER(abi.McXcom), C.POINTER(abi.McSpectrum), C.c_uint64,
                                  C.c_uint64, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                  C.POINTER(C.c_uint64)]
    prim = np.zeros((g.n_views, g.nu, g.nv), np.int64)
    scat = np.zeros_like(prim)
    st = (C.c_uint64 * 8)()
    rc = L.oracle_mc_ref64(C.byref(g), C.byref(inputs.phantom), C.byref(inputs.xcom),
                           C.byref(inputs.spectrum), seed, per, views[0], views[1],
                           prim.ctypes.data, scat.ctypes.data, st)
    if rc != 0:
        raise ValueError("oracle_mc_ref64 rejected the inputs (%d)" % rc)
    names = ("histories", "woodcock_steps", "interactions", "primary_counts", "scatter_counts",
             "rayleigh", "compton", "photoelectric")
    return prim, scat, dict(zip(names, [int(v) for v in st]))


def stream(seed, history, job, n):
    out = np.zeros(n, np.float32)
    lib().oracle_stream(seed, history, job, n, _fp(out))
    return out


def philox(ctr, key):
    c = np.ascontiguousarray(ctr, np.uint32)
    out = np.zeros(4, np.uint32)
    u32 = C.POINTER(C.c_uint32)
    lib().oracle_philox(c.ctypes.data_as(u32), int(key[0]), int(key[1]), out.ctypes.data_as(u32))
    return out


def logf(x):
    x = np.ascontiguousarray(x, np.float32)
    y = np.zeros_like(x)
    lib().oracle_logf(_fp(x), _fp(y), len(x))
    return y


def sincos_2pi(u):
    u = np.ascontiguousarray(u, np.float32)
    s, c = np.zeros_like(u), np.zeros_like(u)
    lib().oracle_sincos_2pi(_fp(u), _fp(s), _fp(c), len(u))
    return s, c


def compton(E, seed, n):
    """cos(theta) and scattered energy of n Compton events at E keV."""
    ct = np.zeros(n, np.float32)
    e = np.zeros(n, np.float32)
    lib().oracle_compton(E, seed, n, _fp(ct), _fp(e))
    return ct, e


def _fp(a):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _dp(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_double))


def fdk_taps(nu):
    out = np.zeros(2 * nu - 1, np.float32)
    lib().oracle_fdk_taps(nu, _fp(out))
    return out


def fdk_filter(g, proj, precise=False):
    """proj[view][u][v] float32 -> filtered[view][v][u] (float32, or float64
    when precise)."""
    proj = np.ascontiguousarray(proj, np.float32)
    assert proj.shape == (g.n_views, g.nu, g.nv)
    if precise:
        out = np.zeros((g.n_views, g.nv, g.nu), np.float64)
        lib().oracle_fdk_filter_f64(C.byref(g), _fp(proj), _dp(out))
    else:
        out = np.zeros((g.n_views, g.nv, g.nu), np.float32)
        lib().oracle_fdk_filter(C.byref(g), _fp(proj), _fp(out))
    return out


def fdk_backproject(g, filtered, z_range=None, zy=False):
    """filtered[view][v][u] -> vol_xy[nz][ny][nx] (and vol_zy[nx][ny][nz]).
    float32 input: the reference's own arithmetic; float64 input: FP64."""
    z0, z1 = z_range if z_range is not None else (0, g.nz)
    if filtered.dtype == np.float64:
        filtered = np.ascontiguousarray(filtered)
        vol = np.zeros((g.nz, g.ny, g.nx), np.float64)
        lib().oracle_fdk_backproject_f64(C.byref(g), _dp(filtered), _dp(vol), z0, z1)
        return vol
    filtered = np.ascontiguousarray(filtered, np.float32)
    vol = np.zeros((g.nz, g.ny, g.nx), np.float32)
    vzy = np.zeros((g.nx, g.ny, g.nz), np.float32) if zy else None
    lib().oracle_fdk_backproject(C.byref(g), _fp(filtered), _fp(vol),
                                 _fp(vzy) if zy else None, z0, z1)
    return (vol, vzy) if zy else vol


def fdk_forward_project(g, vol64):
    """FP64 transpose of the FP64 backprojection (no flat-edge quirk)."""
    vol64 = np.ascontiguousarray(vol64, np.float64)
    out = np.zeros((g.n_views, g.nv, g.nu), np.float64)
    L = lib()
    L.oracle_fdk_forward_project_f64.argtypes = [C.POINTER(FdkGeom), C.POINTER(C.c_double),
                                                 C.POINTER(C.c_double)]
    L.oracle_fdk_forward_project_f64(C.byref(g), _dp(vol64), _dp(out))
    return out


def fdk_backward(g, grad_vol64):
    """FP64 adjoint of the whole FDK: grad_vol -> grad_proj[view][u][v]."""
    tmp = fdk_forward_project(g, grad_vol64)
    out = np.zeros((g.n_views, g.nu, g.nv), np.float64)
    L = lib()
    L.oracle_fdk_filter_adjoint_f64.argtypes = [C.POINTER(FdkGeom), C.POINTER(C.c_double),
                                                C.POINTER(C.c_double)]
    L.oracle_fdk_filter_adjoint_f64(C.byref(g), _dp(tmp), _dp(out))
    return out
