"""Python front end of libmonte.so (ctypes over the C ABI in include/monte.h).

Arrays are passed as torch CUDA tensors (device memory, MONTE_MEM_DEVICE)
or as numpy arrays / CPU tensors (host memory, MONTE_MEM_HOST).  There is
no fallback: if libmonte.so is missing or no GPU is usable, calls raise.
"""
import ctypes as C
import os

import numpy as np

from . import abi
from .abi import FdkGeom

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libmonte.so")
_LIB = None


class MonteError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("monte error %d: %s" % (code, msg))
        self.code = code


def load(build_if_missing=False):
    """Load libmonte.so (raises if it is missing and build_if_missing is
    False)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise MonteError(abi.MONTE_EUNSUPPORTED,
                             "libmonte.so not built (run monte_gb300.build.build())")
        from .build import build
        build()
    lib = C.CDLL(LIB_PATH)
    P = C.c_void_p
    G = C.POINTER(FdkGeom)
    lib.monte_abi_version.restype = C.c_int
    lib.monte_ctx_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
    lib.monte_ctx_destroy.argtypes = [P]
    lib.monte_last_error.argtypes = [P]
    lib.monte_last_error.restype = C.c_char_p
    lib.monte_ctx_set_stream.argtypes = [P, P]
    lib.monte_ctx_synchronize.argtypes = [P]
    lib.monte_ctx_use_own_stream.argtypes = [P]
    lib.monte_fdk_geom_reference65.argtypes = [G]
    lib.monte_fdk_geom_reference65.restype = None
    lib.monte_fdk_geom_reference325.argtypes = [G]
    lib.monte_fdk_geom_reference325.restype = None
    lib.monte_fdk_filter.argtypes = [P, G, P, P, C.c_int, C.c_int]
    lib.monte_fdk_backproject.argtypes = [P, G, P, P, P, C.c_int, C.c_int]
    lib.monte_fdk.argtypes = [P, G, P, P, P, P, C.c_int, C.c_int, C.c_int]
    lib.monte_fdk_autotune.argtypes = [P, G, C.POINTER(C.c_int)]
    lib.monte_fdk_forward_project.argtypes = [P, G, P, P, C.c_int]
    lib.monte_fdk_backward.argtypes = [P, G, P, P, C.c_int]
    lib.monte_fdk_last_bp_variant.argtypes = [P]
    lib.monte_fdk_last_host_ranges.argtypes = [P]
    lib.monte_fdk_set_bp_variant.argtypes = [P, C.c_int]
    lib.monte_fdk_exact_counts.argtypes = [P, C.POINTER(C.c_uint64), C.c_int]
    lib.monte_ctx_check_status.argtypes = [P]
    MG = C.POINTER(abi.McGeom)
    lib.monte_mc_geom_reference325.argtypes = [MG]
    lib.monte_mc_geom_reference325.restype = None
    lib.monte_mc_geom_reference_cpu.argtypes = [MG]
    lib.monte_mc_geom_reference_cpu.restype = None
    lib.monte_xcom_parse_csv.argtypes = [C.c_char_p, C.c_size_t] + [C.POINTER(C.c_float)] * 4
    lib.monte_mc_run.argtypes = [P, MG, C.POINTER(abi.McPhantom), C.POINTER(abi.McXcom),
                                 C.POINTER(abi.McSpectrum), C.POINTER(abi.McRequest), P, P,
                                 C.POINTER(abi.McStats), C.c_int]
    lib.monte_mc_finalize.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, P, P, P,
                                      P, P, P, C.c_int]
    dp = C.POINTER(C.c_double)
    lib.monte_spectrum_from_cumulative.argtypes = [C.POINTER(C.c_float), C.c_int32, C.c_double,
                                                   C.c_double, dp, dp, C.POINTER(C.c_int32)]
    lib.monte_parse_numbers.argtypes = [C.c_char_p, C.c_size_t, C.POINTER(C.c_float), C.c_int32,
                                        C.POINTER(C.c_int32)]
    lib.monte_mc_sample_energies.argtypes = [P, C.POINTER(abi.McSpectrum), C.c_uint64,
                                             C.c_uint32, C.c_uint64, P, C.c_int]
    lib.monte_batch_create.argtypes = [P, C.POINTER(abi.McXcom), C.POINTER(abi.BatchJob),
                                       C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p)]
    lib.monte_batch_run.argtypes = [P]
    lib.monte_batch_stats.argtypes = [P, C.POINTER(abi.McStats)]
    lib.monte_batch_bp_variant.argtypes = [P, C.c_int]
    lib.monte_batch_destroy.argtypes = [P]
    F2 = C.POINTER(abi.Fbp2Geom)
    lib.monte_fbp2_geom_reference.argtypes = [F2]
    lib.monte_fbp2_geom_reference.restype = None
    lib.monte_fbp2.argtypes = [P, F2, P, P, P, C.c_int]
    SG = C.POINTER(abi.SiddonGrid)
    lib.monte_siddon_forward.argtypes = [P, MG, SG, P, C.c_int, C.c_int, P, P, C.c_int]
    lib.monte_siddon_backward.argtypes = [P, MG, SG, P, C.c_int, C.c_int, P, P, P, C.c_int]
    _LIB = lib
    return lib


def _ptr(a):
    """(address, mem) of a torch tensor or numpy array; None -> (None, None)."""
    if a is None:
        return None, None
    if isinstance(a, np.ndarray):
        assert a.flags.c_contiguous
        return a.ctypes.data, abi.MONTE_MEM_HOST
    # torch tensor
    assert a.is_contiguous()
    return a.data_ptr(), (abi.MONTE_MEM_DEVICE if a.is_cuda else abi.MONTE_MEM_HOST)


def _mem_of(*arrays):
    mems = {m for _, m in (_ptr(a) for a in arrays if a is not None)}
    if len(mems) != 1:
        raise ValueError("all arrays of one call must live in the same memory space")
    return mems.pop()


def parse_xcom_csv(path_or_bytes):
    """monte_xcom_parse_csv: an XCOM CSV -> float32 [4][201] (coh, incoh,
    photo, total) indexed by keV.  Needs no GPU."""
    lib = load()
    if isinstance(path_or_bytes, (bytes, bytearray)):
        data = bytes(path_or_bytes)
    else:
        with open(path_or_bytes, "rb") as f:
            data = f.read()
    out = np.zeros((4, 201), np.float32)
    fp = C.POINTER(C.c_float)
    rc = lib.monte_xcom_parse_csv(data, len(data), *[out[i].ctypes.data_as(fp) for i in range(4)])
    if rc != 0:
        raise MonteError(rc, "could not parse XCOM csv")
    return out


def spectrum_from_cumulative(cum, bin_kev=0.5, fallback_kev=140.0):
    """monte_spectrum_from_cumulative: the reference's cumulative table
    cum[0..n_bins] -> (energies, weights) float64 lines, the fallback last.
    Needs no GPU."""
    lib = load()
    cum = np.ascontiguousarray(cum, np.float32)
    n_bins = len(cum) - 1
    e = np.zeros(n_bins + 1, np.float64)
    w = np.zeros(n_bins + 1, np.float64)
    n = C.c_int32()
    dp = C.POINTER(C.c_double)
    rc = lib.monte_spectrum_from_cumulative(cum.ctypes.data_as(C.POINTER(C.c_float)), n_bins,
                                            bin_kev, fallback_kev, e.ctypes.data_as(dp),
                                            w.ctypes.data_as(dp), C.byref(n))
    if rc != 0:
        raise MonteError(rc, "bad cumulative spectrum table")
    return e[:n.value], w[:n.value]


def parse_numbers(path_or_bytes, max_values=4096):
    """monte_parse_numbers: whitespace-separated numbers of a text table
    (the reference's 125kv_al*.txt) -> float32 array.  Needs no GPU."""
    lib = load()
    if isinstance(path_or_bytes, (bytes, bytearray)):
        data = bytes(path_or_bytes)
    else:
        with open(path_or_bytes, "rb") as f:
            data = f.read()
    out = np.zeros(max_values, np.float32)
    n = C.c_int32()
    rc = lib.monte_parse_numbers(data, len(data), out.ctypes.data_as(C.POINTER(C.c_float)),
                                 max_values, C.byref(n))
    if rc != 0:
        raise MonteError(rc, "could not parse the table")
    return out[:n.value].copy()


class Context:
    """One libmonte context (device + stream).  Use torch's current stream
    for device work by passing stream=torch.cuda.current_stream()."""

    def __init__(self, device=0, stream=None):
        self.lib = load()
        h = C.c_void_p()
        rc = self.lib.monte_ctx_create(C.byref(h), device)
        if rc != 0:
            raise MonteError(rc, self.lib.monte_last_error(None).decode())
        self.h = h
        if stream is not None:
            self.set_stream(stream)

    def close(self):
        if getattr(self, "h", None):
            self.lib.monte_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def check(self, rc):
        if rc != 0:
            raise MonteError(rc, self.lib.monte_last_error(self.h).decode())
        return rc

    def set_stream(self, stream):
        handle = getattr(stream, "cuda_stream", stream)
        self.check(self.lib.monte_ctx_set_stream(self.h, C.c_void_p(handle)))

    def synchronize(self):
        self.check(self.lib.monte_ctx_synchronize(self.h))

    def check_status(self):
        """Raise MonteError(MONTE_ETIMEOUT) if a bounded device wait gave up."""
        self.check(self.lib.monte_ctx_check_status(self.h))

    def fdk_autotune(self, g):
        best = C.c_int(-1)
        self.check(self.lib.monte_fdk_autotune(self.h, C.byref(g), C.byref(best)))
        return best.value

    def last_bp_variant(self):
        return self.lib.monte_fdk_last_bp_variant(self.h)

    def last_host_ranges(self):
        """View ranges of the last host-memory fdk() (0: it ran unpipelined)."""
        return self.lib.monte_fdk_last_host_ranges(self.h)

    def fdk_exact_counts(self, reset=True):
        """monte_fdk_exact_counts: (voxel-view pairs decided in double,
        (column, view) weight signs taken in double) since the last reset."""
        c = (C.c_uint64 * 2)()
        self.check(self.lib.monte_fdk_exact_counts(self.h, c, 1 if reset else 0))
        return int(c[0]), int(c[1])

    def set_bp_variant(self, variant):
        self.check(self.lib.monte_fdk_set_bp_variant(self.h, variant))

    # ---- FDK ----------------------------------------------------------
    def fdk_filter(self, g, proj, filtered, mode=abi.MONTE_FILTER_FP32):
        mem = _mem_of(proj, filtered)
        self.check(self.lib.monte_fdk_filter(self.h, C.byref(g), _ptr(proj)[0],
                                             _ptr(filtered)[0], mode, mem))

    def fdk_backproject(self, g, filtered, vol_xy, vol_zy=None, mode=abi.MONTE_BP_PLAIN):
        mem = _mem_of(filtered, vol_xy, vol_zy)
        self.check(self.lib.monte_fdk_backproject(self.h, C.byref(g), _ptr(filtered)[0],
                                                  _ptr(vol_xy)[0], _ptr(vol_zy)[0], mode, mem))

    # ---- Monte Carlo ----------------------------------------------------
    def mc_run(self, g, inputs, request, primary, scatter):
        """Add the histories of `request` into the int64 tallies; returns the
        run statistics as a dict."""
        mem = _mem_of(inputs.labels, primary, scatter)
        st = abi.McStats()
        self.check(self.lib.monte_mc_run(self.h, C.byref(g), C.byref(inputs.phantom),
                                         C.byref(inputs.xcom), C.byref(inputs.spectrum),
                                         C.byref(request), _ptr(primary)[0], _ptr(scatter)[0],
                                         C.byref(st), mem))
        return st.as_dict()

    def mc_sample_energies(self, spectrum, seed, out, job=0):
        """monte_mc_sample_energies: source energies of histories 0..n-1 of
        stream (seed, job) into out (float32[n])."""
        self.check(self.lib.monte_mc_sample_energies(self.h, C.byref(spectrum), seed, job,
                                                     out.numel() if hasattr(out, "numel")
                                                     else out.size, _ptr(out)[0],
                                                     _ptr(out)[1]))

    def mc_finalize(self, n_views, nu, nv, per, primary, scatter=None, proj0=None, map0=None,
                    proj5=None, map5=None):
        mem = _mem_of(primary, scatter, proj0, map0, proj5, map5)
        self.check(self.lib.monte_mc_finalize(self.h, n_views, nu, nv, per, _ptr(primary)[0],
                                              _ptr(scatter)[0], _ptr(proj0)[0], _ptr(map0)[0],
                                              _ptr(proj5)[0], _ptr(map5)[0], mem))

    def fdk_forward_project(self, g, vol_xy, out):
        """Adjoint of fdk_backproject (plain): vol_xy -> out[view][v][u]."""
        mem = _mem_of(vol_xy, out)
        self.check(self.lib.monte_fdk_forward_project(self.h, C.byref(g), _ptr(vol_xy)[0],
                                                      _ptr(out)[0], mem))

    def fdk_backward(self, g, grad_vol, grad_proj):
        """Adjoint of the whole FDK: grad_vol -> grad_proj[view][u][v]."""
        mem = _mem_of(grad_vol, grad_proj)
        self.check(self.lib.monte_fdk_backward(self.h, C.byref(g), _ptr(grad_vol)[0],
                                               _ptr(grad_proj)[0], mem))

    # ---- primary signal ------------------------------------------------
    def siddon_forward(self, g, grid, mu, views, line=None, transmission=None):
        mem = _mem_of(mu, line, transmission)
        self.check(self.lib.monte_siddon_forward(self.h, C.byref(g), C.byref(grid), _ptr(mu)[0],
                                                 views[0], views[1], _ptr(line)[0],
                                                 _ptr(transmission)[0], mem))

    def siddon_backward(self, g, grid, mu, views, grad_mu, grad_line=None, grad_transmission=None):
        mem = _mem_of(mu, grad_mu, grad_line, grad_transmission)
        self.check(self.lib.monte_siddon_backward(self.h, C.byref(g), C.byref(grid), _ptr(mu)[0],
                                                  views[0], views[1], _ptr(grad_line)[0],
                                                  _ptr(grad_transmission)[0], _ptr(grad_mu)[0],
                                                  mem))

    def fdk(self, g, proj, vol_xy, filtered=None, vol_zy=None,
            filter_mode=abi.MONTE_FILTER_FP32, bp_mode=abi.MONTE_BP_PLAIN):
        mem = _mem_of(proj, vol_xy, filtered, vol_zy)
        self.check(self.lib.monte_fdk(self.h, C.byref(g), _ptr(proj)[0], _ptr(filtered)[0],
                                      _ptr(vol_xy)[0], _ptr(vol_zy)[0], filter_mode, bp_mode,
                                      mem))

    # ---- 2-D fan-beam FBP --------------------------------------------------
    def fbp2(self, g, proj, image, filtered=None):
        """monte_fbp2: proj[view][det] -> image[ny][nx] (and filtered[view][det])."""
        mem = _mem_of(proj, image, filtered)
        self.check(self.lib.monte_fbp2(self.h, C.byref(g), _ptr(proj)[0], _ptr(filtered)[0],
                                       _ptr(image)[0], mem))

    # ---- batches ---------------------------------------------------------
    def batch(self, xcom, jobs, mode=abi.MONTE_BATCH_FUSED, options=0):
        """monte_batch_create over a list of abi.BatchJob; returns a Batch."""
        arr = (abi.BatchJob * len(jobs))(*jobs)
        h = C.c_void_p()
        self.check(self.lib.monte_batch_create(self.h, C.byref(xcom), arr, len(jobs), mode,
                                               options, C.byref(h)))
        return Batch(self, h)


class Batch:
    """A created batch plan (monte_batch_*); destroyed with close()."""

    def __init__(self, ctx, handle):
        self.ctx, self.h = ctx, handle

    def run(self):
        self.ctx.check(self.ctx.lib.monte_batch_run(self.h))

    def stats(self):
        st = abi.McStats()
        self.ctx.check(self.ctx.lib.monte_batch_stats(self.h, C.byref(st)))
        return st.as_dict()

    def bp_variant(self, job):
        return self.ctx.lib.monte_batch_bp_variant(self.h, job)

    def close(self):
        if self.h:
            self.ctx.lib.monte_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
