"""monte_mc_run_noalloc: the Monte Carlo entry point for callers that cannot
allocate device memory (a service that reserves all GPU memory for its own
pool, a framework whose allocator owns every device allocation, a loop
where a cudaMalloc would stall the device).  It keeps its scratch in a
static device array shared by all calls, so this test calls it twice in a
row, through the C ABI, and checks each result against monte_mc_run, the
entry point that allocates its scratch per context.  Tallies are integer
counts from the same random streams: they must be equal, bit for bit.

This file is collected last; it needs nothing from the other tests and also
passes on its own in a fresh process."""
import ctypes as C

import numpy as np
import pytest
import torch

from helpers import golden
from monte_gb300 import abi, phantoms
from monte_gb300.lib import load

pytestmark = pytest.mark.gpu


def _inputs():
    x = golden("xcom")
    lab, vox, org = phantoms.cylinder_inserts_labels()
    E = np.arange(20.0, 81.0)
    return abi.McInputs(torch.from_numpy(lab).cuda(), vox, org, [-1, 0, 1, 1, 1],
                        [0.0, 1.0, 1.2, 1.5, 1.9], [x["water"], x["ca"]], E, 80.0 - E)


def _noalloc(lib, g, inp, req, prim, scat):
    lib.monte_mc_run_noalloc.argtypes = [C.POINTER(abi.McGeom), C.POINTER(abi.McPhantom),
                                         C.POINTER(abi.McXcom), C.POINTER(abi.McSpectrum),
                                         C.POINTER(abi.McRequest), C.c_void_p, C.c_void_p,
                                         C.POINTER(abi.McStats), C.c_void_p]
    st = abi.McStats()
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.monte_mc_run_noalloc(C.byref(g), C.byref(inp.phantom), C.byref(inp.xcom),
                                  C.byref(inp.spectrum), C.byref(req), prim.data_ptr(),
                                  scat.data_ptr(), C.byref(st), C.c_void_p(stream))
    assert rc == 0, lib.monte_last_error(None)
    return st.as_dict()


def test_noalloc_equals_allocating_entry_point_twice(ctx):
    lib = load()
    inp = _inputs()
    g = abi.mc_geom(90, 64, 64, 0.1, 50.0, 100.0, 3.5, flags=abi.MONTE_MC_STALE_SIN_PHI)
    requests = [abi.mc_request(101, 5, (0, 3), (0, 64), (0, 64), abi.MONTE_MC_PERSISTENT),
                abi.mc_request(202, 3, (7, 9), (10, 50), (0, 64), abi.MONTE_MC_PERSISTENT)]
    for req in requests:  # two calls in a row on the shared static scratch
        p0 = torch.zeros((g.n_views, g.nu, g.nv), dtype=torch.int64, device="cuda")
        s0 = torch.zeros_like(p0)
        st0 = ctx.mc_run(g, inp, req, p0, s0)
        p1 = torch.zeros_like(p0)
        s1 = torch.zeros_like(p0)
        st1 = _noalloc(lib, g, inp, req, p1, s1)
        torch.cuda.synchronize()
        assert torch.equal(p0, p1) and torch.equal(s0, s1)
        assert st1 == st0
        assert st1["histories"] == req.histories_per_pixel * (req.view_end - req.view_begin) * \
            (req.u_end - req.u_begin) * (req.v_end - req.v_begin)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = load()
    inp = _inputs()
    g = abi.mc_geom(2048, 64, 64, 0.1, 50.0, 100.0, 3.5)
    p = torch.zeros(1, dtype=torch.int64, device="cuda")
    lib.monte_mc_run_noalloc.argtypes = [C.POINTER(abi.McGeom), C.POINTER(abi.McPhantom),
                                         C.POINTER(abi.McXcom), C.POINTER(abi.McSpectrum),
                                         C.POINTER(abi.McRequest), C.c_void_p, C.c_void_p,
                                         C.POINTER(abi.McStats), C.c_void_p]
    rc = lib.monte_mc_run_noalloc(C.byref(g), C.byref(inp.phantom), C.byref(inp.xcom),
                                  C.byref(inp.spectrum),
                                  C.byref(abi.mc_request(1, 1, (0, 1), (0, 64), (0, 64))),
                                  p.data_ptr(), p.data_ptr(), None, None)
    assert rc == abi.MONTE_EINVAL
    assert b"static scratch" in lib.monte_last_error(None)


def test_noalloc_back_to_back_without_sync_and_plain_kernel(ctx):
    """Two calls queued on one stream with no statistics (so no wait in
    between: the second call's tables overwrite the shared array while the
    first kernel may still be queued -- stream order keeps them apart),
    then one synchronize; the plain kernel as well as the persistent one."""
    lib = load()
    inp = _inputs()
    g = abi.mc_geom(90, 64, 64, 0.1, 50.0, 100.0, 3.5, flags=abi.MONTE_MC_STALE_SIN_PHI)
    lib.monte_mc_run_noalloc.argtypes = [C.POINTER(abi.McGeom), C.POINTER(abi.McPhantom),
                                         C.POINTER(abi.McXcom), C.POINTER(abi.McSpectrum),
                                         C.POINTER(abi.McRequest), C.c_void_p, C.c_void_p,
                                         C.POINTER(abi.McStats), C.c_void_p]
    requests = [abi.mc_request(303, 4, (2, 4), (0, 64), (0, 64), abi.MONTE_MC_PLAIN),
                abi.mc_request(404, 2, (5, 8), (8, 56), (4, 60), abi.MONTE_MC_PERSISTENT)]
    outs = []
    stream = torch.cuda.current_stream().cuda_stream
    for req in requests:
        p = torch.zeros((g.n_views, g.nu, g.nv), dtype=torch.int64, device="cuda")
        s = torch.zeros_like(p)
        rc = lib.monte_mc_run_noalloc(C.byref(g), C.byref(inp.phantom), C.byref(inp.xcom),
                                      C.byref(inp.spectrum), C.byref(req), p.data_ptr(),
                                      s.data_ptr(), None, C.c_void_p(stream))
        assert rc == 0, lib.monte_last_error(None)
        outs.append((p, s))
    torch.cuda.synchronize()
    for req, (p, s) in zip(requests, outs):
        p0 = torch.zeros_like(p)
        s0 = torch.zeros_like(p)
        ctx.mc_run(g, inp, req, p0, s0)
        torch.cuda.synchronize()
        assert torch.equal(p, p0) and torch.equal(s, s0), req.kernel


def test_noalloc_rejects_host_pointers_and_capture():
    lib = load()
    inp = _inputs()
    g = abi.mc_geom(90, 64, 64, 0.1, 50.0, 100.0, 3.5, flags=abi.MONTE_MC_STALE_SIN_PHI)
    req = abi.mc_request(5, 1, (0, 1), (0, 64), (0, 64))
    lib.monte_mc_run_noalloc.argtypes = [C.POINTER(abi.McGeom), C.POINTER(abi.McPhantom),
                                         C.POINTER(abi.McXcom), C.POINTER(abi.McSpectrum),
                                         C.POINTER(abi.McRequest), C.c_void_p, C.c_void_p,
                                         C.POINTER(abi.McStats), C.c_void_p]
    host = np.zeros((g.n_views, g.nu, g.nv), np.int64)
    dev = torch.zeros((g.n_views, g.nu, g.nv), dtype=torch.int64, device="cuda")
    rc = lib.monte_mc_run_noalloc(C.byref(g), C.byref(inp.phantom), C.byref(inp.xcom),
                                  C.byref(inp.spectrum), C.byref(req), host.ctypes.data,
                                  dev.data_ptr(), None, None)
    assert rc == abi.MONTE_EINVAL
    # a capturing stream: refused before any work is issued
    s = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        graph.capture_begin(capture_error_mode="relaxed")
        rc = lib.monte_mc_run_noalloc(C.byref(g), C.byref(inp.phantom), C.byref(inp.xcom),
                                      C.byref(inp.spectrum), C.byref(req), dev.data_ptr(),
                                      dev.data_ptr(), None, C.c_void_p(s.cuda_stream))
        graph.capture_end()
    assert rc == abi.MONTE_EUNSUPPORTED
