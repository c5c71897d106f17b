"""Monte Carlo on the GPU through the C ABI.

* Seeded replay: the plain and the persistent kernels produce int64 tallies
  bit-equal to the CPU replay harness (same Philox streams, same step
  functions), for monochromatic and polychromatic sources and every physics
  switch.
* Physics: chi-square against the reference CPU program's 10^7-history
  scatter image (tests/golden/cbct_real2.npz).
* Post-processing equals the reference formula (CBCT_real325im.cu:261-294).
"""
import numpy as np
import pytest
import torch

import oracle
from helpers import block_sum, chi2_two_sample, golden
from monte_gb300 import abi, phantoms

pytestmark = pytest.mark.gpu


def cfg1_inputs(device=None, spectrum="mono"):
    x = golden("xcom")
    lab, vox, org = phantoms.cylinder_inserts_labels()
    if device is not None:
        lab = torch.from_numpy(lab).to(device)
    if spectrum == "mono":
        E, W = [60.0], None
    else:
        E = np.arange(20.0, 81.0)
        W = 80.0 - E
    return abi.McInputs(lab, vox, org, [-1, 0, 1, 1, 1], [0.0, 1.0, 1.2, 1.5, 1.9],
                        [x["water"], x["ca"]], E, W)


def cfg1_geom(flags=abi.MONTE_MC_STALE_SIN_PHI):
    # 64x64 pixels of 1 mm, SOD 500 mm, SDD 1000 mm, 90 views
    return abi.mc_geom(90, 64, 64, 0.1, 50.0, 100.0, 3.5, flags=flags)


def _gpu_run(ctx, g, inp_dev, req):
    prim = torch.zeros((g.n_views, g.nu, g.nv), dtype=torch.int64, device="cuda")
    scat = torch.zeros_like(prim)
    st = ctx.mc_run(g, inp_dev, req, prim, scat)
    ctx.synchronize()
    return prim.cpu().numpy(), scat.cpu().numpy(), st


@pytest.mark.parametrize("spectrum", ["mono", "poly"])
@pytest.mark.parametrize("flags", [abi.MONTE_MC_STALE_SIN_PHI, 0,
                                   abi.MONTE_MC_FIRST_COMPTON_Z | abi.MONTE_MC_NO_RAYLEIGH_TALLY,
                                   abi.MONTE_MC_STALE_SIN_PHI | abi.MONTE_MC_LOCAL_MAJORANT])
def test_replay_is_bit_exact(ctx, spectrum, flags):
    g = cfg1_geom(flags)
    host = cfg1_inputs(None, spectrum)
    dev = cfg1_inputs("cuda", spectrum)
    req = abi.mc_request(31337, 6, (10, 13), (0, 64), (0, 64))
    p_ref, s_ref, st_ref = oracle.mc_run(g, host, req)
    assert s_ref.sum() > 0 and p_ref.sum() > 0
    for kernel in (abi.MONTE_MC_PLAIN, abi.MONTE_MC_PERSISTENT):
        req.kernel = kernel
        p, s, st = _gpu_run(ctx, g, dev, req)
        assert np.array_equal(p, p_ref), kernel
        assert np.array_equal(s, s_ref), kernel
        assert st["histories"] == st_ref["histories"]
        assert st["woodcock_steps"] == st_ref["woodcock_steps"]
        assert st["interactions"] == st_ref["interactions"]
        for kind in ("rayleigh", "compton", "photoelectric"):
            assert st[kind] == st_ref[kind], (kernel, kind)
        assert st["rayleigh"] + st["compton"] + st["photoelectric"] == st["interactions"]
        assert st["majorant_legs"] == st_ref["majorant_legs"]
        assert (st["majorant_legs"] > 0) == bool(flags & abi.MONTE_MC_LOCAL_MAJORANT)


def test_local_majorant_tables_follow_the_labels(ctx):
    """The context keeps the local-majorant tables of its last phantom and
    reuses them while the labels are the same bytes (checked on the device
    against its copy).  Labels changed in place between two calls on the
    same buffer must rebuild them: the second run equals the CPU replay of
    the changed phantom, and the label check then reuses the new tables."""
    g = cfg1_geom(abi.MONTE_MC_STALE_SIN_PHI | abi.MONTE_MC_LOCAL_MAJORANT)
    dev = cfg1_inputs("cuda")
    req = abi.mc_request(4242, 4, (3, 5), (0, 64), (0, 64))
    _gpu_run(ctx, g, dev, req)  # builds and keeps the tables
    host = cfg1_inputs(None)
    lab = host.labels.copy()
    # turn a slab of the cylinder into the densest insert's label: a
    # material the old tables' majorants around it do not cover
    dense = int(lab.max())
    slab = lab[20:45, 10:30, 25:40]
    lab[20:45, 10:30, 25:40] = np.where(slab > 0, dense, slab)
    dev.labels.copy_(torch.from_numpy(lab).to(dev.labels.device))
    host.labels[...] = lab  # the same array the phantom struct points at
    p_ref, s_ref, st_ref = oracle.mc_run(g, host, req)
    for _ in range(2):  # rebuilt, then reused
        p, s, st = _gpu_run(ctx, g, dev, req)
        assert np.array_equal(p, p_ref) and np.array_equal(s, s_ref)
        assert st["majorant_legs"] == st_ref["majorant_legs"]


def test_split_runs_sum_to_the_whole(ctx):
    """Any partition of (views, pixels) reproduces the single run's tallies:
    the sharding contract for multi-GPU runs."""
    g = cfg1_geom()
    dev = cfg1_inputs("cuda")
    whole = _gpu_run(ctx, g, dev, abi.mc_request(9, 5, (0, 4), (0, 64), (0, 64)))
    prim = torch.zeros((g.n_views, g.nu, g.nv), dtype=torch.int64, device="cuda")
    scat = torch.zeros_like(prim)
    for views in ((0, 1), (1, 4)):
        for us in ((0, 20), (20, 64)):
            ctx.mc_run(g, dev, abi.mc_request(9, 5, views, us, (0, 64)), prim, scat)
    ctx.synchronize()
    assert np.array_equal(prim.cpu().numpy(), whole[0])
    assert np.array_equal(scat.cpu().numpy(), whole[1])


@pytest.mark.parametrize("kernel", [abi.MONTE_MC_PLAIN, abi.MONTE_MC_PERSISTENT])
def test_scatter_image_matches_cbct_real2(ctx, kernel):
    gold = golden("cbct_real2")
    n = int(gold["histories"])
    x = golden("xcom")
    lab = torch.from_numpy(phantoms.sphere_labels_185()).cuda()
    inp = abi.McInputs(lab, phantoms.SPHERE185_VOXEL, phantoms.SPHERE185_ORIGIN, [-1, 0],
                       [0.0, 1.0], [x["water"]], [140.0])
    g = abi.mc_geom_reference_cpu()
    p, s, st = _gpu_run(ctx, g, inp, abi.mc_request(77, n, (0, 1), (32, 33), (32, 33), kernel))
    assert st["histories"] == n and st["dropped"] == 0
    for k in (1, 5):
        x2, dof, pv = chi2_two_sample(block_sum(s[0], k), block_sum(gold["image"], k), n, n)
        assert pv > 1e-3, (k, x2, dof, pv)


def test_finalize_matches_reference_formula(ctx):
    rng = np.random.default_rng(3)
    per = 2000
    prim = rng.integers(0, 2500, size=(4, 8, 8)).astype(np.int64)
    prim[0, 0, :3] = 0
    scat = rng.integers(0, 300, size=(4, 8, 8)).astype(np.int64)
    outs = [np.zeros((4, 8, 8), np.int32), np.zeros((4, 8, 8), np.float32),
            np.zeros((4, 8, 8), np.int32), np.zeros((4, 8, 8), np.float32)]
    ctx.mc_finalize(4, 8, 8, per, prim, scat, *outs)
    for tally, proj, mp in ((prim, outs[0], outs[1]), (prim + scat, outs[2], outs[3])):
        n = np.clip(tally, None, per)
        n[n == 0] = 1
        assert np.array_equal(proj, n.astype(np.int32))
        want = (-np.log(n.astype(np.float64)) + np.float64(np.float32(np.log(per)))).astype(np.float32)
        assert np.array_equal(mp, want)


def test_host_memory_path(ctx):
    g = cfg1_geom()
    req = abi.mc_request(4, 3, (0, 2), (0, 64), (0, 64))
    d = _gpu_run(ctx, g, cfg1_inputs("cuda"), req)
    host = cfg1_inputs(None)
    prim = np.zeros((g.n_views, g.nu, g.nv), np.int64)
    scat = np.zeros_like(prim)
    ctx.mc_run(g, host, req, prim, scat)
    assert np.array_equal(prim, d[0]) and np.array_equal(scat, d[1])


def test_bad_arguments(ctx):
    from monte_gb300.lib import MonteError
    g = cfg1_geom()
    dev = cfg1_inputs("cuda")
    prim = torch.zeros((g.n_views, g.nu, g.nv), dtype=torch.int64, device="cuda")
    for bad in (dict(view_end=91), dict(u_end=65), dict(kernel=5)):
        req = abi.mc_request(1, 1, (0, 1), (0, 64), (0, 64))
        for k, v in bad.items():
            setattr(req, k, v)
        with pytest.raises(MonteError) as e:
            ctx.mc_run(g, dev, req, prim, prim.clone())
        assert e.value.code == abi.MONTE_EINVAL
    g.sdd = 10.0  # detector inside the source distance
    with pytest.raises(MonteError):
        ctx.mc_run(g, dev, abi.mc_request(1, 1, (0, 1), (0, 64), (0, 64)), prim, prim.clone())
    # MONTE_MEM_DEVICE with a pageable host tally: rejected before any work
    # (the kernel would fault on it)
    import ctypes as C
    g = cfg1_geom()
    host = np.zeros((g.n_views, g.nu, g.nv), np.int64)
    st = abi.McStats()
    rc = ctx.lib.monte_mc_run(ctx.h, C.byref(g), C.byref(dev.phantom), C.byref(dev.xcom),
                              C.byref(dev.spectrum), C.byref(abi.mc_request(1, 1, (0, 1), (0, 64), (0, 64))),
                              host.ctypes.data, prim.data_ptr(), C.byref(st), abi.MONTE_MEM_DEVICE)
    assert rc == abi.MONTE_EINVAL
    assert int(prim.abs().sum()) == 0


def test_empty_requests_change_nothing(ctx):
    """Empty view or pixel ranges and zero histories per pixel are valid
    requests that run no history and leave the tallies as they were."""
    g = cfg1_geom(abi.MONTE_MC_STALE_SIN_PHI | abi.MONTE_MC_LOCAL_MAJORANT)
    dev = cfg1_inputs("cuda")
    prim = torch.full((g.n_views, g.nu, g.nv), 7, dtype=torch.int64, device="cuda")
    scat = torch.full_like(prim, 3)
    for req in (abi.mc_request(9, 4, (5, 5), (0, 64), (0, 64)),
                abi.mc_request(9, 4, (0, 2), (10, 10), (0, 64)),
                abi.mc_request(9, 4, (0, 2), (0, 64), (64, 64)),
                abi.mc_request(9, 0, (0, 2), (0, 64), (0, 64))):
        for kernel in (abi.MONTE_MC_PLAIN, abi.MONTE_MC_PERSISTENT):
            req.kernel = kernel
            st = ctx.mc_run(g, dev, req, prim, scat)
            ctx.synchronize()
            assert st["histories"] == 0, (kernel, st)
    assert bool((prim == 7).all()) and bool((scat == 3).all())


def test_fan_beam_one_row_detector_replay(ctx):
    """2-D (fan-beam) Monte Carlo with the same kernels.  The phantom is one
    z-invariant slice of the cylinder phantom (one voxel 100 cm tall) and
    the detector one row as tall, so every photon that reaches the detector
    line is tallied whatever its height: the set-up of the reference's 2-D
    programs (monte_cpp/c3_l.cpp: a 65x65 label image, a 65-bin detector row
    per angle).  Seeded replay stays bit-exact with the CPU harness."""
    lab, vox, org = phantoms.cylinder_inserts_labels()
    x = golden("xcom")
    sl = np.ascontiguousarray(lab[32:33])

    def inputs(labels):
        return abi.McInputs(labels, (vox, vox, 100.0), (org[0], org[1], -50.0),
                            [-1, 0, 1, 1, 1], [0.0, 1.0, 1.2, 1.5, 1.9],
                            [x["water"], x["ca"]], np.arange(20.0, 81.0), 80.0 - np.arange(20.0, 81.0))

    host, dev = inputs(sl), inputs(torch.from_numpy(sl).cuda())
    g = abi.mc_geom(60, 64, 1, 0.1, 50.0, 100.0, 3.5)
    g.dv, g.half_v = 100.0, 50.0
    req = abi.mc_request(4242, 64, (0, 6), (0, 64), (0, 1))
    p_ref, s_ref, st_ref = oracle.mc_run(g, host, req)
    assert p_ref.shape == (60, 64, 1) and p_ref.sum() > 0 and s_ref.sum() > 0
    for kernel in (abi.MONTE_MC_PLAIN, abi.MONTE_MC_PERSISTENT):
        req.kernel = kernel
        p, s, st = _gpu_run(ctx, g, dev, req)
        assert np.array_equal(p, p_ref), kernel
        assert np.array_equal(s, s_ref), kernel
        assert st["interactions"] == st_ref["interactions"]
