"""Benchmark of the Monte FDK hot path on GB300 (one JSON line on stdout).

Workload (default): FDK at the recon-325 size -- 360 views of a 512 (u,
in-plane) x 384 (v, axial) FP32 detector at 0.8 mm, SOD 500 mm, SDD 1000 mm,
exact line integrals of 20 seeded random ellipsoids plus N(0, 0.01^2)
noise, reconstructed into a 325^3 FP32 volume at 0.4 mm.  A step is one
full FDK (weight + ramp filter + backprojection) of that stack.  The metric
is GUPS: voxel-view updates (325^3 * 360) per second.

  value  device-resident inputs, CUDA events around K steps on the context's
         stream (inputs 283 MB > L2, so no extra L2 flush)
  e2e    the same call through the C ABI with pinned host buffers: the
         projection upload and the volume download are inside each step
         (monte_fdk overlaps them with the filter and the backprojection)
  --impl reference  the CPU oracle (a restatement of recon/bp3d20.cpp) on
         all host cores over a bounded sample, scaled to GUPS

Multi-GPU (torchrun): every rank reconstructs its own stack (replicas, weak
scaling); the step time is the max over ranks.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

import numpy as np  # noqa: E402


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--filter", default="auto", choices=["auto", "fp32", "bf16x3"])
    ap.add_argument("--bp", default="tiled", choices=["plain", "tiled"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-form FDK timing")
    ap.add_argument("--no-mc", action="store_true", help="skip the Monte Carlo timing")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-scan timing")
    ap.add_argument("--no-diff", action="store_true", help="skip the differentiable-mode timing")
    ap.add_argument("--batch-scale", type=float, default=0.1,
                    help="histories per view of the batched scans, as a fraction of 1e6-1e7")
    ap.add_argument("--tile", type=int, default=-1,
                    help="backprojection tile shape (default: autotune)")
    ap.add_argument("--small", action="store_true", help="reduced sizes (for profiling runs)")
    ap.add_argument("--mc-case", action="store_true",
                    help="only run one view of the Monte Carlo workload at 16 histories per "
                         "pixel, once per transport (the case profiled with ncu), and exit")
    return ap.parse_args()


WORKLOAD = "fdk: 360 views x 512(u) x 384(v) FP32 @0.8mm, SOD 500, SDD 1000 mm -> 325^3 FP32 @0.4mm"
# DRAM traffic per backprojection launch of WORKLOAD, by tile shape:
# dram__bytes_read.sum + dram__bytes_write.sum from one-pass ncu captures of
# `bench.py --no-mc --no-plain --no-cpu-baseline --no-batch --no-diff
# --tile T --steps 3 --warmup 3` (shapes 36-40 captured with the current
# voxel loop; the others with earlier loops, which move the same bytes)
BP_TRAFFIC = {40: 327.78e6 + 126.51e6, 39: 325.75e6 + 126.72e6, 38: 292.02e6 + 124.59e6,
              36: 306.77e6 + 125.24e6,
              33: 280.64e6 + 127.57e6, 29: 280.82e6 + 127.04e6,
              24: 342.49e6 + 144.32e6, 26: 980.36e6 + 178.60e6, 16: 904.65e6 + 164.43e6}


def geometry(small=False):
    from monte_gb300.abi import fdk_geom_recon325
    if small:
        # profiling case: the same detector and volume over 180 views (141 MB of
        # projections, above the 129 MB L2)
        return fdk_geom_recon325(n_views=180)
    return fdk_geom_recon325()


def make_input(g, device):
    from monte_gb300.phantoms import ellipsoid_line_integrals, random_ellipsoids
    ell = random_ellipsoids(1002)
    return ellipsoid_line_integrals(g, ell, noise_sigma=0.01, seed=1002, device=device)


class Clocks:
    """nvidia-smi sampler running during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.lines = []

    INTERVAL_MS = 50

    def start(self):
        """Start sampling and wait (up to 3 s) for the first sample, so that
        the region timed next is covered from its start."""
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", str(self.INTERVAL_MS), "-i", str(self.dev)],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        t = time.time()
        while not self.lines and time.time() - t < 3.0:
            time.sleep(0.01)

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append((time.time(), ln.strip()))

    def stop(self, t0=None, t1=None):
        """Summary of the samples taken in the host-time window [t0, t1]
        (plus one sampling interval), or of all samples."""
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.th.join(timeout=2)
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        lines = self.lines
        if t0 is not None:
            window = [x for x in lines if t0 <= x[0] <= t1 + self.INTERVAL_MS / 1e3]
            lines = window or [x for x in lines if x[0] >= t0][:1]
        for _, ln in lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
                power.append(float(p[3]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "power_w_max": max(power) if power else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup(args):
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world, device):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def cpu_model():
    """The host CPU's model name (lscpu), else the machine type."""
    import platform
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return platform.machine()


def cpu_baseline(g, slices_per_core=8):
    """Time the CPU oracle (FP64 restatement of recon/bp3d20.cpp, all host
    threads) on a bounded sample and scale to GUPS for the full workload:
    the filter on a few views and the backprojection on slices_per_core
    z-slices per host thread of all views (8: ~10 s on 16 cores; the
    reference arm, which repeats it every step, takes 1);
    T = n_views * t_view + updates * t_update."""
    import oracle
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    rng = np.random.Generator(np.random.PCG64(3))
    nviews_s = 8
    gs = g.copy()
    gs.n_views = nviews_s
    proj = rng.random((nviews_s, g.nu, g.nv), dtype=np.float32)
    t0 = time.perf_counter()
    oracle.fdk_filter(gs, proj)
    t_view = (time.perf_counter() - t0) / nviews_s
    filt = np.zeros((g.n_views, g.nv, g.nu), np.float32)
    filt[:] = rng.random((g.nv, g.nu), dtype=np.float32)
    nz_s = max(2, min(g.nz, slices_per_core * min(cores, 16)))
    t0 = time.perf_counter()
    oracle.fdk_backproject(g, filt, z_range=(g.nz // 2, g.nz // 2 + nz_s))
    t_bp = time.perf_counter() - t0
    upd_s = nz_s * g.nx * g.ny * g.n_views
    t_upd = t_bp / upd_s
    updates = g.nx * g.ny * g.nz * g.n_views
    T = g.n_views * t_view + updates * t_upd
    return {"value": updates / T / 1e9, "unit": "GUPS", "cores": cores, "cpu": cpu_model(),
            "kind": "port",
            "sample": "oracle filter on %d views + backprojection of %d z-slices x %d views, "
                      "scaled to the full workload (est. %.1f s per FDK)" % (nviews_s, nz_s,
                                                                            g.n_views, T)}


MC_WORKLOAD = ("mc: 325^3 labels @0.8mm (water / Ca-water bone 1.5-1.9 / air, 20 seeded "
               "ellipsoids), 20-80 keV lines weighted (80-E), 512x384 pixels @0.8mm, SOD 500, "
               "SDD 1000 mm, 509 histories per pixel per view (1.0e8 per view), 5 interactions")


def mc_workload():
    """Geometry, host labels and an inputs factory (labels -> abi.McInputs)
    of the 325^3 Monte Carlo workload."""
    from monte_gb300 import abi, phantoms
    x = np.load(os.path.join(REPO, "tests", "golden", "xcom.npz"))
    lab, vox, org, dens, mats = phantoms.ellipsoid_labels()
    E = np.arange(20.0, 81.0)

    def make(labels):
        return abi.McInputs(labels, vox, org, mats, dens, [x["water"], x["ca"]], E, 80.0 - E)

    g = abi.mc_geom(360, 512, 384, 0.08, 50.0, 100.0, 14.0, flags=abi.MONTE_MC_STALE_SIN_PHI)
    return g, lab, make


def mc_cpu_baseline(g, inp, per=32768):
    """The CPU replay harness (oracle/mc_oracle.c: the reference kernel's
    history loop restated, the same step functions and streams, all host
    cores, the reference's single majorant) on a bounded sample of the
    325^3 workload: view 0, the central 64 x 64 pixels, `per` histories
    each (1.34e8 histories, ~11 s on 16 cores)."""
    import oracle
    from monte_gb300 import abi
    cores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    u0, v0 = g.nu // 2 - 32, g.nv // 2 - 32
    req = abi.mc_request(2024, per, (0, 1), (u0, u0 + 64), (v0, v0 + 64))
    t0 = time.perf_counter()
    _, _, st = oracle.mc_run(g, inp, req)
    dt = time.perf_counter() - t0
    return {"value": st["histories"] / dt, "unit": "histories/s", "cores": cores, "cpu": cpu_model(), "kind": "port",
            "sample": "CPU replay of view 0, central 64x64 pixels, %d histories each "
                      "(%d histories, %.1f s)" % (per, st["histories"], dt)}


# Warp instructions per history and active lanes per issued instruction of
# the persistent kernel on this workload, from one ncu capture of one view
# at 16 histories per pixel per transport (`bench.py --mc-case` under ncu
# with smsp__inst_executed.sum and smsp__thread_inst_executed.sum: 3,145,728
# histories per launch), for the issue roofline of the Monte Carlo line.
MC_PROFILE = {"global": {"warp_inst_per_history": 520.7, "lanes_per_instruction": 17.95},
              "local": {"warp_inst_per_history": 240.5, "lanes_per_instruction": 12.52}}


def mc_bench(ctx, device, steps=3, per=509, with_cpu=True):
    """Histories/s on one view of the 325^3 workload (1.0e8 histories per
    step) in three forms: the plain kernel with the reference's single
    majorant (the one-instance form), the persistent kernel with it, and
    the persistent kernel with local majorants (MONTE_MC_LOCAL_MAJORANT, the
    headline)."""
    import torch
    from monte_gb300 import abi
    g, lab, make = mc_workload()
    inp = make(torch.from_numpy(lab).to(device))
    prim = torch.zeros((g.n_views, g.nu, g.nv), dtype=torch.int64, device=device)
    scat = torch.zeros_like(prim)
    out = {"metric": "MC histories/s", "unit": "histories/s", "workload": MC_WORKLOAD}
    stream = torch.cuda.current_stream(device)
    forms = (("persistent_local", abi.MONTE_MC_PERSISTENT, abi.MONTE_MC_LOCAL_MAJORANT),
             ("persistent", abi.MONTE_MC_PERSISTENT, 0),
             ("plain", abi.MONTE_MC_PLAIN, 0))
    for name, kernel, extra in forms:
        g.flags = abi.MONTE_MC_STALE_SIN_PHI | extra
        req = abi.mc_request(2024, per, (0, 1), (0, g.nu), (0, g.nv), kernel)
        st = ctx.mc_run(g, inp, req, prim, scat)  # warm-up (builds the local tables)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(device)
        e0.record(stream)
        for i in range(steps):
            req.view_begin, req.view_end = 1 + i, 2 + i
            st = ctx.mc_run(g, inp, req, prim, scat)
        e1.record(stream)
        torch.cuda.synchronize(device)
        dt = e0.elapsed_time(e1) / 1e3
        hist = steps * per * g.nu * g.nv
        h = st["histories"]
        out[name] = {"value": hist / dt, "ms_per_view": dt / steps * 1e3,
                     "woodcock_steps_per_history": st["woodcock_steps"] / h,
                     "majorant_legs_per_history": st["majorant_legs"] / h,
                     "interactions_per_history": st["interactions"] / h,
                     "rayleigh_compton_photo": [st["rayleigh"], st["compton"],
                                                st["photoelectric"]]}
    g.flags = abi.MONTE_MC_STALE_SIN_PHI
    best = out["persistent_local"]
    out["value"] = best["value"]
    out["persistent_over_plain"] = best["value"] / out["plain"]["value"]
    out["local_over_global_majorant"] = best["value"] / out["persistent"]["value"]
    # roofline: every event (Woodcock step, majorant leg, interaction) reads
    # one 32-byte sector (a label, a class cell or a table row) and every
    # history adds one 8-byte tally; the 34 MB label volume stays in L2
    ev = (best["woodcock_steps_per_history"] + best["majorant_legs_per_history"] +
          best["interactions_per_history"])
    bytes_per_hist = 32.0 * ev + 8.0
    out["roofline_l2"] = {"kernel": "mc_persistent_kernel", "bound": "l2",
                          "algorithmic_bytes_per_history": bytes_per_hist,
                          "achieved": bytes_per_hist * best["value"] / 1e9, "unit": "GB/s",
                          "note": "label gathers hit L2; no measured L2 peak in "
                                  "MEASURED_PEAKS.json, so no fraction"}
    prof = MC_PROFILE.get("local")
    if prof:
        peaks = {}
        try:
            with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
                peaks = json.load(f)
        except OSError:
            pass
        clk = float(peaks.get("sm_max_mhz", 2070.0)) * 1e6
        n_sm = torch.cuda.get_device_properties(device).multi_processor_count
        peak = n_sm * 4 * clk / 1e12  # warp instructions per second, in T/s
        ach = prof["warp_inst_per_history"] * best["value"] / 1e12
        out["roofline"] = {"kernel": "mc_persistent_kernel", "bound": "issue",
                           "achieved": ach, "peak": peak, "unit": "T warp-instructions/s",
                           "frac": ach / peak,
                           "warp_inst_per_history": prof["warp_inst_per_history"],
                           "lanes_per_instruction": prof["lanes_per_instruction"],
                           "peak_source": "%d SMs x 4 schedulers x %.0f MHz" % (n_sm, clk / 1e6)}
    if with_cpu:
        out["cpu_baseline"] = mc_cpu_baseline(g, make(lab))
    return out


BATCH_WORKLOAD = ("batch: 64 scans, cube phantoms of side U{65..257} at 0.8 mm (ellipsoids of "
                  "water / Ca-water bone 1.5-1.9 in air), views U{60..360}, detector nu in "
                  "{128..512 step 64} x nv in {128, 256, 384}, 20-80 keV lines weighted "
                  "(80-E), Monte Carlo then FDK of the total map into side^3")


def batch_bench(ctx, device, scale):
    """Wall time of the whole 64-scan batch: FUSED (one persistent Monte
    Carlo launch + per-scan BF16x3 filter and autotuned tiled backprojection,
    one CUDA graph) against SEQUENTIAL (64 x plain Monte Carlo, finalize,
    FP32 filter, plain backprojection).  Histories per view are the drawn
    1e6-1e7 times `scale`."""
    import torch
    from monte_gb300 import abi, batchscan
    x = np.load(os.path.join(REPO, "tests", "golden", "xcom.npz"))
    b = batchscan.Batch(batchscan.specs(hist_scale=scale), x["water"], x["ca"], device=device)
    H, U = b.histories(), b.updates()
    out = {"workload": BATCH_WORKLOAD, "hist_per_view_scale": scale, "histories": H,
           "voxel_view_updates": U}
    stream = torch.cuda.current_stream(device)

    def timed(plan, reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(device)
        e0.record(stream)
        for _ in range(reps):
            plan.run()
        e1.record(stream)
        torch.cuda.synchronize(device)
        return e0.elapsed_time(e1) / 1e3 / reps

    for name, mode, opts, warm in (("fused", abi.MONTE_BATCH_FUSED, abi.MONTE_BATCH_AUTOTUNE, 1),
                                   ("sequential", abi.MONTE_BATCH_SEQUENTIAL, 0, 0)):
        # the fused form transports against local majorants; the sequential
        # one-instance form keeps the reference's single majorant
        for j in b.jobs:
            if mode == abi.MONTE_BATCH_FUSED:
                j.mc.flags |= abi.MONTE_MC_LOCAL_MAJORANT
            else:
                j.mc.flags &= ~abi.MONTE_MC_LOCAL_MAJORANT
        t0 = time.time()
        plan = ctx.batch(b.xcom, b.jobs, mode=mode, options=opts)
        torch.cuda.synchronize(device)
        create_s = time.time() - t0
        for _ in range(warm):
            plan.run()
        t = timed(plan, 1)
        st = plan.stats()
        ctx.check_status()
        out[name] = {"s_per_batch": t, "histories_per_s": H / t, "gups": U / t / 1e9,
                     "create_s": create_s, "dropped": st["dropped"]}
        if name == "fused":
            out[name]["bp_variants"] = sorted({plan.bp_variant(j) for j in range(len(b.jobs))})
        plan.close()
    out["fused_over_sequential"] = out["sequential"]["s_per_batch"] / out["fused"]["s_per_batch"]
    return out


DIFF_WORKLOAD = ("differentiable mode: 257^3 FP32 at 0.8 mm, 360 views x 512 x 384 at 0.8 mm, "
                 "SOD 500, SDD 1000 mm; x, p, x* seeded ellipsoid data")


def diff_bench(ctx, device):
    """Wall time of the gradients of the differentiable mode at 257^3:
    ||A x - p||^2 w.r.t. x (forward projector A, then its adjoint, the
    backprojector), ||FDK(p) - x*||^2 w.r.t. p (FDK, then monte_fdk_backward)
    and exp(-integral mu) w.r.t. mu (Siddon forward and adjoint).  One
    warm-up and two timed calls each; CUDA events on the context's stream."""
    import torch
    from monte_gb300 import abi, phantoms
    g = abi.fdk_geom_recon325(n_views=360, nu=512, nv=384, pitch_mm=0.8, n=257, voxel_mm=0.8)
    g.flags = 0  # the textbook operator (the adjoints need no flat-edge wrap)
    stream = torch.cuda.current_stream(device)
    ell = phantoms.random_ellipsoids(1005)
    p = phantoms.ellipsoid_line_integrals(g, ell, 0.01, 5, device=device).contiguous()
    ax = (torch.arange(g.nx, device=device, dtype=torch.float64) - g.nx / 2 + 0.5) * g.dvox
    Z, Y, X = torch.meshgrid(ax, ax, ax, indexing="ij")
    x = phantoms.ellipsoid_density(ell, X, Y, Z).float().contiguous()
    xstar = phantoms.ellipsoid_density(phantoms.random_ellipsoids(1006), X, Y, Z).float().contiguous()
    del X, Y, Z
    proj_fs = torch.empty((g.n_views, g.nv, g.nu), device=device)
    vol = torch.empty_like(x)
    gp = torch.empty_like(p)

    def timed(fn, reps=2):
        fn()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize(device)
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize(device)
        return e0.elapsed_time(e1) / 1e3 / reps

    updates = g.nx * g.ny * g.nz * g.n_views
    # the tile shape for this geometry (its rows advance 2.4 per voxel, where
    # the benchmark's shape does not fit), as a caller would tune it
    bp_tile = ctx.fdk_autotune(g)
    # ||A x - p||^2: A x in filtered-space layout [view][v][u]; p transposed alike
    p_vu = p.transpose(1, 2).contiguous()

    def grad_x():
        ctx.fdk_forward_project(g, x, proj_fs)
        proj_fs.sub_(p_vu).mul_(2.0)
        ctx.fdk_backproject(g, proj_fs, vol, mode=abi.MONTE_BP_TILED)

    t_fp = timed(lambda: ctx.fdk_forward_project(g, x, proj_fs))
    t_gx = timed(grad_x)

    def grad_p():
        ctx.fdk(g, p, vol, filter_mode=abi.MONTE_FILTER_BF16X3, bp_mode=abi.MONTE_BP_TILED)
        vol.sub_(xstar).mul_(2.0)
        ctx.fdk_backward(g, vol, gp)

    t_gp = timed(grad_p)
    # primary signal: the Monte Carlo's rays through mu = x (1/cm)
    mg = abi.mc_geom(360, 512, 384, 0.08, 50.0, 100.0, 20.0)
    grid = abi.siddon_grid((g.nz, g.ny, g.nx), g.dvox, (-g.nx * g.dvox / 2,) * 3)
    tr = torch.empty((mg.n_views, mg.nu, mg.nv), device=device)
    gmu = torch.zeros_like(x)
    gt = torch.ones_like(tr)
    t_sf = timed(lambda: ctx.siddon_forward(mg, grid, x, (0, mg.n_views), transmission=tr), reps=1)
    t_sb = timed(lambda: ctx.siddon_backward(mg, grid, x, (0, mg.n_views), gmu,
                                             grad_transmission=gt), reps=1)
    ctx.check_status()
    rays = mg.n_views * mg.nu * mg.nv
    return {"workload": DIFF_WORKLOAD,
            "forward_projector": {"ms": t_fp * 1e3, "gups": updates / t_fp / 1e9},
            "bp_tile_variant": bp_tile,
            "grad_x_least_squares": {"ms": t_gx * 1e3, "note": "A x - p, then 2 A^T r (tiled)"},
            "grad_p_fdk": {"ms": t_gp * 1e3, "note": "FDK (BF16x3 + tiled), then FDK^T"},
            "siddon_forward": {"ms": t_sf * 1e3, "rays_per_s": rays / t_sf},
            "siddon_backward": {"ms": t_sb * 1e3, "rays_per_s": rays / t_sb}}


def run_reference(args):
    # rank 0 alone times the CPU implementation; no collective is needed,
    # so no process group is created
    if int(os.environ.get("RANK", "0")) != 0:
        return
    g = geometry(args.small)
    vals = []
    cb = None
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline(g, slices_per_core=1)
        if i >= args.warmup:
            vals.append(cb["value"])
    v = statistics.median(vals)
    cb["value"] = v
    mg, mlab, mmake = mc_workload()
    mc_cb = mc_cpu_baseline(mg, mmake(mlab))
    line = {"impl": "reference", "metric": "FDK GUPS (voxel-view updates/s)", "value": v,
            "unit": "GUPS", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": WORKLOAD},
            "cpu_baseline": cb,
            "mc": {"metric": "MC histories/s", "unit": "histories/s", "value": mc_cb["value"],
                   "workload": MC_WORKLOAD, "cpu_baseline": mc_cb},
            "e2e": {"value": v, "unit": "GUPS", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    world, rank, local = dist_setup(args)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from monte_gb300 import abi
    from monte_gb300.lib import Context
    g = geometry(args.small)
    stream = torch.cuda.current_stream(dev)
    ctx = Context(local, stream=stream)
    fmode = {"auto": abi.MONTE_FILTER_BF16X3, "fp32": abi.MONTE_FILTER_FP32,
             "bf16x3": abi.MONTE_FILTER_BF16X3}[args.filter]
    if args.filter == "auto":
        try:  # the tensor-core filter needs nu % 64 == 0 and nv % 128 == 0
            pt = torch.zeros((1, 64, 128), device=dev)
            gt = g.copy()
            gt.n_views, gt.nu, gt.nv = 1, 64, 128
            ctx.fdk_filter(gt, pt, torch.empty_like(pt), mode=fmode)
        except Exception:
            fmode = abi.MONTE_FILTER_FP32
    bmode = abi.MONTE_BP_TILED if args.bp == "tiled" else abi.MONTE_BP_PLAIN

    proj = make_input(g, dev)
    if args.tile >= 0:
        tile = args.tile
        ctx.set_bp_variant(tile)
    else:
        tile = ctx.fdk_autotune(g) if bmode == abi.MONTE_BP_TILED else -1
    filt = torch.empty((g.n_views, g.nv, g.nu), dtype=torch.float32, device=dev)
    vol = torch.empty((g.nz, g.ny, g.nx), dtype=torch.float32, device=dev)
    updates = g.nx * g.ny * g.nz * g.n_views

    def step():
        ctx.fdk_filter(g, proj, filt, mode=fmode)
        ctx.fdk_backproject(g, filt, vol, mode=bmode)

    clocks = Clocks(local)
    clocks.start()
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize(dev)
    h0 = time.time()
    t_all0 = torch.cuda.Event(enable_timing=True)
    t_all1 = torch.cuda.Event(enable_timing=True)
    t_all0.record(stream)
    for i in range(args.steps):
        ev[i][0].record(stream)
        ctx.fdk_filter(g, proj, filt, mode=fmode)
        ev[i][1].record(stream)
        ctx.fdk_backproject(g, filt, vol, mode=bmode)
        ev[i][2].record(stream)
    t_all1.record(stream)
    torch.cuda.synchronize(dev)
    h1 = time.time()
    barrier(world)
    clk = clocks.stop(h0, h1)
    elapsed = t_all0.elapsed_time(t_all1) / 1e3
    elapsed = max_over_ranks(elapsed, world, dev)
    t_filter = statistics.mean(e[0].elapsed_time(e[1]) for e in ev) / 1e3
    t_bp = statistics.mean(e[1].elapsed_time(e[2]) for e in ev) / 1e3
    ms_per_step = elapsed / args.steps * 1e3
    value = world * updates * args.steps / elapsed / 1e9

    # how much of one backprojection left FP32: voxel-view pairs decided in
    # double next to the operator's discontinuities, weight signs in double
    exact = None
    if bmode == abi.MONTE_BP_TILED:
        ctx.fdk_exact_counts(reset=True)
        ctx.fdk_backproject(g, filt, vol, mode=bmode)
        n_pairs, n_signs = ctx.fdk_exact_counts(reset=True)
        n_cols = g.nx * g.ny * g.n_views
        exact = {"voxel_view_pairs_in_double": n_pairs, "share_of_updates": n_pairs / updates,
                 "weight_signs_in_double": n_signs, "share_of_column_views": n_signs / n_cols}

    # end to end through the C ABI with pinned host buffers
    h_proj = proj.cpu().pin_memory()
    h_vol = torch.empty((g.nz, g.ny, g.nx), dtype=torch.float32).pin_memory()
    for _ in range(2):
        ctx.fdk(g, h_proj, h_vol, filter_mode=fmode, bp_mode=bmode)
    barrier(world)
    t0 = time.perf_counter()
    n_e2e = max(3, args.steps // 2)
    for _ in range(n_e2e):
        ctx.fdk(g, h_proj, h_vol, filter_mode=fmode, bp_mode=bmode)
    t_e2e = time.perf_counter() - t0
    t_e2e = max_over_ranks(t_e2e, world, dev)
    e2e_val = world * updates * n_e2e / t_e2e / 1e9
    e2e_ranges = ctx.last_host_ranges()
    # the host link's rates on this machine, one pinned copy each way of the
    # same buffers (the end-to-end figure follows them: only the first
    # view range's upload and the last range's volume store are exposed)
    d_tmp = torch.empty_like(proj)
    h2d, d2h = [], []
    for _ in range(3):
        c0, c1, c2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        c0.record()
        d_tmp.copy_(h_proj, non_blocking=True)
        c1.record()
        h_vol.copy_(vol, non_blocking=True)
        c2.record()
        c2.synchronize()
        h2d.append(h_proj.numel() * 4 / (c0.elapsed_time(c1) / 1e3) / 1e9)
        d2h.append(h_vol.numel() * 4 / (c1.elapsed_time(c2) / 1e3) / 1e9)
    del d_tmp, h_vol

    peaks = {}
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    sm_max = float(peaks.get("sm_max_mhz", 2070.0))
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = n_sm * 128 * 2 * sm_max * 1e6 / 1e12  # TFLOP/s
    bp_flops = 10.0 * updates
    bp_bytes = g.n_views * g.nu * g.nv * 4 + g.nx * g.ny * g.nz * 4
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    # DRAM bytes (read + write) of one backprojection launch of this workload,
    # from one-pass ncu captures (dram__bytes_read.sum + dram__bytes_write.sum)
    # of the tile shapes that lead it
    traffic = BP_TRAFFIC.get(ctx.last_bp_variant()) if not args.small else None

    line = {
        "metric": "FDK GUPS (voxel-view updates/s)", "value": value, "unit": "GUPS",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD if not args.small else "reduced (profiling) " + WORKLOAD,
                   "filter": {abi.MONTE_FILTER_FP32: "fp32", abi.MONTE_FILTER_BF16X3: "bf16x3"}[fmode],
                   "backprojector": args.bp, "bp_tile_variant": ctx.last_bp_variant(),
                   "autotuned_tile": tile,
                   "l2": "inputs 283 MB > 129 MB L2 (no flush)",
                   "parallelism": "replicas" if world > 1 else "single"},
        "breakdown_ms": {"filter": t_filter * 1e3, "backprojection": t_bp * 1e3},
        "roofline": {"kernel": "backprojection", "bound": "fp32",
                     "achieved": bp_flops / t_bp / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": bp_flops / t_bp / 1e12 / fp32_peak, "traffic": traffic,
                     "peak_source": "%d SMs x 128 FP32 lanes x 2 x %.0f MHz (sm_max_mhz of "
                                    "MEASURED_PEAKS.json)" % (n_sm, sm_max),
                     "algorithmic": "10 flop per voxel-view update"},
        "roofline_hbm": {"kernel": "backprojection", "bound": "hbm",
                         "achieved": bp_bytes / t_bp / 1e9, "peak": hbm_peak, "unit": "GB/s",
                         "frac": bp_bytes / t_bp / 1e9 / hbm_peak, "traffic": traffic},
        # the pipe the voxel loop saturates first: its four bilinear taps per
        # update come from the shared-memory tile, one warp-wide 4-byte load
        # each, and shared memory delivers 128 bytes per cycle per SM
        "roofline_smem": {"kernel": "backprojection", "bound": "shared-memory loads",
                          "achieved": 16.0 * updates / t_bp / 1e9,
                          "peak": n_sm * 128 * sm_max * 1e6 / 1e9, "unit": "GB/s",
                          "frac": 16.0 * updates / t_bp / (n_sm * 128 * sm_max * 1e6),
                          "algorithmic": "4 FP32 taps (16 B) per voxel-view update",
                          "peak_source": "%d SMs x 128 B x %.0f MHz" % (n_sm, sm_max)},
        "e2e": {"value": e2e_val, "unit": "GUPS",
                "h2d_bytes_per_step": int(g.n_views * g.nu * g.nv * 4),
                "d2h_bytes_per_step": int(g.nx * g.ny * g.nz * 4),
                "pipeline_view_ranges": e2e_ranges, "fraction_of_value": e2e_val / value,
                "h2d_gbs": statistics.median(h2d), "d2h_gbs": statistics.median(d2h)},
        "gpu_launches": 2 * args.steps,
        "exact_path": exact,
        "clocks": clk,
    }
    # the plain one-instance FP32 form of the same FDK (FP32 filter, one voxel
    # per thread backprojection), for the tuned-over-plain ratio
    if not args.no_plain:
        ctx.fdk(g, proj, vol, filtered=filt, filter_mode=abi.MONTE_FILTER_FP32,
                bp_mode=abi.MONTE_BP_PLAIN)
        torch.cuda.synchronize(dev)
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        n_plain = 3
        p0.record(stream)
        for _ in range(n_plain):
            ctx.fdk(g, proj, vol, filtered=filt, filter_mode=abi.MONTE_FILTER_FP32,
                    bp_mode=abi.MONTE_BP_PLAIN)
        p1.record(stream)
        torch.cuda.synchronize(dev)
        t_plain = p0.elapsed_time(p1) / 1e3 / n_plain
        line["fdk_plain"] = {"value": updates / t_plain / 1e9, "unit": "GUPS",
                             "ms_per_step": t_plain * 1e3,
                             "tuned_over_plain": value / world / (updates / t_plain / 1e9)}
    if not args.no_mc:
        line["mc"] = mc_bench(ctx, dev, with_cpu=rank == 0 and not args.no_cpu_baseline)
        line["gpu_launches_mc"] = 3 * 4
    if not args.no_batch and not args.small:
        line["batch"] = batch_bench(ctx, dev, args.batch_scale)
    if not args.no_diff and not args.small:
        line["diff"] = diff_bench(ctx, dev)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(g)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def mc_case():
    """One view of the 325^3 Monte Carlo workload at 16 histories per pixel
    with the single majorant, then with local majorants: two launches of the
    persistent kernel, small enough to capture with ncu."""
    import torch
    from monte_gb300 import abi
    from monte_gb300.lib import Context
    g, lab, make = mc_workload()
    inp = make(torch.from_numpy(lab).cuda())
    ctx = Context(0, stream=torch.cuda.current_stream())
    for extra in (0, abi.MONTE_MC_LOCAL_MAJORANT):
        g.flags = abi.MONTE_MC_STALE_SIN_PHI | extra
        prim = torch.zeros((g.n_views, g.nu, g.nv), dtype=torch.int64, device="cuda")
        scat = torch.zeros_like(prim)
        st = ctx.mc_run(g, inp, abi.mc_request(2024, 16, (0, 1), (0, g.nu), (0, g.nv)), prim, scat)
        torch.cuda.synchronize()
        print(json.dumps({"flags": g.flags, "stats": st}), flush=True)
    ctx.close()


def main():
    args = parse()
    if args.mc_case:
        mc_case()
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
