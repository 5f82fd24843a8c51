#!/usr/bin/env python
"""Benchmark of the GB300 SPH particle pipeline: particle-updates/s.

Default workload: WCSPH double dam break, 4,194,304 fluid particles (two 128^3 lattice blocks
at dx = 0.005 m, h = 0.01 m, dt = 5e-5 s) in a 2x1x1 m container of ~321k boundary particles,
PHYSICS mode, FP32.  A step is one sph_simulate() (one CUDA-graph replay): bin, onesweep sort,
reorder, cell ranges, density/pressure, normals, forces with fused leapfrog integration.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload ...]

Prints ONE JSON line (rank 0).  value = N_fluid x K x ranks / max-over-ranks device time of K
steps (CUDA events on the context stream; inputs larger than L2 every step).  e2e repeats the
metric through the C ABI with host buffers (pinned), copying the particle state in and the
step's result out every step.  With several GPUs each rank runs an independent replica
(the single-scene path has no data-parallel split without a halo exchange).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "particle-updates/s (WCSPH/PCISPH @4M); batched & adjoint vs plain, same GPU"
UNIT = "particle-updates/s"
PEAKS_FILE = os.path.join(ROOT, "MEASURED_PEAKS.json")
FALLBACK_HBM_GBS = 6800.0

# Algorithmic HBM bytes per fluid particle of each kernel (compulsory traffic; neighbour data
# is assumed to come from L1/L2).  The list-based kernels also move their neighbour lists:
# LIST_BYTES[k] = (bytes per fluid-list entry, bytes per boundary-list entry, fixed bytes),
# multiplied by the step's mean list lengths.
ALG_BYTES = {
    "k_hashes": 16 + 4 + 4 + 4 + 8,          # pos in; key, mask out; cell_prev in; clear 8 B/cell (upper bound)
    "k_gather": 4 + 3 * 16 * 2 + 4 * 2,      # perm; pos/vel/vhalf gathered and written; ids
    "k_cell_ranges": 16 + 8 + 4 + 8,         # sorted pos, 2 keys, cell id out, range writes (per cell)
    "k_gather_ranges": 4 + 3 * 16 * 2 + 4 * 2 + 8 + 4 + 8,   # the gather + keys, cell id out, range writes
    "k_wc_density": 16 + 8,                  # own position; density and pressure out
    "k_lists_density": 16 + 8 + 16 + 16,     # own position; density, pressure, aux, (x, y, z, rho) out (+ lists)
    "k_normals": 16 + 16,                    # own position; normal out (+ the fluid list it reads)
    "k_wc_forces": 16 * 3 + 4 + 4 + 16 + 4 + 16 * 3 + 4,   # pos,vel,vhalf,rho,p,normal,id in; pos,vel,vhalf,id out
}
LIST_BYTES = {
    "k_lists_density": (4, 4, 8),            # entries written, two lengths written
    "k_normals": (4, 0, 4),                  # fluid entries read, its length read
    "k_wc_forces": (4, 4, 8),                # both lists read, both lengths read
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["wcsph4m", "wcsph1m", "wcsph65k", "pcisph", "pcisph4m"], default="wcsph4m",
                    help="wcsph1m: the 4M scene's blocks at 80^3 (profiling case)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--neighbor-mode", type=int, default=1, help="0 = cell scan in every pass, 1 = lists")
    ap.add_argument("--batched-steps", type=int, default=500, help="0 skips the batched comparison")
    ap.add_argument("--adjoint-steps", type=int, default=200, help="0 skips the adjoint comparison")
    ap.add_argument("--pcisph-steps", type=int, default=500,
                    help="0 skips the PCISPH line (500 = the PCISPH configuration's stated length)")
    ap.add_argument("--wcsph65k-steps", type=int, default=1000,
                    help="0 skips the 65,536-particle dam-break line (1000 = its stated length)")
    ap.add_argument("--pcisph4m-steps", type=int, default=20, help="0 skips the PCISPH 4M line")
    ap.add_argument("--render-frames", type=int, default=20, help="0 skips the screen-space surface line")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("LOCAL_RANK", "0")), int(
        os.environ.get("WORLD_SIZE", "1"))


def load_workload(name, mode, seed=0):
    from fluids_gb300 import workloads
    if name == "wcsph4m":
        return workloads.double_dam_4m(mode=mode, seed=seed)
    if name == "wcsph1m":
        return workloads.double_dam_4m(mode=mode, seed=seed, n=80)
    if name == "wcsph65k":
        return workloads.dam_break_65k(mode=mode, seed=seed)
    if name == "pcisph4m":
        return workloads.pcisph_double_dam_4m(mode=mode, seed=seed)
    return workloads.pcisph_cube(mode=mode, seed=seed)


def workload_config(name, method, n, nb, dx, h, dt, container, lists):
    """The ``config`` of a bench line: what the workload is (both arms report the same one
    for the same scene); how an arm computes it goes in its top-level keys."""
    return {
        "workload": name,
        "method": method,
        "particles": n,
        "boundary_particles": nb,
        "dx_m": dx,
        "h_m": h,
        "dt_s": dt,
        "container_m": list(container),
        "neighbors": "list" if lists else "cell-scan",
        "l2": ("inputs larger than L2 every step (particle state %.0f MB > 129 MB)" if n * 200 > 129e6 else
               "particle state %.0f MB (fits the 129 MB L2)") % (n * 200 / 1e6),
    }


def describe_workload(w, n, nb, params):
    p = params
    return workload_config(w["name"], "PCISPH" if p.method == 1 else "WCSPH", n, nb, w["dx"], p.support_radius,
                           p.time_step, w["container"], p.neighbor_mode == 1 or p.method == 1)


def summary_of(line):
    """The headline numbers of a bench line in a few keys, printed last so that a truncated
    copy of the line still carries them."""
    g = lambda d, *ks: (None if d is None else (d.get(ks[0]) if len(ks) == 1 else g(d.get(ks[0]), *ks[1:])))  # noqa
    r = lambda x, k=4: None if x is None else float("%.*g" % (k, x))  # noqa
    return {"updates_per_s": r(line.get("value")), "e2e_updates_per_s": r(g(line, "e2e", "value")),
            "ms_per_step": r(line.get("ms_per_step")),
            "dominant_kernel": g(line, "roofline", "kernel"), "hbm_frac": r(g(line, "roofline", "frac"), 3),
            "issue_frac": r(g(line, "roofline", "issue", "frac"), 3),
            "batched_speedup": r(g(line, "batched", "speedup"), 3),
            "batched_mean_compression": r(g(line, "batched", "mean_density_error_batched"), 3),
            "pcisph_358k_updates_per_s": r(g(line, "pcisph", "updates_per_s")),
            "pcisph_4m_updates_per_s": r(g(line, "pcisph_4m", "updates_per_s")),
            "wcsph_65k_updates_per_s": r(g(line, "wcsph_65k", "updates_per_s")),
            "adjoint_over_plain_time": r(g(line, "adjoint", "adjoint_over_plain_time"), 3),
            "cpu_baseline_updates_per_s": r(g(line, "cpu_baseline", "value"))}


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, nm in enumerate(names):
                if r[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def measured_hbm_peak():
    try:
        d = json.load(open(PEAKS_FILE))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def measured_traffic(kernel, workload):
    """dram read+write bytes per launch of a kernel, from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "roofline_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        f = line.split()
        if len(f) >= 3 and f[0] == kernel and f[1] == workload:
            return float(f[2])
    return None


def measured_instructions(kernel):
    """(warp instructions per fluid particle, source workload) of a kernel from the committed
    ncu summary, or None."""
    path = os.path.join(ROOT, "profiles", "roofline_instructions.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        f = line.split()
        if len(f) >= 4 and f[0] == kernel:
            return float(f[2]) / float(f[3]), f[1]
    return None


def cpu_baseline(wl_name, mode, sample_steps, sample_desc_prefix, crop=None):
    """Times the oracle (the CPU port of the same step) on the host cores."""
    from oracle import Oracle, kwargs_from_params
    w = load_workload(wl_name, mode)
    fluid = w["fluid"]
    if crop is not None:
        fluid = fluid[crop]
    threads = os.cpu_count() or 1
    o = Oracle(threads=threads, **kwargs_from_params(w["params"], w["container"]))
    for pts, rot, mv, mass in w["bodies"]:
        o.add_boundary(pts, can_move=mv, rot3x4=rot, mass=mass)
    o.set_fluid(fluid)
    o.step(1)
    t0 = time.perf_counter()
    o.step(sample_steps)
    dt = time.perf_counter() - t0
    n = len(fluid)
    return {"value": n * sample_steps / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "%s: %d steps of %d fluid particles (+%d boundary), %.1f s" % (
                sample_desc_prefix, sample_steps, n, sum(len(b[0]) for b in w["bodies"]), dt)}


def bench_batched(steps, warmup, torch, nscenes=256, rank=0, world=1):
    """256 independent dam breaks (N log-uniform in [2048, 65536], containers a x 1 x 1 with
    a ~ U[1, 3], per-scene viscosity and c0): one batched context against looping the plain
    single-scene solver over the same scenes, both on one stream, same steps.  With several
    ranks the scenes are split by particle count (replicas.partition_scenes) and the
    throughputs are whole-job (sum of particles / slowest rank)."""
    from fluids_gb300 import autotune, capi, replicas, workloads
    scenes = workloads.batched_scenes(nscenes, seed=0)
    if world > 1:
        mine = replicas.partition_scenes([len(s["fluid"]) for s in scenes], world)[rank]
        scenes = [scenes[i] for i in mine]
    shared = workloads.batched_params()
    stream = torch.cuda.Stream()
    b = capi.BatchContext(shared, scenes)
    b.set_stream(stream.cuda_stream)
    n = b.particle_count()
    tuned_b = autotune.tune(b, shared.method, shared.mode, True)
    tile_shape = b.tile_shape()
    b.simulate(warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.simulate(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    tb = e0.elapsed_time(e1) / 1000.0
    sb = b.scene_stats()
    flags_b = b.device_flags()
    b.close()
    singles = []
    tuned_l = {}
    for s in scenes:
        c = workloads.build_scene_context(shared, s)
        c.set_stream(stream.cuda_stream)
        r = autotune.tune(c, shared.method, shared.mode, False)
        tuned_l[r["key"].split("|")[-1]] = r["block_size"]
        singles.append(c)
    for c in singles:
        c.simulate(warmup)
    torch.cuda.synchronize()
    e0.record(stream)
    for c in singles:
        c.simulate(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    tl = e0.elapsed_time(e1) / 1000.0
    sl = np.array([[c.stats()[k] for k in ("mean_compression", "mean_abs_density_error")] for c in singles])
    for c in singles:
        c.close()
    tb, units = replicas.aggregate(tb, n * steps, device="cuda")
    tl, _ = replicas.aggregate(tl, n * steps, device="cuda")
    n_all = int(round(units / steps))
    return {"scenes": nscenes, "particles": n_all, "ranks": world,
            "boundary_particles": int(sum(len(s["boundary"]) for s in scenes)),
            "steps": steps, "batched_updates_per_s": units / tb, "looped_updates_per_s": units / tl,
            "speedup": tl / tb, "batched_ms_per_step": 1000 * tb / steps, "looped_ms_per_step": 1000 * tl / steps,
            "mean_density_error_batched": float(sb[:, 0].mean()), "mean_density_error_looped": float(sl[:, 0].mean()),
            "mean_abs_density_error_batched": float(sb[:, 1].mean()),
            "mean_abs_density_error_looped": float(sl[:, 1].mean()),
            "density_error_definitions": "mean_density_error_*: mean over particles of max(rho / rho0 - 1, 0), the "
                                         "compression the <= 1 % criterion reads; mean_abs_density_error_*: mean "
                                         "of |rho - rho0| / rho0 (free-surface particles count at their full "
                                         "deficit)", "device_flags": flags_b,
            "block_size_batched": tuned_b["block_size"],
            "tile_shape_batched": dict(tile_shape, tuned_from=tuned_b.get("source"),
                                       seconds_per_step_by_shape=tuned_b.get("seconds_per_step")),
            "block_size_looped_by_size": tuned_l}


def bench_adjoint(torch, steps=200, every=20):
    """Differentiable WCSPH, 32^3 particles (Fourier initial velocity, 200 steps, checkpoint
    every 20): adjoint forward + backward against the plain solver's forward on the same
    scene and GPU, plus central differences of the GPU forward (FP32) for the gradients."""
    from fluids_gb300 import capi, workloads
    w = workloads.adjoint_block(32, steps=steps, checkpoint_every=every)
    stream = torch.cuda.Stream()
    ctx = workloads.build_context(w)
    ctx.set_stream(stream.cuda_stream)
    n = ctx.particle_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        torch.cuda.synchronize()
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1000.0

    ctx.simulate(3)
    t_plain = timed(lambda: ctx.simulate(steps))
    adj = capi.Adjoint(ctx, steps, every)
    dev = torch.device("cuda")
    x0 = torch.tensor(w["fluid"], device=dev)
    v0 = torch.tensor(w["velocities"], device=dev)
    y = torch.tensor(w["target"], device=dev)
    xT, vT, gx = torch.empty_like(x0), torch.empty_like(x0), torch.zeros_like(x0)
    gx0, gv0 = torch.empty_like(x0), torch.empty_like(x0)
    mu, k = w["mu"], w["kgas"]

    def fwd(v=v0, m=mu, kk=k):
        adj.forward(x0.data_ptr(), v.data_ptr(), m, kk, out_x=xT.data_ptr(), out_v=vT.data_ptr())

    res = {}

    def bwd():
        res.update(adj.backward(gx.data_ptr(), None, out_gx0=gx0.data_ptr(), out_gv0=gv0.data_ptr()))

    fwd()
    gx[:, :3] = 2.0 * (xT[:, :3] - y[:, :3]) / n
    bwd()
    t_fwd = min(timed(fwd) for _ in range(3))
    t_bwd = min(timed(bwd) for _ in range(3))

    def loss(**kw):
        fwd(**kw)
        torch.cuda.synchronize()
        return float(((xT[:, :3].double() - y[:, :3].double()) ** 2).sum(dim=1).mean())

    fd = {}
    e = 0.1 * mu
    fd["mu"] = dict(eps_rel=0.1, fd=(loss(m=mu + e) - loss(m=mu - e)) / (2 * e), adjoint=res["g_mu"])
    c0, e = w["c0"], 0.01 * w["c0"]
    fd["c0"] = dict(eps_rel=0.01, fd=(loss(kk=workloads.tait_stiffness(c0 + e)) -
                                      loss(kk=workloads.tait_stiffness(c0 - e))) / (2 * e), adjoint=res["g_c0"])
    dd = torch.tensor(workloads.fourier_velocity(w["fluid"], 8, 1.0, seed=99), device=dev)
    e = 1e-2
    fd["v0_smooth_direction"] = dict(eps=e, fd=(loss(v=v0 + e * dd) - loss(v=v0 - e * dd)) / (2 * e),
                                     adjoint=float((gv0[:, :3].double() * dd[:, :3].double()).sum()))
    for d in fd.values():
        d["rel_err"] = abs(d["adjoint"] - d["fd"]) / abs(d["fd"])
    out = {"particles": n, "steps": steps, "checkpoint_every": every,
           "plain_updates_per_s": n * steps / t_plain, "plain_ms": 1000 * t_plain,
           "adjoint_forward_ms": 1000 * t_fwd, "adjoint_backward_ms": 1000 * t_bwd,
           "adjoint_updates_per_s": n * steps / (t_fwd + t_bwd),
           "adjoint_over_plain_time": (t_fwd + t_bwd) / t_plain,
           "gradients": {"d_mu": res["g_mu"], "d_c0": res["g_c0"], "d_k": res["g_k"]},
           "fd_check_fp32": fd,
           "fd_check_fp32_note": "informational: central differences of the FP32 GPU forward (FP32 rounding "
                                 "dominates the differences in mu); the 1e-3 criterion is checked against FP64 "
                                 "central differences and the FP64 adjoint on the 4,096-particle copy "
                                 "(tests/test_gpu_adjoint.py)",
           "flags": adj.flags(), "tape_bytes": adj.tape_bytes()}
    adj.close()
    ctx.close()
    return out


def bench_pcisph(torch, steps, warmup, large=False):
    """PCISPH double block + rotated cube (358,400 fluid particles), or with `large` the
    4,194,304-particle double dam break, PHYSICS mode: device time of `steps` graph-replayed
    steps, each between its own CUDA events so that its predict-correct iteration count (the
    loop is one persistent kernel) can be read after it; the kernel split comes from one
    profiled step, whose iteration count is given beside it."""
    from fluids_gb300 import capi, workloads
    w = (workloads.pcisph_double_dam_4m if large else workloads.pcisph_cube)(capi.SPH_MODE_PHYSICS)
    stream = torch.cuda.Stream()
    ctx = workloads.build_context(w)
    ctx.set_stream(stream.cuda_stream)
    n, nb = ctx.particle_count(), ctx.boundary_particle_count()
    ctx.simulate(warmup)
    # each timed step between its own pair of events on the context stream, its iteration
    # count read after it (outside the events)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    iters = []
    torch.cuda.synchronize()
    for a, b in ev:
        a.record(stream)
        ctx.simulate(1)
        b.record(stream)
        iters.append(int(ctx.get("PCI_ITERS")[0]))
    torch.cuda.synchronize()
    t = sum(a.elapsed_time(b) for a, b in ev) / 1000.0
    flags = ctx.device_flags()
    prof = ctx.profile_step(1)
    prof_iters = int(ctx.get("PCI_ITERS")[0])
    hist = {str(k): int(v) for k, v in zip(*np.unique(iters, return_counts=True))}
    out = {"workload": w["name"], "particles": n, "boundary_particles": nb, "steps": steps,
           "updates_per_s": n * steps / t, "ms_per_step": 1000 * t / steps,
           "pci_iterations_mean": float(np.mean(iters)), "pci_iterations_histogram": hist, "device_flags": flags,
           "kernel_ms_per_step": prof, "kernel_ms_iterations": prof_iters}
    ctx.close()
    return out


def bench_wcsph65k(torch, steps, warmup):
    """The plain WCSPH dam break (65,536 particles on a 32 x 64 x 32 lattice at dx = 0.015 m,
    FishTank walls, dt = 2e-4 s), PHYSICS mode, for its stated 1000 steps: device time of the
    graph-replayed steps on the context stream."""
    from fluids_gb300 import autotune, capi, workloads
    w = workloads.dam_break_65k(capi.SPH_MODE_PHYSICS)
    stream = torch.cuda.Stream()
    ctx = workloads.build_context(w)
    ctx.set_stream(stream.cuda_stream)
    tuned = autotune.tune(ctx, w["params"].method, w["params"].mode, False)
    n, nb = ctx.particle_count(), ctx.boundary_particle_count()
    ctx.simulate(warmup)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    ctx.simulate(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1000.0
    st = ctx.stats()
    out = {"workload": w["name"], "particles": n, "boundary_particles": nb, "steps": steps,
           "updates_per_s": n * steps / t, "ms_per_step": 1000 * t / steps, "block_size": tuned["block_size"],
           "device_flags": ctx.device_flags(), "kernel_ms_per_step": ctx.profile_step(1),
           "final_mean_compression": st["mean_compression"], "final_kinetic_energy_j": st["kinetic"]}
    ctx.close()
    return out


def bench_render(torch, ctx, stream, frames, width=1920, height=1080):
    """Screen-space surface of the context's particles (depth sprites, two blur iterations,
    normals, final shading over a background gradient with a random 256^2 cube map) at
    width x height with the reference's default camera (view and projection) and sprite
    radius; device time per
    stage from CUDA events on the context stream, averaged over `frames` frames."""
    from fluids_gb300 import capi, render
    cam = render.Camera(width, height)
    mv = cam.transformation()   # the reference's default view of the container
    r = render.SSpaceFluidRenderer(width, height)
    s = stream.cuda_stream
    for _ in range(3):
        r.render(ctx, cam, mv, s)
    pr = cam.projection()
    ipr = np.linalg.inv(pr.astype(np.float64)).astype(np.float32)
    view = capi.make_view(mv, pr, r.point_radius, cam.point_scale(), width, height)
    # a background gradient and a 256^2 cube map stand in for the scene behind and the skybox
    dev = r.depth.device
    yy, xx = torch.meshgrid(torch.linspace(0, 1, height, device=dev), torch.linspace(0, 1, width, device=dev),
                            indexing="ij")
    bkg = torch.stack([xx, yy, 0.5 * torch.ones_like(xx), torch.ones_like(xx)], -1).contiguous()
    cube = torch.rand((6, 256, 256, 4), generator=torch.Generator(device=dev).manual_seed(0), device=dev)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
    tot = np.zeros(4)
    torch.cuda.synchronize()
    for _ in range(frames):
        ev[0].record(stream)
        ctx.render_depth(view, r.depth.data_ptr())
        ev[1].record(stream)
        capi.render_smooth(r.depth.data_ptr(), r.blurred.data_ptr(), width, height, r.filter_iterations, s)
        ev[2].record(stream)
        capi.render_normals(r.depth.data_ptr(), r.normals.data_ptr(), width, height, ipr, s)
        ev[3].record(stream)
        capi.render_shade(r.depth.data_ptr(), r.normals.data_ptr(), bkg.data_ptr(), cube.data_ptr(), 256, width,
                          height, mv, ipr, r.color.data_ptr(), s)
        ev[4].record(stream)
        torch.cuda.synchronize()
        tot += [ev[k].elapsed_time(ev[k + 1]) for k in range(4)]
    ms = tot / frames
    return {"image": [width, height], "particles": ctx.particle_count(), "point_radius": r.point_radius,
            "filter_iterations": r.filter_iterations, "frames": frames, "ms_per_frame": float(ms.sum()),
            "ms_depth": float(ms[0]), "ms_blur": float(ms[1]), "ms_normals": float(ms[2]),
            "ms_shade": float(ms[3]), "coverage": float((r.depth != 0).float().mean().item()),
            "kernels_per_frame": 7 + 2 * r.filter_iterations + 2}


def bench_voxelize(reps=5):
    """GPU voxel sampler (sph_scene_voxelize, Model::surface_sampling): a level-4 icosphere
    of radius 0.25 m (5,120 triangles) at particle spacing 0.005 m; host wall time per call
    (it is synchronous: upload, count, emit, bucket sort, duplicate test, corners, download)."""
    from fluids_gb300 import scenes
    v, ix = scenes.icosphere(0.25, 4)
    out = scenes.voxelize(v, ix, 0.005)
    t0 = time.perf_counter()
    for _ in range(reps):
        out = scenes.voxelize(v, ix, 0.005)
    ms = 1000.0 * (time.perf_counter() - t0) / reps
    return {"mesh": "icosphere level 4, r = 0.25 m", "triangles": len(ix) // 3, "spacing_m": 0.005,
            "particles": len(out), "ms_per_call": ms, "calls": reps}


def run_reference(args):
    """The reference arm: the reference's own WCSPH kernels (kernels/*.cl through the CPU
    runtime of oracle/ref_shim, work-groups on every host core) stepping the benchmark's
    whole scene, launch for launch as WCSPHSimulation::simulate.  For the default workload
    the scene comes from oracle.refscene (its walls from the reference's own
    FishTank::surface_sampling), so this process loads none of the product's libraries.
    Where the reference kernels are not built, or for the PCISPH workloads, the oracle's
    COMPAT restatement of them runs instead on all cores."""
    rank, _, world = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    stepper = None
    if args.workload == "wcsph4m":
        try:
            from oracle import refkernels, refscene
            if refkernels.build() is not None:
                from oracle.refstep import RefWCSPH
                r = refscene.double_dam_4m()
                fluid, walls, pr = r["fluid"], r["walls"], r["params"]
                t0 = time.perf_counter()
                stepper = RefWCSPH(fluid, walls, r["container"], pr["time_step"], pr["max_vel"], pr["k_viscosity"],
                                   pr["surface_tension"], pr["gas_stiffness"], pr["rest_density"], pr["gravity"],
                                   pr["particle_radius"], pr["support_radius"])
                setup_s = time.perf_counter() - t0
                f32 = lambda x: float(np.float32(x))  # noqa: E731 -- the solver's FP32 parameter values
                cfg = workload_config(r["name"], "WCSPH", len(fluid), len(walls), r["dx"], f32(pr["support_radius"]),
                                      f32(pr["time_step"]), r["container"], True)
        except Exception as e:  # noqa: BLE001 -- fall back to the restatement, say why
            print("reference kernels unavailable (%s); timing the oracle's restatement" % e, file=sys.stderr)
            stepper = None
    if stepper is not None:
        kind = "reference"
        what = ("the reference's own kernels (kernels/grid.cl, wcsph.cl, normals.cl) on a CPU OpenCL-C runtime "
                "(oracle/ref_shim, %d threads; key sort = the stable sort clogs performs), its 5 m grid with the "
                "1 GB cell table cleared every step; the whole %d-particle scene (set-up %.1f s untimed)"
                % (threads, len(fluid), setup_s))
        n, nb = len(fluid), len(walls)

        def run(k):
            for _ in range(k):
                stepper.step()
    else:
        from fluids_gb300 import capi
        from oracle import Oracle, kwargs_from_params
        w = load_workload(args.workload, capi.SPH_MODE_COMPAT)
        p = w["params"]
        o = Oracle(threads=threads, **kwargs_from_params(p, w["container"]))
        for pts, rot, mv, mass in w["bodies"]:
            o.add_boundary(pts, can_move=mv, rot3x4=rot, mass=mass)
        o.set_fluid(w["fluid"])
        n, nb = len(w["fluid"]), sum(len(b[0]) for b in w["bodies"])
        cfg = describe_workload(w, n, nb, p)
        kind = "port"
        what = "reference kernels' CPU port (oracle, COMPAT mode: 5 m grid, 50-entry neighbour lists), whole scene"

        def run(k):
            o.step(k)
    run(max(args.warmup, 0))
    t0 = time.perf_counter()
    run(args.steps)
    dt = time.perf_counter() - t0
    v = n * args.steps / dt
    sample = "%s; %d fluid + %d boundary particles, %d steps in %.1f s" % (what, n, nb, args.steps, dt)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000 * dt / max(args.steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded lattice + jitter)",
            "config": cfg,
            "mode": ("compat: the reference's kernel text, defects included (its density passes r, not r^2, "
                     "to poly6, so densities are negative and compute_acceleration skips the fluid pressure, "
                     "viscosity and surface-tension pairs behind its density > 0 guard, wcsph.cl:61-62,152)"),
            "parallelism": "%d host threads" % threads,
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": kind, "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    rank, local_rank, world = dist_env()
    import torch
    import torch.distributed as dist
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
    torch.cuda.set_device(local_rank)
    import fluids_gb300
    from fluids_gb300 import capi, replicas, workloads
    fluids_gb300.build()
    w = load_workload(args.workload, capi.SPH_MODE_PHYSICS, seed=rank)
    params = w["params"]
    params.neighbor_mode = args.neighbor_mode
    stream = torch.cuda.Stream()
    ctx = capi.Context(params)
    capi.check(capi.lib().sph_set_stream(ctx.h, capi.C.c_void_p(stream.cuda_stream)), ctx.h)
    ctx.set_rect_limits(*w["container"])
    for pts, rot, mv, mass in w["bodies"]:
        ctx.add_boundary(pts, can_move=mv, rot3x4=rot, mass=mass)
    ctx.add_volume(w["fluid"], w.get("velocities"))
    n, nb = ctx.particle_count(), ctx.boundary_particle_count()
    d = capi.describe(params, w["container"])
    from fluids_gb300 import autotune
    tuned = autotune.tune(ctx, params.method, params.mode, False)

    ctx.simulate(max(args.warmup, 3))
    ctx.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler() if rank == 0 else None
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    if clocks:
        clocks.start()
    e0.record(stream)
    ctx.simulate(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = clocks.stop() if clocks else None
    t = e0.elapsed_time(e1) / 1000.0
    t, units = replicas.aggregate(t, n * args.steps, device="cuda")   # max time, sum over ranks
    flags = ctx.device_flags()
    value = units / t

    # per-kernel device time of the same step (events between the kernels, no graph)
    kern = ctx.profile_step(min(args.steps, 20))
    top = max(kern, key=kern.get)
    peak, peak_kind = measured_hbm_peak()
    alg = ALG_BYTES.get(top)
    roof = None
    mean_len = (float(ctx.get("NEIGH_LEN").mean()), float(ctx.get("SB_NEIGH_LEN").mean()) if nb > 0 else 0.0)
    if alg is not None:
        bnd_extra = 20.0 * nb if top in ("k_wc_density", "k_wc_forces") else 0.0
        lb = LIST_BYTES.get(top)
        if lb is not None and params.neighbor_mode == 1:
            alg = alg + lb[0] * mean_len[0] + lb[1] * mean_len[1] + lb[2]
        bytes_launch = alg * n + bnd_extra
        achieved = bytes_launch / (kern[top] / 1000.0) / 1e9
        tr = measured_traffic(top, w["name"])
        roof = {"bound": "hbm", "kernel": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "algorithmic_bytes": bytes_launch,
                "mean_list_lengths": {"fluid": mean_len[0], "boundary": mean_len[1]},
                "traffic": tr,
                "traffic_from": ("profiles/roofline_traffic.txt: dram__bytes_read.sum + dram__bytes_write.sum of "
                                 "one ncu capture of this kernel on this workload, stored with the code (not "
                                 "measured in this run)") if tr is not None else None,
                "ms_per_launch": kern[top]}
    # the pair loops are bound by FP32 issue, not DRAM: the same kernel against the SM issue rate
    ins = measured_instructions(top)
    if roof is not None and ins is not None:
        sms = torch.cuda.get_device_properties(local_rank).multi_processor_count
        mhz, mhz_from = (clk or {}).get("sm_mhz"), "SM clock sampled in the timed region"
        if not mhz:
            mhz, mhz_from = 2070.0, "maximum SM clock"
        peak_ips = sms * 4 * mhz * 1e6
        ach = ins[0] * n / (kern[top] / 1000.0)
        roof["issue"] = {"bound": "fp32-issue", "achieved": ach, "peak": peak_ips, "unit": "warp-instructions/s",
                         "frac": ach / peak_ips, "warp_instructions_per_particle": ins[0],
                         "instructions_from": ("profiles/roofline_instructions.txt: ncu smsp__inst_executed.sum "
                                               "of one capture on " + ins[1] + ", stored with the code (not "
                                               "measured in this run)"),
                         "peak_from": "%d SMs x 4 schedulers x %.0f MHz (%s)" % (sms, mhz, mhz_from)}
    # kernel nodes of the step's CUDA graph (the timed region replays it)
    launches_per_step = ctx.step_kernel_launches()
    # e2e through the C ABI with pinned host buffers: state in, result out, every step
    e2e = None
    if not args.no_e2e:
        hp = torch.empty((n, 4), dtype=torch.float32, pin_memory=True).numpy()
        hv = torch.empty((n, 4), dtype=torch.float32, pin_memory=True).numpy()
        hh = torch.empty((n, 4), dtype=torch.float32, pin_memory=True).numpy()
        L = capi.lib()
        for f, a in (("POS", hp), ("VEL", hv), ("VEL_HALF", hh)):
            capi.check(L.sph_get_field(ctx.h, capi.FIELDS[f], a.ctypes.data, a.nbytes), ctx.h)
        # one untimed host step builds the host step's graph for these buffers
        capi.check(L.sph_simulate_host(ctx.h, hp.ctypes.data, hv.ctypes.data, hh.ctypes.data, 1), ctx.h)
        capi.check(L.sph_synchronize(ctx.h), ctx.h)
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()
        k_e2e = args.steps
        t0 = time.perf_counter()
        # every step: the whole particle state (pos, vel, vel_half) in from pinned host memory,
        # one step, the whole state back out, and a host wait for it
        state = (("POS", hp), ("VEL", hv), ("VEL_HALF", hh))
        for _ in range(k_e2e):
            capi.check(L.sph_simulate_host(ctx.h, hp.ctypes.data, hv.ctypes.data, hh.ctypes.data, 1), ctx.h)
            capi.check(L.sph_synchronize(ctx.h), ctx.h)
        te = time.perf_counter() - t0
        # the same copies without the step: the host link's share of the e2e time
        t1 = time.perf_counter()
        for _ in range(k_e2e):
            for f, a in state:
                capi.check(L.sph_set_field_async(ctx.h, capi.FIELDS[f], a.ctypes.data, a.nbytes), ctx.h)
            capi.check(L.sph_synchronize(ctx.h), ctx.h)
        th = (time.perf_counter() - t1) / k_e2e
        t1 = time.perf_counter()
        for _ in range(k_e2e):
            for f, a in state:
                capi.check(L.sph_get_field_async(ctx.h, capi.FIELDS[f], a.ctypes.data, a.nbytes), ctx.h)
            capi.check(L.sph_synchronize(ctx.h), ctx.h)
        td = (time.perf_counter() - t1) / k_e2e
        ms_e2e = te * 1e3 / k_e2e
        te, units_e = replicas.aggregate(te, n * k_e2e, device="cuda")
        e2e = {"value": units_e / te, "unit": UNIT, "h2d_bytes_per_step": 48 * n,
               "d2h_bytes_per_step": 48 * n, "steps": k_e2e, "host_buffers": "pinned",
               "copies": ("pos, vel, vel_half in and out every step through sph_simulate_host (the velocity "
                          "uploads beside the step's binning, sort and list pass); one host wait per step"),
               "ms_per_step": ms_e2e, "copy_ms_per_step": (th + td) * 1e3,
               "h2d_gbs": 48 * n / th / 1e9, "d2h_gbs": 48 * n / td / 1e9}
    rend = vox = None
    if args.render_frames > 0:
        rend = bench_render(torch, ctx, stream, args.render_frames)
        vox = bench_voxelize()
    ctx.close()
    batched = None
    if args.batched_steps > 0 and args.workload == "wcsph4m":
        batched = bench_batched(args.batched_steps, max(args.warmup, 3), torch, rank=rank, world=world)
    adjoint = pcisph = pcisph4m = None
    if args.adjoint_steps > 0 and args.workload == "wcsph4m":
        adjoint = bench_adjoint(torch, args.adjoint_steps)
    if args.pcisph_steps > 0 and args.workload == "wcsph4m":
        pcisph = bench_pcisph(torch, args.pcisph_steps, max(args.warmup, 3))
    if args.pcisph4m_steps > 0 and args.workload == "wcsph4m":
        pcisph4m = bench_pcisph(torch, args.pcisph4m_steps, 3, large=True)
    wcsph65k = None
    if args.wcsph65k_steps > 0 and args.workload == "wcsph4m":
        wcsph65k = bench_wcsph65k(torch, args.wcsph65k_steps, max(args.warmup, 3))
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        z = w["fluid"][:, 2]
        crop = np.nonzero(z < np.quantile(z, 1.0 / 16))[0] if args.workload == "wcsph4m" else None
        cpu = cpu_baseline(args.workload, capi.SPH_MODE_PHYSICS, 10 if crop is not None else 3,
                           "oracle PHYSICS FP32 (same step as the GPU path), z-slab of the workload", crop)
    if rank == 0:
        cfg = describe_workload(w, n, nb, params)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1000.0 * t / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded lattice + jitter)",
                "config": cfg, "mode": "physics" if params.mode == 1 else "compat",
                "grid_cells": d["grid_dims"], "parallelism": "replicas" if world > 1 else "single GPU",
                "block_size": tuned["block_size"], "roofline": roof, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": launches_per_step * args.steps, "clocks": clk,
                "kernel_ms_per_step": kern, "device_flags": flags, "batched": batched, "adjoint": adjoint,
                "pcisph": pcisph, "pcisph_4m": pcisph4m, "wcsph_65k": wcsph65k, "render": rend, "voxelize": vox}
        line["summary"] = summary_of(line)
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
