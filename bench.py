#!/usr/bin/env python3
"""Benchmark: forward+adjoint optimisation iterations per second.

Workload (default): the icosphere configuration -- 2,562 vertices / 5,120
triangles, point light (3,3,3) intensity 10 with per-vertex albedo, 8 ring
cameras at distance 3, 512x512, 16 spp, W*H edge samples per view, FP32.
One step = one optimiser iteration over all 8 views: forward render, MSE
loss + adjoint, interior adjoint, edge sampling, the reference's "Adam"
update and the LBVH refit (d_render_and_compare + OptStep + OptUpdateScene
of src/optimizer_simple.cpp).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl drgb|reference]
                    [--workload icosphere|cube]

value: iterations/s with everything resident on the GPU (optimiser graph
replays timed with CUDA events on the renderer stream; L2 flushed before
every step).  e2e: the same metric through the public C-ABI call
drgb_d_render_and_compare with host buffers (targets H2D, gradient + loss
D2H inside the timed region).  The reference arm times the reference's own
CPU implementation (its d_render_and_compare with the brute-force caster and
OpenMP, rebuilt from the reference sources by oracle/ref/build_ref.py; the
oracle port where they are absent) on a bounded sample and extrapolates
linearly in pixels x views.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

WORKLOADS = {
    "icosphere": dict(name="icosphere5120_pointlight_8views_512x512_16spp", sub=4, mode=16, spp=16, res=512,
                      views=8, sample_res=64, sample_views=1),
    "cube": dict(name="cube12_vertexcolor_1view_256x256_16spp", sub=None, mode=2, spp=16, res=256, views=1,
                 sample_res=256, sample_views=1),
    # small case of the icosphere kernels for ncu section captures
    "icosphere_small": dict(name="icosphere5120_pointlight_2views_256x256_16spp", sub=4, mode=16, spp=16, res=256,
                            views=2, sample_res=32, sample_views=1),
}


def make_problem(w):
    import diffrender_tutorials_gb300 as D
    if w["sub"] is None:
        true = D.make_cube(seed=1)
        init = D.perturb_vertices(true, 0.1, seed=2)
        init.colors = np.clip(true.colors + np.random.default_rng(3).normal(0, 0.1, (8, 3)), 0, 1).astype(np.float32)
        cams = [D.CamInfo(origin=(0, 0, 3), width=w["res"], height=w["res"])]
    else:
        true = D.make_icosphere(w["sub"], seed=1)
        init = D.perturb_vertices(true, 0.02, seed=2, radial=True)
        cams = D.ring_cameras(w["views"], 3.0, w["res"], w["res"])
    ts, isc = D.Scene(), D.Scene()
    ts.add_mesh(true)
    isc.add_mesh(init)
    return ts, isc, cams


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in self.rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        pg = dist
    return ws, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([float(x)])
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def cpu_sample(w, reps=1):
    """The reference's own CPU path on a bounded sample of the workload:
    returns (seconds per full-workload iteration, factor, threads, kind,
    description).  The reference driver (oracle/ref/build_ref.py: brute-force
    caster + OpenMP, with the point-light model of oracle/ref/ref_pointlight.h)
    is built from the reference sources where they are available; otherwise
    the oracle port of the same algorithm is timed."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "oracle", "ref"))
    import pyoracle as O
    import diffrender_tutorials_gb300 as D
    ts, isc, cams = make_problem(w)
    sres, sv = w["sample_res"], w["sample_views"]
    scams = [D.CamInfo(origin=c.origin, target=c.target, up=c.up, width=sres, height=sres) for c in cams[:sv]]
    cores = os.cpu_count() or 1
    factor = (w["res"] * w["res"] * w["views"]) / (sres * sres * sv)
    what = (f"{sv} view(s) at {sres}x{sres} of the same scene, extrapolated x{factor:g}" if factor != 1 else
            f"the full workload ({sv} view(s) at {sres}x{sres}), not extrapolated")
    O.set_threads(cores)
    tgt = O.render(ts, scams, w["mode"], w["spp"])
    exe = None
    try:
        import build_ref
        exe = build_ref.build()
    except Exception:  # noqa: BLE001 - no compiler or sources: time the port
        exe = None
    if exe:
        import refrun
        items = {"task": np.array([4], np.int32), "mode": np.array([w["mode"]], np.int32),
                 "spp": np.array([w["spp"]], np.int32), **refrun.cam_items(scams), **refrun.scene_items(isc),
                 "targets": tgt, "dmesh_ids": np.array([0], np.int32),
                 "edge_samples": np.array([sres * sres], np.int32)}
        dt = 0.0
        for _ in range(reps):
            dt += float(refrun.run(exe, items)["seconds"][0])
        dt /= reps
        # the reference runs its loops on 14 OpenMP threads (MAXTHREADS, src/drender.h:12) whatever the
        # host has: more threads than cores when the host has fewer than 14
        return dt * factor, factor, 14, "reference", what + f" (reference d_render_and_compare, " \
            f"brute-force caster, OpenMP: 14 threads on {cores} host cores)"
    t0 = time.perf_counter()
    for _ in range(reps):
        O.d_render_and_compare(isc, scams, w["mode"], w["spp"], tgt, sres * sres)
    dt = (time.perf_counter() - t0) / reps
    return dt * factor, factor, cores, "port", what + " (oracle: CPU port of the reference path)"


def reference_arm(args, w, ws, rank, pg):
    if rank != 0:
        return
    # warm-up then timed samples; each step is one bounded sample
    for _ in range(args.warmup):
        cpu_sample(w)
    times = []
    for _ in range(args.steps):
        t, factor, cores, kind, desc = cpu_sample(w)
        times.append(t)
    mean = sum(times) / len(times)
    val = 1.0 / mean
    # the small workload (cube, 256x256, one view) timed at its full size, not extrapolated
    cube = WORKLOADS["cube"]
    cube_t = [cpu_sample(cube)[0] for _ in range(max(3, min(args.steps, 10)))]
    line = {"impl": "reference", "metric": "fwd+adjoint iters/s", "value": val, "unit": "iters/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": w["name"], "parallelism": "replicas"},
            "cpu_baseline": {"value": val, "unit": "iters/s", "cores": cores, "kind": kind, "sample": desc,
                             "host_cores": os.cpu_count() or 1},
            "extrapolation": {"factor": factor, "sample_ms_per_step": mean * 1e3 / factor,
                              "note": "each step times one bounded sample of the workload (one reduced view) and "
                                      "scales it by pixels x views; ms_per_step is the scaled figure"},
            "cube_full_size": {"workload": cube["name"], "value": 1.0 / (sum(cube_t) / len(cube_t)),
                               "unit": "iters/s", "ms_per_step": 1e3 * sum(cube_t) / len(cube_t),
                               "steps": len(cube_t), "extrapolated": False},
            "e2e": {"value": val, "unit": "iters/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def read_traffic():
    """Per-launch DRAM bytes of the pixel kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "k_pixels_icosphere_traffic.md")
    try:
        for line in open(p):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


BVH_BUILDERS = {"lbvh": 0, "sah": 1, "two_level": 2, "flat_sah": 3}
# camera and point-light shadow rays: hierarchy, tiles and cells where they pay (autotuned), always tiles and cells
RASTER = {"off": 0, "auto": 1, "always": 2}


def drgb_arm(args, w, ws, rank, local, pg):
    import torch
    import diffrender_tutorials_gb300 as D
    from diffrender_tutorials_gb300 import build as B
    from diffrender_tutorials_gb300 import native as N
    B.build()
    torch.cuda.set_device(local)
    ts, isc, cams = make_problem(w)
    S = D.SHADING_MODEL(w["mode"])
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(S, w["spp"]), device=local)
    r.set_option(N.OPT_BVH_BUILDER, BVH_BUILDERS[args.bvh])
    r.set_option(N.OPT_PRIMARY_RASTER, RASTER[args.raster])
    r.commit(ts)
    targets = r.render(ts, cams)
    p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.01)
    p.base_lr = 0.01
    p.flags = D.OptimizerParameters._OPT_POS | D.OptimizerParameters._OPT_COL
    opt = D.CreateSimpleOptimizer()
    opt.Init(isc, r, cams, targets, p)
    tuned = opt.autotune(3)
    stream = torch.cuda.ExternalStream(r.stream(), device=local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    for _ in range(args.warmup):
        opt.run_async(1)
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    barrier(pg)
    torch.cuda.synchronize()
    k0 = D.kernel_launches()
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            for i in range(args.steps):
                flush.zero_()  # L2 flush (256 MiB write) outside the timed events
                starts[i].record(stream)
                opt.run_async(1)
                ends[i].record(stream)
        torch.cuda.synchronize()
    launches = D.kernel_launches() - k0 - 0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    total_ms = allmax(pg, sum(step_ms))
    barrier(pg)
    value = ws * args.steps / (total_ms / 1e3)
    losses = opt.losses

    # e2e: the reference's call sequence through the public C ABI with host
    # buffers, one iteration per step: drgb_commit of the scene (the
    # reference's d_render_and_compare commits the scene it is given on every
    # call, src/drender.h:176; here a commit of the same triangles uploads the
    # mesh, flattens it and refits the hierarchy), then
    # drgb_d_render_and_compare (targets in from pinned memory, gradient and
    # loss out)
    r2 = D.MakeDifferentialRenderer(D.DiffRenderSettings(S, w["spp"]), device=local)
    r2.set_option(N.OPT_BVH_BUILDER, BVH_BUILDERS[args.bvh])
    r2.set_option(N.OPT_PRIMARY_RASTER, RASTER[args.raster])
    r2.commit(isc)
    tg_pinned = torch.empty(targets.size, dtype=torch.float32, pin_memory=True).numpy()
    tg_pinned[:] = targets.reshape(-1)
    ds = D.DScene(r2, [0])
    ds.data = torch.zeros(ds.data.size, dtype=torch.float32, pin_memory=True).numpy()
    edge_samples = w["res"] * w["res"]
    for _ in range(max(1, args.warmup)):
        r2.commit(isc)
        r2.d_render_and_compare(isc, cams, tg_pinned, edge_samples, ds)
    e2e_ms = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        r2.commit(isc)
        r2.d_render_and_compare(isc, cams, tg_pinned, edge_samples, ds)
        e2e_ms.append((time.perf_counter() - t0) * 1e3)
    e2e_total = allmax(pg, sum(e2e_ms))
    e2e_value = ws * args.steps / (e2e_total / 1e3)
    scene_bytes = sum(a.nbytes for m in isc.meshes for a in (m.vertices, m.indices, m.colors, m.normals, m.tc)
                      if a is not None) + sum(64 * len(t) for t in isc.transforms)
    h2d = scene_bytes + tg_pinned.nbytes + 168 * len(cams)
    d2h = ds.data.nbytes + 4

    # the same iteration with the deterministic gradient reduction
    from diffrender_tutorials_gb300 import native as N
    r.set_option(N.OPT_DETERMINISTIC, 1)
    for _ in range(args.warmup):
        opt.run_async(1)
    torch.cuda.synchronize()
    det_ms = []
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            opt.run_async(1)
            ends[i].record(stream)
    torch.cuda.synchronize()
    det_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    det_prof = opt.profile(2)
    r.set_option(N.OPT_DETERMINISTIC, 0)
    deterministic = {"value": args.steps / (sum(det_ms) / 1e3), "unit": "iters/s",
                     "ms_per_step": sum(det_ms) / args.steps, "phases_ms": det_prof,
                     "how": "DRGB_OPT_DETERMINISTIC: gradient records sorted by index, fixed-order sums "
                            "(tiles and cells by the size rule, as in the batched engine)"}

    # the same iteration sampling silhouette edges only (DRGB_OPT_EDGE_SET = 1)
    r.set_option(N.OPT_EDGE_SET, 1)
    for _ in range(args.warmup):
        opt.run_async(1)
    torch.cuda.synchronize()
    with torch.cuda.stream(stream):
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            opt.run_async(1)
            ends[i].record(stream)
    torch.cuda.synchronize()
    sil_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    silhouette = {"value": args.steps / (sum(sil_ms) / 1e3), "unit": "iters/s",
                  "ms_per_step": sum(sil_ms) / args.steps, "phases_ms": opt.profile(2),
                  "how": "DRGB_OPT_EDGE_SET = 1: edge samples on silhouette and boundary edges only"}
    r.set_option(N.OPT_EDGE_SET, 0)

    # roofline of the dominant kernel (fused forward/adjoint pixel kernel)
    prof = opt.profile(3)
    work = opt.count_work()
    clocks = clk.summary()
    import json as _j
    peaks = {}
    try:
        peaks = _j.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    npix = w["res"] * w["res"] * w["views"]
    # algorithmic bytes of one pixel-kernel launch: targets read (12 B/px),
    # adjoint written (16 B/px), the raster pass's record of every forward
    # and adjoint camera sample read (16 B; 24 B for the point-light model,
    # whose record adds u, v to the shading point), scene data read once
    # (pos/col/nrm/tc 56 B/vertex, triangles+indices 64 B/triangle, nodes
    # 64 B/node), gradients written
    n_tri = sum(m.face_count for m in isc.meshes)
    n_v = sum(m.vertex_count for m in isc.meshes)
    S_eff = int(math.isqrt(w["spp"])) ** 2
    rec_bytes = 24 if w["mode"] == 16 else 16
    alg_bytes = npix * (12 + 16) + 2 * rec_bytes * npix * S_eff + n_v * 56 + n_tri * (64 + 64) + n_v * 24
    px_s = prof["pixels"] / 1e3
    ach = alg_bytes / px_s / 1e9
    traffic = read_traffic()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    sm_mhz = clocks.get("sm_mhz") or 1900.0
    fp32_peak = sms * 128 * sm_mhz * 1e6 / 1e12  # T lane-ops/s, FMA counted once
    # FP32 lane-ops: 18 per slab test, 61 per Moller-Trumbore test, ~60 per
    # ray for generation/shading, 19 per footprint test of a screen-tile or
    # light-cell list (box: 4 compares, 3 edge lines: 2 mul, 2 add, 1 compare
    # each), ~120 per shaded edge sample (edge_grad etc.)
    ops = (18 * work["box_tests"] + 61 * work["tri_tests"] + 60 * work["rays"] + 19 * work["footprint_tests"] +
           120 * work["edge_samples"])
    iter_s = prof["total"] / 1e3
    line = {
        "metric": "fwd+adjoint iters/s", "value": value, "unit": "iters/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded icosphere/cube, rendered targets)",
        "config": {"workload": w["name"], "triangles": n_tri, "vertices": n_v, "resolution": w["res"],
                   "views": w["views"], "spp": w["spp"], "edge_samples_per_view": edge_samples,
                   "shading": S.name, "l2": "flushed (256 MiB write) before every timed step",
                   "parallelism": "replicas", "step": "d_render_and_compare + Adam + BVH refit (CUDA graph)",
                   "bvh": args.bvh,
                   "autotuned": tuned},
        "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99))},
        "clocks": clocks,
        "e2e": {"value": e2e_value, "unit": "iters/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "api": "drgb_commit (scene from host memory) + drgb_d_render_and_compare (host pointers, pinned)",
                "p50_ms": float(np.percentile(e2e_ms, 50)), "p99_ms": float(np.percentile(e2e_ms, 99))},
        "gpu_launches": int(launches),
        "phases_ms": prof,
        "deterministic": deterministic,
        "edge_set_silhouette": silhouette,
        "work_per_iter": work,
        "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s", "frac": ach / hbm_peak,
                     "traffic": traffic, "kernel": "k_pixels (forward+loss+interior adjoint)",
                     "note": "algorithmic bytes / CUDA-event time of the pixel phase; the kernel is bound by FP32 "
                             "issue and latency, see roofline_fp32"},
        "roofline_fp32": {"bound": "fp32", "achieved": ops / iter_s / 1e12, "peak": fp32_peak, "unit": "Tops/s",
                          "frac": ops / iter_s / 1e12 / fp32_peak,
                          "peak_source": "nominal: SMs x 128 FP32 lanes x median sampled SM clock "
                                         "(MEASURED_PEAKS.json has no FP32 figure)",
                          "ops_per_iter": ops},
        "final_loss": losses[-1] if losses else None,
    }
    del opt, r, r2
    if w is WORKLOADS["icosphere"] and not args.no_patterns:
        # the small workload at its own size (the reference arm times it at full size too)
        line["cube"] = single_job_rate(WORKLOADS["cube"], local, args.steps, args.warmup)
        # the batched and served forms against the plain one-job-at-a-time path on the same GPU:
        # 64 uneven jobs, and a Poisson trace of 16 jobs at 20 jobs/s with an HBM budget of 150 GB
        line["batched"] = batch_measure(local, 64, max(3, min(args.steps, 5)), min(args.warmup, 3))
        line["served"] = serve_measure(local, 16, 0, 20.0, min(args.warmup, 3))
    if ws == 1 and rank == 0 and not args.no_cpu_baseline:
        t, factor, cores, kind, desc = cpu_sample(w)
        line["cpu_baseline"] = {"value": 1.0 / t, "unit": "iters/s", "cores": cores, "kind": kind, "sample": desc,
                                "host_cores": os.cpu_count() or 1}
    if rank == 0:
        print(json.dumps(line), flush=True)


def single_job_rate(w, local, steps, warmup):
    """Optimiser iterations/s of one job of workload w (graph replays timed
    with CUDA events on the renderer's stream, L2 flushed before each)."""
    import torch
    import diffrender_tutorials_gb300 as D
    ts, isc, cams = make_problem(w)
    S = D.SHADING_MODEL(w["mode"])
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(S, w["spp"]), device=local)
    r.commit(ts)
    targets = r.render(ts, cams)
    p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.01)
    p.base_lr = 0.01
    p.flags = D.OptimizerParameters._OPT_POS | D.OptimizerParameters._OPT_COL
    opt = D.CreateSimpleOptimizer()
    opt.Init(isc, r, cams, targets, p)
    opt.autotune(2)
    stream = torch.cuda.ExternalStream(r.stream(), device=local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    opt.run_async(warmup)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(stream):
        for e0, e1 in ev:
            flush.zero_()
            e0.record(stream)
            opt.run_async(1)
            e1.record(stream)
    torch.cuda.synchronize()
    ms = [e0.elapsed_time(e1) for e0, e1 in ev]
    return {"workload": w["name"], "value": steps / (sum(ms) / 1e3), "unit": "iters/s",
            "ms_per_step": sum(ms) / steps, "steps": steps}


def batch_measure(local, jobs, steps, warmup, mix="c4"):
    """64 uneven optimisation jobs: batched (one fused launch sequence per
    iteration, CUDA graph) against the plain path (each job's own iteration
    graph, one job at a time).  Returns the measurement as a dict."""
    import torch
    import diffrender_tutorials_gb300 as D
    from diffrender_tutorials_gb300 import workloads as WL
    torch.cuda.set_device(local)
    if mix == "small":  # jobs too small to fill the GPU alone
        specs = WL.batch_jobs(jobs, seed=0, tri_range=(200, 3_000), resolutions=(64, 96, 128), spps=(4, 8),
                              views=(1, 2))
    else:
        specs = WL.batch_jobs(jobs, seed=0)
    setups = []
    for sp in specs:
        ts, isc = D.Scene(), D.Scene()
        ts.add_mesh(sp.true_mesh)
        isc.add_mesh(sp.init_mesh)
        r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL(sp.mode), sp.spp), device=local)
        r.commit(ts)
        setups.append((isc, sp.cams, r.render(ts, sp.cams), sp))
        del r

    def params():
        p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.005)
        p.base_lr = 0.005
        p.flags = D.OptimizerParameters._OPT_POS | D.OptimizerParameters._OPT_COL
        return p

    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    # batched
    b = D.BatchOptimizer(device=local)
    for isc, cams, tgt, sp in setups:
        b.add_job(isc, cams, tgt, D.DiffRenderSettings(D.SHADING_MODEL(sp.mode), sp.spp), params())
    tuned = b.autotune(2)
    b.run(warmup)
    bs = torch.cuda.ExternalStream(b.stream(), device=local)
    st = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    en = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    k0 = D.kernel_launches()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        with torch.cuda.stream(bs):
            for i in range(steps):
                flush.zero_()
                st[i].record(bs)
                b.run_async(1)
                en[i].record(bs)
        torch.cuda.synchronize()
    b.sync()
    launches = D.kernel_launches() - k0
    step_ms = [s.elapsed_time(e) for s, e in zip(st, en)]
    batched_ms = sum(step_ms)
    n = len(setups)
    batched = n * steps / (batched_ms / 1e3)
    del b
    # plain: one job at a time
    opts = []
    for isc, cams, tgt, sp in setups:
        r = D.MakeDifferentialRenderer(D.DiffRenderSettings(D.SHADING_MODEL(sp.mode), sp.spp), device=local)
        o = D.CreateSimpleOptimizer()
        o.Init(isc, r, cams, tgt, params())
        o.autotune(2)
        o.run_async(warmup)
        opts.append((r, o))
    torch.cuda.synchronize()
    plain_ms = 0.0
    job_ms = []
    for i in range(steps):
        # L2 flushed once per step, as for the batched arm (not before every job)
        flush.zero_()
        torch.cuda.synchronize()
        for r, o in opts:
            s = torch.cuda.ExternalStream(r.stream(), device=local)
            with torch.cuda.stream(s):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(s)
                o.run_async(1)
                e1.record(s)
            e1.synchronize()
            job_ms.append(e0.elapsed_time(e1))
            plain_ms += job_ms[-1]
    del opts
    plain = n * steps / (plain_ms / 1e3)
    tris = [sp.triangles for _, _, _, sp in setups]
    return {
        "value": batched, "unit": "job-iters/s", "steps": steps, "warmup": warmup,
        "ms_per_step": batched_ms / steps,
        "config": {"workload": f"batch{n}_{'small_' if mix == 'small' else ''}displaced_spheres_lambert_pointlight",
                   "jobs": n, "triangles_min": min(tris), "triangles_max": max(tris),
                   "resolutions": sorted({sp.cams[0].width for *_, sp in setups}),
                   "spp": sorted({sp.spp for *_, sp in setups}), "l2": "flushed (256 MiB write) before every step",
                   "autotuned": tuned, "plain_autotuned": "each job's tile and grids by drgb_optimizer_autotune"},
        "plain": {"value": plain, "unit": "job-iters/s", "ms_per_step": plain_ms / steps,
                  "latency_ms": {"job_iteration_p50": float(np.percentile(job_ms, 50)),
                                 "job_iteration_p99": float(np.percentile(job_ms, 99))},
                  "how": "each job's own iteration graph, one job at a time; L2 flushed once per step of all jobs"},
        "speedup_vs_plain": batched / plain,
        "latency_ms": {"p50": float(np.percentile(step_ms, 50)), "p99": float(np.percentile(step_ms, 99))},
        "clocks": clk.summary(), "gpu_launches": int(launches),
    }


def batch_arm(args, ws, rank, local, pg):
    from diffrender_tutorials_gb300 import build as B
    B.build()
    m = batch_measure(local, args.jobs, args.steps, args.warmup, args.mix)
    line = {"metric": "batched fwd+adjoint job-iterations/s", "value": m.pop("value"), "unit": m.pop("unit"),
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": m.pop("ms_per_step"),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded displaced spheres)", "config": dict(m.pop("config"), parallelism="replicas")}
    m.pop("steps")
    m.pop("warmup")
    line.update(m)
    if rank == 0:
        print(json.dumps(line), flush=True)


def stress_problem(n_tris=200_000, res=1024, seed=0):
    """Displaced sphere (8 seeded radial sinusoids, amplitude 0.05) with about
    n_tris triangles, the 2-bounce diffuse path model, one view."""
    import diffrender_tutorials_gb300 as D
    from diffrender_tutorials_gb300 import workloads as WL
    true = WL.sphere_with_triangles(n_tris, seed=seed)
    init = D.perturb_vertices(true, 0.01, seed=seed + 2, radial=True)
    ts, isc = D.Scene(), D.Scene()
    ts.add_mesh(true)
    isc.add_mesh(init)
    cams = [D.CamInfo(origin=(0.0, 0.4, 2.6), width=res, height=res)]
    return ts, isc, cams


def instances_problem(n_inst=64, sub=4, res=512, views=4, seed=0):
    """One icosphere (sub 4: 5,120 triangles) instanced on a 4x4x4 grid: scale
    0.35, translations chosen so that the traced spheres (the instance
    transform is applied twice, as the reference's brute-force caster does)
    sit 0.5 apart with radius 0.12.  The initial scene moves every instance
    by N(0, 0.02) per axis; ring cameras."""
    import diffrender_tutorials_gb300 as D
    rng = np.random.default_rng(seed)
    mesh = D.make_icosphere(sub, seed=1)
    s = 0.35
    side = round(n_inst ** (1 / 3))
    true_tr, init_tr = [], []
    for i in range(n_inst):
        c = np.array([i % side, (i // side) % side, i // (side * side)], np.float64)
        c = (c - (side - 1) / 2) * 0.5
        for lst, off in ((true_tr, 0.0), (init_tr, rng.normal(0.0, 0.02, 3))):
            m = np.eye(4, dtype=np.float32)
            m[0, 0] = m[1, 1] = m[2, 2] = s
            m[:3, 3] = (c / (1 + s) + off).astype(np.float32)
            lst.append(m)
    ts, isc = D.Scene(), D.Scene()
    ts.add_mesh(mesh, true_tr)
    isc.add_mesh(mesh, init_tr)
    cams = D.ring_cameras(views, 3.0, res, res)
    return ts, isc, cams


def instances_arm(args, ws, rank, local, pg):
    """Instanced scene (64 instances of a 5,120-triangle icosphere, point
    light, 4 views at 512x512, 16 spp), instance transforms optimised: the
    flat binned-SAH hierarchy over all 327,680 triangles against the two-level
    build (one hierarchy per mesh, shared by its instances, under one over the
    instances).  Per builder: the commit (flatten + host build + refit), the
    iteration rate with refits only, and with a rebuild every 10 iterations."""
    import time
    import torch
    import diffrender_tutorials_gb300 as D
    from diffrender_tutorials_gb300 import build as B
    from diffrender_tutorials_gb300 import native as N
    B.build()
    torch.cuda.set_device(local)
    ts, isc, cams = instances_problem()
    S = D.SHADING_MODEL.LAMBERT_POINT_VCOLOR
    spp = 16
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(S, spp), device=local)
    r.commit(ts)
    tgt = r.render(ts, cams)
    p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.0, transforms_lr=0.002)
    p.flags = D.OptimizerParameters._OPT_TFM
    n_tri = sum(m.face_count * len(t) for m, t in zip(isc.meshes, isc.transforms))
    out = {}
    for label, builder in (("lbvh", 0), ("flat_sah", 3), ("two_level", 1)):  # 1: the default, two-level here
        commit_ms = []
        for _ in range(3):  # a new renderer each time: a commit of the same triangles keeps the topology
            rb = D.MakeDifferentialRenderer(D.DiffRenderSettings(S, spp), device=local)
            rb.set_option(N.OPT_BVH_BUILDER, builder)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rb.commit(isc)
            torch.cuda.synchronize()
            commit_ms.append((time.perf_counter() - t0) * 1e3)
            del rb
        res = {"commit_ms": float(np.median(commit_ms))}
        for period in (0, 10):
            ro = D.MakeDifferentialRenderer(D.DiffRenderSettings(S, spp), device=local)
            ro.set_option(N.OPT_BVH_BUILDER, builder)
            ro.set_option(N.OPT_PRIMARY_RASTER, RASTER[args.raster])
            ro.set_option(N.OPT_BVH_REBUILD, period)
            opt = D.CreateSimpleOptimizer()
            opt.Init(isc, ro, cams, tgt, p)
            stream = torch.cuda.ExternalStream(ro.stream(), device=local)
            for _ in range(args.warmup):
                opt.run_async(1)
            torch.cuda.synchronize()
            with ClockSampler(local) as clk:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                with torch.cuda.stream(stream):
                    e0.record(stream)
                    opt.run_async(args.steps)
                    e1.record(stream)
                torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            key = "refit_only" if period == 0 else "rebuild_every_10"
            res[key] = {"value": args.steps / (ms / 1e3), "ms_per_step": ms / args.steps, "clocks": clk.summary()}
            if period == 0:
                res[key]["phases_ms"] = opt.profile(2)
            del opt, ro
        out[label] = res
    best = out["two_level"]["rebuild_every_10"]
    line = {
        "metric": "fwd+adjoint iters/s", "value": best["value"], "unit": "iters/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": best["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (instanced icosphere grid)",
        "config": {"workload": f"instances64_icosphere5120_pointlight_4views_512x512_16spp", "triangles": n_tri,
                   "instances": 64, "optimised": "instance transforms", "bvh_rebuild_period": 10,
                   "l2": "inputs larger than L2 (flattened scene + hierarchy ~60 MB, image buffers ~50 MB)",
                   "parallelism": "replicas"},
        "builders": out,
        "clocks": best["clocks"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def fd_check(r, isc, cams, tgt, grad_pos, coords, h=1e-3):
    """Central finite differences of the loss at `coords` (flat vertex
    coordinate indices of mesh 0) against the gradient's position block."""
    import diffrender_tutorials_gb300 as D
    fd = []
    scratch = D.DScene(r, [0])
    for c in coords:
        vals = []
        for sgn in (1.0, -1.0):
            s = isc.copy()
            v = s.meshes[0].vertices.reshape(-1)
            v[c] = np.float32(v[c] + sgn * h)
            r.commit(s)
            vals.append(r.d_render_and_compare(s, cams, tgt, 0, scratch))
        fd.append((vals[0] - vals[1]) / (2 * h))
    r.commit(isc)
    # the returned loss is the MSE / (views*W*H) while the adjoint 2(I-T), and
    # so the gradient, belong to the sum of squared errors (src/drender.h:184-190)
    n_pix = sum(int(c.width) * int(c.height) for c in cams)
    fd = np.asarray(fd, np.float64) * n_pix
    g = np.asarray(grad_pos[coords], np.float64)
    rel = float(np.linalg.norm(g - fd) / max(np.linalg.norm(fd), 1e-30))
    big = np.abs(fd) > 0.1 * np.abs(fd).max()
    return {"coords": len(coords), "rel_l2": rel,
            "sign_agreement": float(np.mean(np.sign(g[big]) == np.sign(fd[big]))) if big.any() else None,
            "correlation": float(np.corrcoef(g, fd)[0, 1]) if np.std(g) > 0 and np.std(fd) > 0 else None,
            "slope": float(np.dot(g, fd) / max(np.dot(fd, fd), 1e-30)),
            "fd_norm": float(np.linalg.norm(fd)), "grad_norm": float(np.linalg.norm(g))}


def stress_arm(args, ws, rank, local, pg):
    """Differentiation stress: 200k-triangle displaced sphere, 2-bounce path
    model, 1024x1024, 4 spp, 1,048,576 edge samples.  Re-traced vs stored
    adjoint hits (bytes of the hit buffer), and the gradient against central
    finite differences (h = 1e-3) on 64 seeded vertex coordinates."""
    import torch
    import diffrender_tutorials_gb300 as D
    from diffrender_tutorials_gb300 import build as B
    from diffrender_tutorials_gb300 import native as N
    B.build()
    torch.cuda.set_device(local)
    ts, isc, cams = stress_problem(res=args.res)
    S = D.SHADING_MODEL.PATH_DIFFUSE
    spp = 4
    r = D.MakeDifferentialRenderer(D.DiffRenderSettings(S, spp), device=local)
    r.set_option(N.OPT_BVH_BUILDER, BVH_BUILDERS[args.bvh])
    r.commit(ts)
    tgt = r.render(ts, cams)
    edge = args.res * args.res
    n_tri = isc.meshes[0].face_count
    p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.001)
    p.base_lr = 0.01
    p.flags = D.OptimizerParameters._OPT_POS | D.OptimizerParameters._OPT_COL
    results = {}
    for label, hits in (("recompute", 0), ("stored_hits", 1)):
        ro = D.MakeDifferentialRenderer(D.DiffRenderSettings(S, spp), device=local)
        ro.set_option(N.OPT_ADJOINT_HITS, hits)
        ro.set_option(N.OPT_BVH_BUILDER, BVH_BUILDERS[args.bvh])
        ro.set_option(N.OPT_PRIMARY_RASTER, RASTER[args.raster])
        opt = D.CreateSimpleOptimizer()
        opt.Init(isc, ro, cams, tgt, p)
        stream = torch.cuda.ExternalStream(ro.stream(), device=local)
        for _ in range(args.warmup):
            opt.run_async(1)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        with ClockSampler(local) as clk:
            with torch.cuda.stream(stream):
                for e0, e1 in ev:
                    e0.record(stream)
                    opt.run_async(1)
                    e1.record(stream)
            torch.cuda.synchronize()
        ms = [e0.elapsed_time(e1) for e0, e1 in ev]
        n_samples = args.res * args.res * spp
        results[label] = {"value": args.steps / (sum(ms) / 1e3), "ms_per_step": sum(ms) / args.steps,
                          "phases_ms": opt.profile(2), "clocks": clk.summary(),
                          "hit_buffer_bytes_per_iter": (2 * 16 * n_samples) if hits else 0}
        del opt, ro
    # a long run: 200 iterations with the default hierarchy rebuild every 100
    # (host SAH of 200k triangles, overlapped with the next 50 iterations)
    # against refits only
    long_run = {}
    for period in (0, 100):
        ro = D.MakeDifferentialRenderer(D.DiffRenderSettings(S, spp), device=local)
        ro.set_option(N.OPT_BVH_BUILDER, BVH_BUILDERS[args.bvh])
        ro.set_option(N.OPT_PRIMARY_RASTER, RASTER[args.raster])
        ro.set_option(N.OPT_BVH_REBUILD, period)
        opt = D.CreateSimpleOptimizer()
        opt.Init(isc, ro, cams, tgt, p)
        stream = torch.cuda.ExternalStream(ro.stream(), device=local)
        opt.run_async(args.warmup)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            opt.run_async(200)
            e1.record(stream)
        torch.cuda.synchronize()
        long_run["rebuild_every_100" if period else "refit_only"] = 200 / (e0.elapsed_time(e1) / 1e3)
        del opt, ro
    # gradient at the initial mesh and the finite-difference check
    r.commit(isc)
    ds = D.DScene(r, [0])
    r.d_render_and_compare(isc, cams, tgt, edge, ds)
    gpos = ds.get_dmeshes()[0].pos().reshape(-1).copy()
    rng = np.random.default_rng(args.seed)
    nv = isc.meshes[0].vertex_count
    coords = rng.choice(3 * nv, size=64, replace=False)
    fd_random = fd_check(r, isc, cams, tgt, gpos, coords)
    # 64 coordinates of silhouette vertices (normal nearly perpendicular to the view ray)
    V = isc.meshes[0].vertices.astype(np.float64)
    nrm = isc.meshes[0].normals.astype(np.float64)
    view = V - np.asarray(cams[0].origin, np.float64)
    cosang = np.abs(np.sum(view * nrm, 1)) / (np.linalg.norm(view, axis=1) * np.linalg.norm(nrm, axis=1))
    sil = np.argsort(cosang)[:2000]
    sv = rng.choice(sil, size=64, replace=False)
    coords_sil = 3 * sv + rng.integers(0, 3, size=64)
    fd_sil = fd_check(r, isc, cams, tgt, gpos, coords_sil)
    rec = results["recompute"]
    line = {
        "metric": "fwd+adjoint iters/s", "value": rec["value"], "unit": "iters/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": rec["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded displaced sphere)",
        "config": {"workload": f"stress_sphere{n_tri}_path2_{args.res}x{args.res}_4spp", "triangles": n_tri,
                   "resolution": args.res, "spp": spp, "edge_samples": edge, "shading": "PATH_DIFFUSE (2 bounces)",
                   "l2": "inputs larger than L2 (scene + LBVH ~40 MB, image buffers ~50 MB, edge queue 16 MB)",
                   "parallelism": "replicas"},
        "adjoint": results,
        "long_run_200_iters_per_s": long_run,
        "fd_check": {"h": 1e-3, "random_coords": fd_random, "silhouette_coords": fd_sil,
                     "note": "the method's position gradient is the edge (visibility) term only; the path "
                             "model's smooth dependence of shading on positions is not differentiated, as in "
                             "the reference (interior gradients cover the albedo only)"},
        "clocks": rec["clocks"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


def serve_setups(local, jobs, seed, rate, mix="c5"):
    """The Poisson trace with its target images rendered from the true meshes."""
    import diffrender_tutorials_gb300 as D
    from diffrender_tutorials_gb300 import workloads as WL
    if mix == "small":
        specs = WL.serving_trace(jobs, seed=seed, rate=rate, tri_range=(200, 3_000), res_range=(64, 192),
                                 views=(1, 2), steps=(50, 200))
    else:
        specs = WL.serving_trace(jobs, seed=seed, rate=rate)
    out = []
    for sp in specs:
        ts, isc = D.Scene(), D.Scene()
        ts.add_mesh(sp.true_mesh)
        isc.add_mesh(sp.init_mesh)
        st = D.DiffRenderSettings(D.SHADING_MODEL(sp.mode), sp.spp)
        r = D.MakeDifferentialRenderer(st, device=local)
        r.commit(ts)
        out.append((isc, sp.cams, r.render(ts, sp.cams), st, sp))
        del r
    return out


def serve_params(sp):
    import diffrender_tutorials_gb300 as D
    p = D.OptimizerParameters(D.OptimizerParameters.GD_Adam, pos_lr=0.002)
    p.base_lr = 0.01
    p.flags = D.OptimizerParameters._OPT_POS | D.OptimizerParameters._OPT_COL
    return p


def serve_measure(local, jobs, seed, rate, warmup, budget_gb=150.0, slots=8, mix="c5"):
    """Poisson arrivals of optimisation jobs (wall clock): the serving loop
    (continuous batching, admission by memory budget) against the plain path
    (each job alone with its own optimiser, first come first served), on the
    same trace.  Per-iteration latency = device time of the step that ran the
    iteration; per-job latency = completion - arrival.  Returns a dict."""
    import torch
    import diffrender_tutorials_gb300 as D
    torch.cuda.set_device(local)
    setups = serve_setups(local, jobs, seed, rate, mix)
    n = len(setups)
    total_iters = sum(sp.steps for *_, sp in setups)
    # warm-up: load the kernels and the graph path once
    warm = D.OptimizationServer(device=local)
    for isc, cams, tgt, st, sp in setups[:2]:
        warm.submit(isc, cams, tgt, st, serve_params(sp), warmup)
    warm.wait(0)
    warm.close()
    torch.cuda.synchronize()

    # served
    srv = D.OptimizationServer(device=local, hbm_budget_bytes=int(budget_gb * 1e9), max_jobs=slots)
    k0 = D.kernel_launches()
    h2d = 0
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        tickets = []
        for isc, cams, tgt, st, sp in setups:
            dt = t0 + sp.arrival - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            tickets.append(srv.submit(isc, cams, tgt, st, serve_params(sp), sp.steps))
            h2d += tgt.nbytes + sum(m.vertices.nbytes + m.indices.nbytes + (m.colors.nbytes if m.colors is not None
                                                                              else 0) for m in isc.meshes)
        srv.wait(0)
    launches = D.kernel_launches() - k0
    stats = srv.stats()
    infos = [srv.info(t) for t in tickets]
    assert all(i["state"] == "done" for i in infos), [i["state"] for i in infos]
    ms, resident = srv.step_times()
    d2h = sum(sum(m.vertices.nbytes + (m.colors.nbytes if m.colors is not None else 0) for m in s[0].meshes) +
              4 * sp.steps for s, sp in zip(setups, [x[4] for x in setups]))
    first = min(i["t_submit"] for i in infos)
    makespan = max(i["t_done"] for i in infos) - first
    served = total_iters / makespan
    job_lat = [i["t_done"] - i["t_submit"] for i in infos]
    it_lat = np.repeat(ms, resident)  # every resident job's iteration took the step's time
    srv.close()

    # plain: one job at a time in arrival order, each with its own optimiser
    plain_it, plain_job = [], []
    plain_busy = 0.0
    t0 = time.perf_counter()
    for isc, cams, tgt, st, sp in setups:
        dt = t0 + sp.arrival - time.perf_counter()
        if dt > 0:
            time.sleep(dt)
        r = D.MakeDifferentialRenderer(st, device=local)
        o = D.CreateSimpleOptimizer()
        o.Init(isc, r, cams, tgt, serve_params(sp))
        s = torch.cuda.ExternalStream(r.stream(), device=local)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(sp.steps)]
        with torch.cuda.stream(s):
            for e0, e1 in ev:
                e0.record(s)
                o.run_async(1)
                e1.record(s)
        ev[-1][1].synchronize()
        o.current_scene()  # results back on the host, as the server does
        plain_job.append(time.perf_counter() - t0 - sp.arrival)
        its = [e0.elapsed_time(e1) for e0, e1 in ev]
        plain_busy += sum(its) / 1e3
        plain_it += its
        del o, r
    plain_makespan = time.perf_counter() - t0 - setups[0][4].arrival
    plain = total_iters / plain_makespan

    pct = lambda xs, q: float(np.percentile(np.asarray(xs, np.float64), q))  # noqa: E731
    tris = [sp.triangles for *_, sp in setups]
    res = [sp.cams[0].width for *_, sp in setups]
    return {
        "value": served, "unit": "iters/s", "steps": total_iters, "warmup": warmup,
        "ms_per_step": 1e3 / served,
        "config": {"workload": f"serve{n}_{'small_' if mix == 'small' else ''}poisson{rate:g}_displaced_spheres",
                   "jobs": n, "rate_per_s": rate,
                   "triangles": [min(tris), max(tris)], "resolution": [min(res), max(res)],
                   "views": [min(len(sp.cams) for *_, sp in setups), max(len(sp.cams) for *_, sp in setups)],
                   "steps_per_job": [min(sp.steps for *_, sp in setups), max(sp.steps for *_, sp in setups)],
                   "models": sorted({D.SHADING_MODEL(sp.mode).name for *_, sp in setups}),
                   "hbm_budget_gb": budget_gb, "slots": slots or "unlimited",
                   "l2": f"not flushed: back-to-back steps over a resident working set of "
                         f"{stats['bytes_peak'] / 1e9:.2f} GB (> L2)"},
        "latency_ms": {"iteration_p50": pct(it_lat, 50), "iteration_p99": pct(it_lat, 99),
                       "job_p50": 1e3 * pct(job_lat, 50), "job_p99": 1e3 * pct(job_lat, 99)},
        "plain": {"value": plain, "unit": "iters/s", "how": "each job alone with its own optimiser graph, "
                  "first come first served, same arrivals",
                  "latency_ms": {"iteration_p50": pct(plain_it, 50), "iteration_p99": pct(plain_it, 99),
                                 "job_p50": 1e3 * pct(plain_job, 50), "job_p99": 1e3 * pct(plain_job, 99)},
                  "gpu_busy_s": plain_busy, "makespan_s": plain_makespan},
        "speedup_vs_plain": served / plain,
        "makespan_s": makespan, "gpu_busy_s": stats["busy_seconds"], "batched_steps": int(stats["batch_steps"]),
        "resident_jobs": {"max": int(resident.max()), "mean": float(resident.mean())},
        "hbm_peak_gb": stats["bytes_peak"] / 1e9,
        "e2e": {"value": served, "unit": "iters/s", "h2d_bytes_per_step": int(h2d / total_iters),
                "d2h_bytes_per_step": int(d2h / total_iters),
                "api": "drgb_server_submit/wait (host inputs copied at submission, results copied back)"},
        "clocks": clk.summary(), "gpu_launches": int(launches),
    }


def serve_arm(args, ws, rank, local, pg):
    from diffrender_tutorials_gb300 import build as B
    B.build()
    m = serve_measure(local, args.jobs, args.seed, args.rate, args.warmup, args.budget_gb, args.slots, args.mix)
    line = {"metric": "served fwd+adjoint iters/s", "value": m.pop("value"), "unit": m.pop("unit"), "n_gpus": ws,
            "steps": m.pop("steps"), "warmup": args.warmup, "ms_per_step": m.pop("ms_per_step"),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded Poisson trace of displaced-sphere optimisation jobs)",
            "config": dict(m.pop("config"), parallelism="replicas")}
    m.pop("warmup")
    line.update(m)
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="drgb", choices=["drgb", "reference"])
    ap.add_argument("--workload", default="icosphere", choices=sorted(WORKLOADS) + ["batch", "serve", "stress", "instances"])
    ap.add_argument("--res", type=int, default=1024, help="stress: view resolution")
    ap.add_argument("--bvh", default="sah", choices=sorted(BVH_BUILDERS), help="hierarchy builder")
    ap.add_argument("--raster", default="auto", choices=sorted(RASTER),
                    help="camera and point-light shadow rays by screen tiles and light cells (DRGB_OPT_PRIMARY_RASTER)")
    ap.add_argument("--jobs", type=int, default=None, help="jobs of the batch (64) or serving (16) workload")
    ap.add_argument("--mix", default="c4", choices=["c4", "small"],
                    help="batch / serve: the configured job mix, or small jobs that cannot fill the GPU alone "
                         "(batch: 256 jobs; serve: 128 jobs at 200/s, 32 slots)")
    ap.add_argument("--rate", type=float, default=20.0, help="serving: Poisson arrival rate, jobs/s")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--budget-gb", type=float, default=150.0, help="serving: device memory budget")
    ap.add_argument("--slots", type=int, default=8, help="serving: resident jobs at most (0: no limit)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-patterns", action="store_true",
                    help="default workload: leave out the batched, served and cube measurements")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 1)
    ws, rank, local, pg = dist_setup()
    if args.impl == "reference" and args.workload not in WORKLOADS:
        # the reference's CPU path is timed on the single-job workloads only
        if rank == 0:
            print(json.dumps({"impl": "reference", "workload": args.workload,
                              "unavailable": "the reference arm times the reference's CPU d_render_and_compare on "
                                             "the single-job workloads (" + ", ".join(sorted(WORKLOADS)) + ")"}),
                  flush=True)
        if pg is not None:
            pg.destroy_process_group()
        return
    if args.workload in ("stress", "instances"):
        (stress_arm if args.workload == "stress" else instances_arm)(args, ws, rank, local, pg)
        if pg is not None:
            pg.destroy_process_group()
        return
    if args.workload in ("batch", "serve"):
        if args.jobs is None:
            args.jobs = (256 if args.mix == "small" else 64) if args.workload == "batch" else \
                (128 if args.mix == "small" else 16)
        if args.workload == "serve" and args.mix == "small":
            if args.rate == 20.0:
                args.rate = 200.0
            if args.slots == 8:
                args.slots = 32
        (batch_arm if args.workload == "batch" else serve_arm)(args, ws, rank, local, pg)
        if pg is not None:
            pg.destroy_process_group()
        return
    w = WORKLOADS[args.workload]
    if args.impl == "reference":
        reference_arm(args, w, ws, rank, pg)
    else:
        drgb_arm(args, w, ws, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
