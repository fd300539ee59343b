#!/usr/bin/env python
"""Headline benchmark: Mrays/s on the 1M-triangle soup.

Workload: 1,000,000 random triangles (centroids U[0,1]^3, seed 1, vertex
offsets U[-0.005, 0.005]), LBVH built then PHR-refined (alpha 0.5, delta 6,
branching 2), rendered at 1920x1080 with one primary ray and one
cosine-weighted diffuse bounce per pixel (spp 1, MaxDepth 0, white miss,
albedo 0.7) -- the reference's benchmark renderer (render.go:60-72) on this
scene.  A step is one frame.  Inputs (scene, BVH) are resident in HBM; L2 is
flushed (a 256 MiB write) before every timed step.

Reported:
  value        rays traced / device time of the K timed frames (CUDA events
               on the library's stream), summed over ranks / max over ranks
  e2e          the same through the C ABI's gbt_render with a pinned host
               image (the image's device->host copy is inside the timed region)
  roofline     traversal kernels: counted bytes (64 B per inner node fetched,
               48 B per primitive record tested, 32 B ray + 16 B hit per ray)
               per second against the measured HBM copy bandwidth
  cpu_baseline the C restatement of the reference (oracle/) on the host cores,
               on a bounded sample of the same workload (full frames)
  lbvh         LBVH build Mtri/s on the same scene, with its own roofline
  phr_build    wall clock of the PHR(0.5, 6, 2) refinement of that LBVH
  batch        the 64-scene batch (log-uniform 1k-2M triangles, 512x512, 16 spp,
               depth 4): the per-scene loop, the batched frame in each form and
               from a CUDA graph, and speedup_batched_vs_plain (same paths, so
               equal RMSE)
  adjoint      ms per forward + L2 loss + backward iteration on the 65k-triangle
               Cornell scene at 512x512, 64 spp
  terrain      the 8.4M-triangle terrain: LBVH Mtri/s with its roofline, the
               grid optimiser's PHR parameters, and Mrays/s of the 64 spp render

--impl reference times the reference's CPU path (the C restatement in
oracle/, since the Go reference cannot be built here) on the same workload.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W, H, SPP, MAX_DEPTH = 1920, 1080, 1, 0
N_TRI = 1_000_000
PHR = (0.5, 6.0, 2)
WORKLOAD = "soup1M_1920x1080_primary+1bounce_spp1"
# the workload both arms time (the GPU arm and --impl reference print the same dict)
CONFIG = {"workload": WORKLOAD, "triangles": N_TRI, "width": W, "height": H, "spp": SPP, "max_depth": MAX_DEPTH,
          "miss": "white", "bvh": "phr(alpha=0.5,delta=6,bf=2)", "frame": "full 1920x1080 frame per step",
          "l2": "GPU arm: flushed before every timed step (256 MiB write); CPU arm: no flush"}

# Algorithmic bytes of one LBVH build per triangle, by kernel:
#   bounds 36 (read vertices) + morton 44 (read 36, write 8-byte key)
#   + histogram 8 + 8 sort passes x 24 (read+write 8-byte key and 4-byte index)
#   + runs 28 (two key reads, 12 bytes written per run)
#   + emission 88 (index 4 + vertices 36 read, 48-byte record written)
#     + 64 (node) + 8 (runs) + 8 (codes for prefix tests)
LBVH_BYTES_PER_TRI = 36 + 44 + 8 + 8 * 24 + 28 + 88 + 64 + 8 + 8
SORT_BYTES_PER_KEY = 8 * 24


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def replica_throughput(dist, rays, ms):
    """Whole-job Mrays/s of N independent replicas: rays summed over ranks divided by the
    slowest rank's device time.  Returns (Mrays/s, max ms, total rays)."""
    ms_max = dist.reduce(ms, "max")
    rays_all = dist.reduce(rays, "sum")
    return rays_all / ms_max / 1e3, ms_max, rays_all


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    def __init__(self, ws, backend):
        self.ws = ws
        self.torch = None
        if ws > 1:
            import torch
            import torch.distributed as dist

            self.torch = torch
            dist.init_process_group(backend=backend)
            self.dist = dist

    def barrier(self):
        if self.ws > 1:
            self.dist.barrier()

    def reduce(self, x, op="max"):
        if self.ws == 1:
            return x
        t = self.torch.tensor([float(x)], dtype=self.torch.float64)
        if self.dist.get_backend() == "nccl":
            t = t.cuda()
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX if op == "max" else self.dist.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.dist.destroy_process_group()


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.p = None
        # raw samples go to a temporary file (GBT_CLOCKS_CSV keeps them at a chosen path)
        self.path = os.environ.get("GBT_CLOCKS_CSV") or os.path.join(tempfile.gettempdir(),
                                                                     "gbt_clocks_%d.csv" % os.getpid())
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.FIELDS,
                                       "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if not self.p:
            return None
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = max(mx, float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(scene, seconds=8.0, threads=None):
    """The oracle's renderer (a C restatement of render.go:91-129) on a bounded
    sample of the workload: full 1920x1080 frames of the same view, repeated
    for about `seconds`, all host threads."""
    from oracle import oracle as O

    threads = threads or (os.cpu_count() or 1)
    t0 = time.perf_counter()
    o = O.lbvh(scene["verts"], threads=threads)
    ph = o.phr(*PHR)
    build_s = time.perf_counter() - t0
    rays, el, frames, seed = 0, 0.0, 0, 1
    while el < seconds or frames == 0:
        t = time.perf_counter()
        ph.render(scene, width=W, height=H, spp=SPP, max_depth=MAX_DEPTH, seed=seed, threads=threads)
        el += time.perf_counter() - t
        rays += ph.last_rays
        frames += 1
        seed += 1
    return {"value": rays / el / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": "%d full %dx%d frames (same camera, spp %d, MaxDepth %d) on the PHR tree; %d rays in %.2f s; "
                      "CPU LBVH+PHR build %.2f s untimed" % (frames, W, H, SPP, MAX_DEPTH, rays, el, build_s)}


def run_reference(args, ws, rank):
    """--impl reference: the reference's CPU path on the host cores, on the same
    workload (full 1920x1080 frames of the PHR tree), every host thread.  The Go
    reference cannot be built on this image, so its C restatement (oracle/)
    stands in."""
    if rank != 0:
        return 0
    from oracle import oracle as O
    from trace_gb300 import scenes

    O.build()
    s = scenes.soup(N_TRI, seed=1, width=W, height=H, spp=SPP, max_depth=MAX_DEPTH)
    threads = os.cpu_count() or 1
    o = O.lbvh(s["verts"], threads=threads)
    ph = o.phr(*PHR)
    for i in range(args.warmup):
        ph.render(s, width=W, height=H, spp=SPP, max_depth=MAX_DEPTH, seed=1000 + i, threads=threads)
    rays, el = 0, 0.0
    for i in range(args.steps):
        t = time.perf_counter()
        ph.render(s, width=W, height=H, spp=SPP, max_depth=MAX_DEPTH, seed=1 + i, threads=threads)
        el += time.perf_counter() - t
        rays += ph.last_rays
    val = rays / el / 1e6
    line = {"impl": "reference", "metric": "Mrays/s", "value": val, "unit": "Mrays/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(CONFIG),
            "cpu_baseline": {"value": val, "unit": "Mrays/s", "cores": threads, "kind": "port",
                             "sample": "one full %dx%d frame per step, %d steps, %d rays" % (W, H, args.steps, rays)},
            "e2e": {"value": val, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "C restatement of pkg/pt (oracle/); the Go reference cannot be built on this image"}
    print(json.dumps(line), flush=True)
    return 0


def run_batch_workload(args):
    print(json.dumps(measure_batch(args, rebuilds=True)), flush=True)
    return 0


def measure_batch(args, rebuilds=True):
    """64 scenes of log-uniform size in [1k, 2M] triangles (seed 3), each a soup or
    an fBm terrain patch, 512x512, 16 spp, depth 4: the per-scene wavefront loop
    (gbt_render_async per scene) against the batched frame over all scenes (the
    autotuned form, and each form), that frame replayed from a CUDA graph, and the
    frame with every LBVH rebuilt first: per scene (rebuild, collapse into the
    4-wide view, render) against one graph holding the rebuilds, the collapses and
    the batched frame.  Mrays/s counts every traced ray."""
    import torch

    from trace_gb300 import _lib, pt, scenes

    count = args.batch_scenes
    ctx = pt.Context(0)
    t0 = time.perf_counter()
    ss = scenes.batch(count=count, seed=3, width=512, height=512, spp=16, max_depth=4)
    gen_s = time.perf_counter() - t0
    bvhs, cams, params, tris = [], [], [], 0
    for k, s in enumerate(ss):
        ds = pt.DeviceScene.from_dict(ctx, s)
        bvhs.append(pt.DefaultLBVH(ds))
        cams.append(s["camera"])
        p = dict(s["render"])
        p["seed"] = 1000 + k
        params.append(p)
        tris += s["verts"].shape[0]
    b = pt.Batch(ctx, bvhs, cams, params)
    stream = torch.cuda.ExternalStream(ctx.stream)
    st = _lib.RenderStats()

    def timed(mode, steps, cfg=None):
        return timed_with(b, mode, steps, cfg)

    def timed_with(obj, mode, steps, cfg=None):
        for _ in range(args.warmup):
            obj.render(mode, cfg)
        ctx.sync()
        ctx.check(ctx.L.gbt_render_last_stats(ctx.h, C.byref(st)))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            obj.render(mode, cfg)
        e1.record(stream)
        ctx.sync()
        ctx.check(ctx.L.gbt_render_last_stats(ctx.h, C.byref(st)))
        ms = e0.elapsed_time(e1) / steps
        return ms, st.rays_traced / steps

    steps = max(2, args.steps // 2)
    ms_plain, rays_plain = timed("plain", steps)
    plain = [b.read(i) for i in range(b.n)]
    forms = {}
    for name, mode, packets in (("wavefront_packets", _lib.BATCH_WAVEFRONT, 1), ("wavefront", _lib.BATCH_WAVEFRONT, 0),
                                ("megakernel", _lib.BATCH_MEGAKERNEL, 0)):
        ms_f, rays_f = timed("batched", steps, _lib.BatchConfig(128, 16, 0, mode, packets))
        forms[name] = {"value": rays_f / ms_f / 1e3, "ms_per_frame": ms_f}
    cfg, tune_ms = b.autotune()
    ms_batch, rays_batch = timed("batched", steps, cfg)
    batched = [b.read(i) for i in range(b.n)]
    b.make_graph(rebuild=False, cfg=cfg)
    ms_graph, rays_graph = timed("graph", steps)
    b.close_graph()
    diff = max(float(np.max(np.abs(x - y))) for x, y in zip(plain, batched))
    rmse = float(np.sqrt(np.mean([np.mean((x - y) ** 2) for x, y in zip(plain, batched)])))
    line = {"metric": "Mrays/s (64-scene batch)", "unit": "Mrays/s", "workload": "batch%d_512x512_spp16_depth4" % count,
            "triangles_total": tris, "scenes": count, "steps": steps,
            "plain": {"value": rays_plain / ms_plain / 1e3, "ms_per_frame": ms_plain, "rays": rays_plain},
            "batched": {"value": rays_batch / ms_batch / 1e3, "ms_per_frame": ms_batch, "rays": rays_batch,
                        "config": {"mode": ["megakernel", "wavefront"][cfg.mode], "block": cfg.block,
                                   "fetch_min": cfg.fetch_min, "stack": cfg.stack, "packets": cfg.packets},
                        "autotune_best_ms": tune_ms},
            "forms": forms,
            "graph": {"value": rays_graph / ms_graph / 1e3, "ms_per_frame": ms_graph},
            "speedup_batched_vs_plain": (rays_batch / ms_batch) / (rays_plain / ms_plain),
            "speedup_graph_vs_plain": (rays_graph / ms_graph) / (rays_plain / ms_plain),
            "images": {"max_abs_diff_batched_vs_plain": diff, "rmse_batched_vs_plain": rmse,
                       "note": "the same paths and random numbers: equal RMSE against any reference image"},
            "scene_generation_s": gen_s}
    if not rebuilds:
        b.close()
        ctx.close()
        return line
    # frames that rebuild every LBVH first
    choices = [g.packets() for g in bvhs]

    class PlainRebuild:
        def render(self, mode=None, cfg=None):
            for g in bvhs:
                ctx.check(ctx.L.gbt_lbvh_rebuild_async(ctx.h, g.h), "rebuild")
            for g, c in zip(bvhs, choices):
                g.set_layout(4)
                g.set_packets(c)  # the measured choice stays: rebuilds over unchanged vertices
            b.render("plain")

    pr = PlainRebuild()
    ms_plain_rb, _ = timed_with(pr, "plain", steps)
    b.make_graph(rebuild=True, cfg=cfg)
    ms_graph_rb, _ = timed("graph", steps)
    rebuilt = [b.read(i) for i in range(b.n)]
    diff_rb = max(float(np.max(np.abs(x - y))) for x, y in zip(plain, rebuilt))
    line["with_lbvh_rebuilds"] = {
        "plain_ms_per_frame": ms_plain_rb, "graph_ms_per_frame": ms_graph_rb,
        "plain_value": rays_plain / ms_plain_rb / 1e3, "graph_value": rays_plain / ms_graph_rb / 1e3,
        "speedup_graph_vs_plain": ms_plain_rb / ms_graph_rb,
        "max_abs_diff_graph_vs_plain": diff_rb}
    b.close()
    ctx.close()
    return line


def run_adjoint_workload(args):
    print(json.dumps(measure_adjoint(args)), flush=True)
    return 0


def measure_adjoint(args):
    """Cornell-box scene with a 256x128 sphere (65,036 triangles), per-triangle albedo and
    emission U[0.2, 0.8] (seed 4), target rendered from seed-5 parameters, 512x512,
    64 spp, depth 5: milliseconds per forward + L2 loss + backward iteration."""
    import torch

    from trace_gb300 import pt, scenes

    ctx = pt.Context(0)
    s = scenes.cornell(sphere_u=256, sphere_v=128, width=512, height=512)
    n = s["verts"].shape[0]
    ds = pt.DeviceScene.from_dict(ctx, s)
    g = pt.DefaultLBVH(ds)
    r4, r5 = np.random.default_rng(4), np.random.default_rng(5)
    a0, e0 = r4.uniform(0.2, 0.8, (n, 3)).astype(np.float32), r4.uniform(0.2, 0.8, n).astype(np.float32)
    a1, e1 = r5.uniform(0.2, 0.8, (n, 3)).astype(np.float32), r5.uniform(0.2, 0.8, n).astype(np.float32)
    f = pt.RenderFunction(g, s["camera"], dict(width=512, height=512, spp=64, max_depth=5, miss_mode=0, seed=7))
    f.set_target(f.Forward(a1, e1))
    f._set(a0, e0)
    L, h = ctx.L, ctx.h
    stream = torch.cuda.ExternalStream(ctx.stream)

    def iteration():
        ctx.check(L.gbt_adjoint_forward_async(h, g.h, C.byref(f.cam), C.byref(f.params), C.c_void_p(f.d_alb),
                                              C.c_void_p(f.d_emi), C.c_void_p(f.d_img)))
        ctx.check(L.gbt_l2_loss_async(h, C.c_void_p(f.d_img), C.c_void_p(f.d_tgt), 512 * 512 * 3,
                                      C.c_void_p(f.d_dimg), C.c_void_p(f.d_loss)))
        ctx.check(L.gbt_adjoint_backward_async(h, g.h, C.byref(f.cam), C.byref(f.params), C.c_void_p(f.d_alb),
                                               C.c_void_p(f.d_emi), C.c_void_p(f.d_dimg), C.c_void_p(f.d_ga),
                                               C.c_void_p(f.d_ge)))

    for _ in range(max(1, args.warmup)):
        iteration()
    ctx.sync()
    steps = max(2, args.steps // 2)
    e_0, e_1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_0.record(stream)
    for _ in range(steps):
        iteration()
    e_1.record(stream)
    ctx.sync()
    ms = e_0.elapsed_time(e_1) / steps
    line = {"metric": "adjoint ms/iter", "value": ms, "unit": "ms", "higher_is_better": False,
            "workload": "cornell_sphere256x128_512x512_spp64_depth5", "triangles": n,
            "parameters": n * 4, "paths_per_pass": 512 * 512 * 64, "steps": steps,
            "timed": "forward + L2 loss + backward, CUDA events on the library's stream"}
    f.close()
    ctx.close()
    return line


def run_terrain_workload(args):
    print(json.dumps(measure_terrain(args)), flush=True)
    return 0


def measure_terrain(args):
    """The 2048x2048 fBm terrain (8,380,418 triangles plus a sun sphere): LBVH build
    Mtri/s with its HBM roofline, the PHR grid optimiser and build, and Mrays/s of the
    1920x1080, 64 spp, MaxDepth 4 render (constant sky 0.5) on the chosen PHR tree.
    Inputs resident in HBM; the scene is far larger than L2."""
    import torch

    from trace_gb300 import _lib, pt, scenes

    ctx = pt.Context(0)
    t0 = time.perf_counter()
    s = scenes.terrain(2048)
    gen_s = time.perf_counter() - t0
    n = s["verts"].shape[0] + s["spheres"].shape[0]
    ds = pt.DeviceScene.from_dict(ctx, s)
    stream = torch.cuda.ExternalStream(ctx.stream)
    L, h = ctx.L, ctx.h
    aux = pt.DefaultLBVH(ds)
    steps = max(3, args.steps)
    for _ in range(args.warmup):
        ctx.check(L.gbt_lbvh_rebuild_async(h, aux.h), "rebuild")
    ctx.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        ctx.check(L.gbt_lbvh_rebuild_async(h, aux.h), "rebuild")
    e1.record(stream)
    ctx.sync()
    lb_ms = e0.elapsed_time(e1) / steps
    hbm, peak_kind = peaks()
    lb_bw = n * LBVH_BYTES_PER_TRI / (lb_ms * 1e-3) / 1e9
    rd = s["render"]
    # PHR parameters from the reference's grid optimiser (optimizer.go:44-94) over a grid that
    # reaches deep enough cuts for this scene: the sun sphere inflates the root box, so the
    # default grid's shallow cuts leave leaves of thousands of triangles
    t0 = time.perf_counter()
    opt = pt.NewGridOptimizer([0.4, 0.5, 0.55], [6, 8, 10, 12], rd["width"], rd["height"])
    alpha, delta = opt.OptimizedPHRparams(aux, 2)
    opt_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    bvh = pt.NewPHRBuilder(alpha, delta, 2).BuildFromAuxilary(aux)
    ctx.sync()
    phr_s = time.perf_counter() - t0
    cam = pt.make_camera(s["camera"])
    rp = _lib.RenderParams(rd["width"], rd["height"], rd["spp"], rd["max_depth"], rd["miss_mode"],
                           (C.c_float * 3)(*rd["miss_color"]), 7)
    d_img = ctx.alloc(rd["width"] * rd["height"] * 3 * 4)
    st = _lib.RenderStats()
    ctx.check(L.gbt_render_async(h, bvh.h, C.byref(cam), C.byref(rp), C.c_void_p(d_img)), "render")
    ctx.sync()
    ctx.check(L.gbt_render_last_stats(h, C.byref(st)))
    frames = 2
    e0.record(stream)
    for _ in range(frames):
        ctx.check(L.gbt_render_async(h, bvh.h, C.byref(cam), C.byref(rp), C.c_void_p(d_img)), "render")
    e1.record(stream)
    ctx.sync()
    ctx.check(L.gbt_render_last_stats(h, C.byref(st)))
    ms = e0.elapsed_time(e1) / frames
    img = np.empty((rd["height"], rd["width"], 3), np.float32)
    ctx.d2h(img, d_img)
    ctx.sync()
    ctx.free(d_img)
    line = {"metric": "Mrays/s (terrain)", "value": st.rays_traced / frames / ms / 1e3, "unit": "Mrays/s",
            "workload": "terrain2048_1920x1080_spp64_depth4", "triangles": n, "ms_per_frame": ms,
            "rays_per_frame": st.rays_traced / frames, "image_mean": float(img.mean()),
            "lbvh": {"mtri_s": n / lb_ms / 1e3, "ms": lb_ms, "steps": steps,
                     "roofline": {"bound": "hbm", "achieved": lb_bw, "peak": hbm, "unit": "GB/s", "frac": lb_bw / hbm,
                                  "bytes_per_tri": LBVH_BYTES_PER_TRI, "peak_source": peak_kind,
                                  "traffic": LBVH_TRAFFIC_PER_TRI["terrain2048"] * n,
                                  "traffic_scope": "DRAM bytes of one build (17 launches), ncu cold-cache capture",
                                  "kernel": "whole build (17 launches)"}},
            "phr": {"alpha": alpha, "delta": delta, "sah_cost": bvh.Cost(), "lbvh_sah_cost": aux.Cost(),
                    "build_s_wall": phr_s, "optimizer_s_wall": opt_s,
                    "grid": [{"alpha": a, "delta": d, "sah": c, "build_cost": b} for a, d, c, b in opt.evaluations]},
            "scene_generation_s": gen_s}
    ctx.close()
    return line


def run_lbvh_workload(args):
    """LBVH build throughput alone: the 1M soup and the 8.4M-triangle terrain (with its
    sun sphere), K timed rebuilds each after W warm-up builds, CUDA events on the
    library's stream, inputs resident in HBM."""
    import torch

    from trace_gb300 import pt, scenes

    ctx = pt.Context(0)
    stream = torch.cuda.ExternalStream(ctx.stream)
    hbm, peak_kind = peaks()
    out = {"metric": "LBVH Mtri/s", "unit": "Mtri/s", "bytes_per_tri": LBVH_BYTES_PER_TRI, "peak": hbm,
           "peak_source": peak_kind}
    for name, s in (("soup1M", scenes.soup(N_TRI, seed=1)), ("terrain2048", scenes.terrain(2048))):
        ds = pt.DeviceScene.from_dict(ctx, s)
        n = ds.n_prim
        aux = pt.DefaultLBVH(ds)
        for _ in range(max(1, args.warmup)):
            ctx.check(ctx.L.gbt_lbvh_rebuild_async(ctx.h, aux.h), "rebuild")
        ctx.sync()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            ctx.check(ctx.L.gbt_lbvh_rebuild_async(ctx.h, aux.h), "rebuild")
        e1.record(stream)
        ctx.sync()
        ms = e0.elapsed_time(e1) / args.steps
        bw = n * LBVH_BYTES_PER_TRI / (ms * 1e-3) / 1e9
        out[name] = {"triangles": n, "ms": ms, "mtri_s": n / ms / 1e3, "achieved_gbs": bw, "frac": bw / hbm}
        aux.close()
        ds.close()
    print(json.dumps(out), flush=True)
    return 0


def run_profile_case(args):
    """The benchmark's scene, without timing: a case small enough for an ncu capture
    (about 0.3 GB on the device for the soup, 3 GB for the terrain).  `render`: 3
    frames on the chosen tree; `lbvh`: 3 LBVH builds (the first one allocates);
    `phr`: 3 PHR refinements of the scene's LBVH."""
    from trace_gb300 import _lib, pt, scenes

    if args.profile == "batch":
        return run_profile_batch(args)
    ctx = pt.Context(0)
    if args.profile_scene == "terrain":
        s = scenes.terrain(2048)
    else:
        s = scenes.soup(N_TRI, seed=1, width=W, height=H, spp=SPP, max_depth=MAX_DEPTH)
    ds = pt.DeviceScene.from_dict(ctx, s)
    aux = pt.DefaultLBVH(ds)
    if args.profile == "lbvh":
        for _ in range(3):
            ctx.check(ctx.L.gbt_lbvh_rebuild_async(ctx.h, aux.h), "rebuild")
        ctx.sync()
        print("profile case lbvh: 3 builds of %d triangles" % s["verts"].shape[0])
        return 0
    if args.profile == "phr":
        params = (PHR[0], PHR[1], args.phr_bf)
        times = []
        for _ in range(3):
            t0 = time.perf_counter()
            b = pt.NewPHRBuilder(*params).BuildFromAuxilary(aux)
            ctx.sync()
            times.append((time.perf_counter() - t0) * 1e3)
            b.close()
        print("profile case phr: 3 PHR%s builds of %d triangles, wall ms %s" % (
            str(params), s["verts"].shape[0], " ".join("%.2f" % t for t in times)))
        return 0
    bvh = pt.NewPHRBuilder(*PHR).BuildFromAuxilary(aux) if args.bvh == "phr" else aux
    ctx.check(ctx.L.gbt_bvh_set_layout(ctx.h, bvh.h, args.layout), "layout")
    cam = pt.make_camera(s["camera"])
    rp = _lib.RenderParams(W, H, SPP, MAX_DEPTH, pt.MISS_WHITE, (C.c_float * 3)(1, 1, 1), 7)
    d_img = ctx.alloc(W * H * 3 * 4)
    for _ in range(3):
        ctx.check(ctx.L.gbt_render_async(ctx.h, bvh.h, C.byref(cam), C.byref(rp), C.c_void_p(d_img)), "render")
    ctx.sync()
    ctx.free(d_img)
    print("profile case render: 3 frames on %s" % args.bvh)
    return 0


def run_profile_batch(args):
    """The 64-scene batch without timing, for a launch-list capture: one warm frame of each
    form, then 2 frames of the per-scene loop (gbt_render_batch_plain_async) and 2 of the
    batched wavefront, each frame's device time printed from CUDA events so that the
    launch list's kernel durations can be set against it (the difference is idle time
    between launches)."""
    import torch

    from trace_gb300 import _lib, pt, scenes

    ctx = pt.Context(0)
    ss = scenes.batch(count=args.batch_scenes, seed=3, width=512, height=512, spp=16, max_depth=4)
    bvhs, cams, params = [], [], []
    for k, s in enumerate(ss):
        bvhs.append(pt.DefaultLBVH(pt.DeviceScene.from_dict(ctx, s)))
        cams.append(s["camera"])
        p = dict(s["render"])
        p["seed"] = 1000 + k
        params.append(p)
    b = pt.Batch(ctx, bvhs, cams, params)
    stream = torch.cuda.ExternalStream(ctx.stream)
    cfg = _lib.BatchConfig(128, 16, 0, _lib.BATCH_WAVEFRONT, 1)
    b.render("plain")
    b.render("batched", cfg)
    ctx.sync()
    for mode in ("plain", "plain", "batched", "batched"):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.render(mode, cfg if mode == "batched" else None)
        e1.record(stream)
        ctx.sync()
        print("profile case batch: %s frame %.3f ms" % (mode, e0.elapsed_time(e1)), flush=True)
    b.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbt", choices=["gbt", "reference"])
    ap.add_argument("--bvh", default="phr", choices=["phr", "lbvh"])
    ap.add_argument("--layout", type=int, default=4, choices=[2, 4],
                    help="traversal layout: the 4-wide view collapsed from the binary tree, or the binary nodes")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="leave out the batch, adjoint and terrain LBVH measurements of the default line")
    ap.add_argument("--cpu-seconds", type=float, default=8.0)
    ap.add_argument("--profile", choices=["render", "lbvh", "phr", "batch"], default=None,
                    help="run a small fixed case for an ncu capture and exit: 3 frames (render), 3 LBVH builds, "
                         "3 PHR refinements of the LBVH, or warm then 2+2 frames of the 64-scene batch (batch)")
    ap.add_argument("--phr-bf", type=int, default=PHR[2], choices=[2, 3, 4],
                    help="branching factor of --profile phr")
    ap.add_argument("--profile-scene", choices=["soup", "terrain"], default="soup",
                    help="scene of --profile lbvh: the 1M soup or the 8.4M-triangle terrain")
    ap.add_argument("--workload", choices=["soup", "batch", "adjoint", "terrain", "lbvh"], default="soup",
                    help="soup: the headline 1M-triangle frame; batch: the 64-scene batched render; "
                         "adjoint: forward+backward iteration of the differentiable render; "
                         "terrain: LBVH/PHR builds and the 64 spp render of the 8.4M-triangle terrain; "
                         "lbvh: LBVH build throughput on the soup and the terrain")
    ap.add_argument("--batch-scenes", type=int, default=64)
    args = ap.parse_args()
    ws, rank, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, ws, rank)
    if args.profile:
        return run_profile_case(args)
    if args.workload == "batch":
        return run_batch_workload(args)
    if args.workload == "adjoint":
        return run_adjoint_workload(args)
    if args.workload == "terrain":
        return run_terrain_workload(args)
    if args.workload == "lbvh":
        return run_lbvh_workload(args)
    args.warmup = max(args.warmup, 3)

    import torch

    from trace_gb300 import _lib, pt, scenes

    torch.cuda.set_device(local)
    dist = Dist(ws, "nccl")
    ctx = pt.Context(local)
    s = scenes.soup(N_TRI, seed=1, width=W, height=H, spp=SPP, max_depth=MAX_DEPTH)
    ds = pt.DeviceScene.from_dict(ctx, s)
    aux = pt.DefaultLBVH(ds)
    bvh_name = "lbvh"
    bvh = aux
    phr_build = None
    if args.bvh == "phr":
        try:
            bvh = pt.NewPHRBuilder(*PHR).BuildFromAuxilary(aux)
            bvh_name = "phr(alpha=0.5,delta=6,bf=2)"
            # PHR build time (host-driven, one launch per tree level): two more builds, wall clock
            walls = []
            for _ in range(2):
                ctx.sync()
                t0 = time.perf_counter()
                extra = pt.NewPHRBuilder(*PHR).BuildFromAuxilary(aux)
                ctx.sync()
                walls.append((time.perf_counter() - t0) * 1e3)
                extra.close()
            phr_build = {"ms": min(walls), "note": "wall clock of PhrBuilder.BuildFromAuxilary incl. its 4-wide view"}
        except _lib.GbtError as e:
            if e.code != -6:
                raise
    L, h = ctx.L, ctx.h
    ctx.check(L.gbt_bvh_set_layout(h, bvh.h, args.layout), "layout")
    cam = pt.make_camera(s["camera"])
    rp = _lib.RenderParams(W, H, SPP, MAX_DEPTH, pt.MISS_WHITE, (C.c_float * 3)(1, 1, 1), 7)
    d_img = ctx.alloc(W * H * 3 * 4)
    stream = torch.cuda.ExternalStream(ctx.stream)
    flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")  # 256 MiB > L2

    def flush_l2():
        with torch.cuda.stream(stream):
            flush.zero_()

    st = _lib.RenderStats()
    # warm-up
    for i in range(args.warmup):
        ctx.check(L.gbt_render_async(h, bvh.h, C.byref(cam), C.byref(rp), C.c_void_p(d_img)), "render")
    ctx.sync()
    # roofline counters: one counting frame (not timed)
    ctx.check(L.gbt_ctx_set_profiling(h, 2))
    ctx.check(L.gbt_render_last_stats(h, C.byref(st)))
    ctx.check(L.gbt_render_async(h, bvh.h, C.byref(cam), C.byref(rp), C.c_void_p(d_img)), "render")
    ctx.check(L.gbt_render_last_stats(h, C.byref(st)))
    count_stats = st.as_dict()
    # timed region: per-step events, L2 flushed before each step
    ctx.check(L.gbt_ctx_set_profiling(h, 1))
    ctx.check(L.gbt_render_last_stats(h, C.byref(st)))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    dist.barrier()
    torch.cuda.synchronize()
    ctx.sync()
    for k in range(args.steps):
        flush_l2()
        ev[k][0].record(stream)
        ctx.check(L.gbt_render_async(h, bvh.h, C.byref(cam), C.byref(rp), C.c_void_p(d_img)), "render")
        ev[k][1].record(stream)
    ctx.sync()
    torch.cuda.synchronize()
    dist.barrier()
    clk = clocks.stop()
    ctx.check(L.gbt_render_last_stats(h, C.byref(st)))
    timed = st.as_dict()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    value, ms_max, rays_all = replica_throughput(dist, timed["rays_traced"], ms)  # Mrays/s
    # roofline of the traversal kernels
    hbm, peak_kind = peaks()
    rays_per_frame = count_stats["rays_traced"]
    node_bytes = 128 if args.layout == 4 else 64
    bytes_frame = node_bytes * count_stats["nodes_visited"] + 48 * count_stats["prims_tested"] + 48 * rays_per_frame
    trav_ms_frame = timed["ms_traverse"] / args.steps
    achieved = bytes_frame / (trav_ms_frame * 1e-3) / 1e9
    roof = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": TRAVERSAL_TRAFFIC.get(bvh_name.split("(")[0]),
            "kernel": "k_trace_pt (persistent, dynamic ray fetch, %s)" % (
                "4-wide view" if args.layout == 4 else "binary nodes"),
            "traffic_scope": "DRAM bytes per frame (both traversal launches), ncu cold-cache capture",
            "peak_source": peak_kind, "bytes_per_frame": bytes_frame,
            "traversal_ms_per_frame": trav_ms_frame, "traversal_share": timed["ms_traverse"] / ms,
            "nodes_per_ray": count_stats["nodes_visited"] / rays_per_frame,
            "prims_per_ray": count_stats["prims_tested"] / rays_per_frame,
            "note": "bytes counted at the node/record level; most are L1/L2 hits, so frac can exceed 1; "
                    "camera rays run as 32-ray packets whose node and record fetches count once per warp",
            # Static figures from one ncu --set full capture of the two traversal
            # kernels on the PHR(0.5,6,2) tree of the 1M soup (not measured by this run).
            "cache_profile": {
                "source": "profiles/traversal_kernels_soup1M_phr.md (ncu --set full)",
                "l2_throughput_pct": {"camera_packets": 1.8, "anyhit_bounce": 16.4},
                "l1_hit_pct": {"camera_packets": 54.7, "anyhit_bounce": 17.1},
                "l2_hit_pct": {"camera_packets": 52.5, "anyhit_bounce": 93.5},
                "warp_efficiency": {"camera_packets": 0.94, "anyhit_bounce": 0.28}}}
    ctx.check(L.gbt_ctx_set_profiling(h, 0))

    # e2e: the C-ABI call with a pinned host image, device->host copy inside the timed region
    hp = C.c_void_p()
    ctx.check(L.gbt_host_alloc(h, W * H * 3 * 4, C.byref(hp)), "host_alloc")
    img = np.ctypeslib.as_array(C.cast(hp, C.POINTER(C.c_float)), shape=(H, W, 3))
    for i in range(2):
        ctx.check(L.gbt_render(h, bvh.h, C.byref(cam), C.byref(rp), hp, None), "render")
    ctx.check(L.gbt_render_last_stats(h, C.byref(st)))
    dist.barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        ctx.check(L.gbt_render(h, bvh.h, C.byref(cam), C.byref(rp), hp, None), "render")
    e2e_s = time.perf_counter() - t0
    dist.barrier()
    ctx.check(L.gbt_render_last_stats(h, C.byref(st)))
    e2e_rays = dist.reduce(st.rays_traced, "sum")
    e2e_s = dist.reduce(e2e_s, "max")
    assert np.isfinite(img).all()
    L.gbt_host_free(h, hp)

    # LBVH rebuild throughput on the same scene
    lb_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.warmup):
        ctx.check(L.gbt_lbvh_rebuild_async(h, aux.h), "rebuild")
    ctx.sync()
    for k in range(args.steps):
        flush_l2()
        lb_ev[k][0].record(stream)
        ctx.check(L.gbt_lbvh_rebuild_async(h, aux.h), "rebuild")
        lb_ev[k][1].record(stream)
    ctx.sync()
    lb_ms = sum(a.elapsed_time(b) for a, b in lb_ev) / args.steps
    lb_ms = dist.reduce(lb_ms, "max")
    lb_bw = N_TRI * LBVH_BYTES_PER_TRI / (lb_ms * 1e-3) / 1e9
    if phr_build is not None:
        phr_build["lbvh_plus_phr_mtri_s"] = N_TRI / (lb_ms + phr_build["ms"]) / 1e3
    lbvh = {"mtri_s": N_TRI / lb_ms / 1e3 * ws, "ms": lb_ms,
            "roofline": {"bound": "hbm", "achieved": lb_bw, "peak": hbm, "unit": "GB/s", "frac": lb_bw / hbm,
                         "bytes_per_tri": LBVH_BYTES_PER_TRI,
                         "traffic": LBVH_TRAFFIC_PER_TRI["soup1M"] * N_TRI if LBVH_TRAFFIC_PER_TRI["soup1M"] else None,
                         "traffic_scope": "DRAM bytes of one build (17 launches), ncu cold-cache capture",
                         "kernel": "whole build (17 launches)"}}

    line = {"metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": dict(CONFIG, bvh=bvh_name) if bvh_name != CONFIG["bvh"] else dict(CONFIG),
            "execution": {"traversal_layout": "%d-wide" % args.layout,
                          "camera_rays": "8x4 pixel tiles per warp", "past_max_depth": "any-hit query",
                          "rays_per_step": timed["rays_traced"] / args.steps,
                          "parallelism": "replicas" if ws > 1 else "single GPU"},
            "roofline": roof,
            "e2e": {"value": e2e_rays / e2e_s / 1e6, "unit": "Mrays/s",
                    "h2d_bytes_per_step": C.sizeof(cam) + C.sizeof(rp), "d2h_bytes_per_step": W * H * 3 * 4,
                    "api": "gbt_render (C ABI), pinned host image"},
            "gpu_launches": int(timed["kernel_launches"]),
            "clocks": clk,
            "lbvh": lbvh,
            "phr_build": phr_build}
    ctx.free(d_img)
    if ws == 1 and not args.no_extras:
        # the metric's other parts, each on its own context after the headline's timed region:
        # the 64-scene batch (batched vs the per-scene loop at equal RMSE), the adjoint's
        # ms/iter, and the terrain's LBVH Mtri/s, PHR grid choice and 64 spp render
        ctx.close()
        line["batch"] = measure_batch(args, rebuilds=False)
        line["adjoint"] = measure_adjoint(args)
        line["terrain"] = measure_terrain(args)
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(s, seconds=args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()
    return 0


# DRAM bytes per triangle of one LBVH build (dram__bytes_read.sum + dram__bytes_write.sum summed
# over the build's 17 launches, one ncu capture of the second of four builds each):
# terrain2048 3510.6 MB / 8,380,419 primitives; soup1M 366.3 MB / 1,000,000 (its keys largely
# stay in the 129 MB L2, so the capture counts fewer bytes than the algorithm moves).
LBVH_TRAFFIC_PER_TRI = {"terrain2048": 3387.0e6 / 8380419, "soup1M": 343.3e6 / 1e6}

# DRAM bytes of one headline frame's two traversal launches on the PHR tree
# (dram__bytes_read.sum + dram__bytes_write.sum of one ncu --set full capture each:
# the camera rays' packet kernel and the any-hit kernel past MaxDepth); the LBVH
# tree was not captured.
TRAVERSAL_TRAFFIC = {"lbvh": None, "phr": (147.453184 + 21.7536 + 152.9536 + 17.157376) * 1e6}

if __name__ == "__main__":
    sys.exit(main())
