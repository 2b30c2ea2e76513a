#!/usr/bin/env python3
"""Benchmark of the GB300 meshlet raster pipeline on the reference's large plain-path scene.

Workload (the headline configuration): 100k meshlets of 64 vertices / 124 triangles (12.4M
triangles), seeded, scattered in a 200^3 volume with log-uniform scale 0.1-10, 64 materials of two
2048^2 RGBA8 layers with full mips, an octahedral 1024^2 R11G11B10 sky, 1920x1080. One step is one
frame of the reference's frame driver (Main.cpp:171-261): clear, CullMeshlets then DrawMeshlets
for the node's meshlets (unbinned semantics, clipping on), Resolve, and DownsampleDepth for the
next frame. The headline frame has no previous depth (frustum culling only, every triangle
of the visible meshlets is set up); `hiz_frame` reports the following frame, whose perturbed
camera is culled against that Hi-Z (in this dense scene the occlusion test removes almost all
meshlets).

Timing: CUDA events on the library's stream (torch's current stream), L2 flushed between timed
steps by a 256 MiB write outside the step's events. `e2e` runs the same frame through the public
API with the scene uploaded from pinned host memory and the colour image read back to host memory
inside the timed region. Host-to-device copies run at about 210 GB/s on the GB300's host link
(0.82 ms for the 172.8 MB scene), so the end-to-end frame draws in batches of 16,000, 24,000,
30,000 and 30,000 meshlets whose uploads go up on a copy stream while the batches before them draw:
only the first batch's 27.6 MB upload is not overlapped. Two rasterizers on two streams take the
batches in turn, so one batch's chunk stage overlaps the next batch's mesh stage. The image goes back while the Hi-Z pyramid builds,
written straight into the pinned host buffer by the de-tiling kernel. The device-timed frame draws
the node in one call (`--frame-batch`); the reference's frame driver draws it in 65,536-meshlet
batches because its cull bitmap is a stack array of that size (Main.cpp:221-222), and the same
frame drawn that way is reported beside it (`frame_driver_batches`). All give the same image (checked). `--impl reference` times the reference's CPU algorithm (the oracle
restatement; the reference itself cannot be compiled here) on the host cores.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "1080p frame time (100k meshlets, 12.4M triangles: cull, draw, resolve, Hi-Z)"
UNIT = "ms/frame"
BATCH = 65536  # Main.cpp:222: the reference draws a node in batches of its stack cull bitmap's size


def gpu_batches(n: int, batch: int) -> list[tuple[int, int]]:
    """The GPU frames' draw calls: the whole node in one call (batch 0), or batches of `batch`
    meshlets. The reference's 65,536-meshlet batches come from its stack-allocated cull bitmap
    (Main.cpp:221-222); the device bitmap has no such limit, and every extra draw call costs the
    mesh and chunk stages' tails (keys are order-independent, so the image is the same)."""
    step = batch or n
    return [(off, min(step, n - off)) for off in range(0, n, step)]


MESHLET_BYTES = 1728  # one Meshlet record (Scene.h:15-30)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--meshlets", type=int, default=100_000)
    p.add_argument("--width", type=int, default=1920)
    p.add_argument("--height", type=int, default=1080)
    p.add_argument("--texture-size", type=int, default=2048)
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-multiview", action="store_true")
    p.add_argument("--multiview-meshlets", type=int, default=200_000)
    p.add_argument("--no-neural", action="store_true")
    p.add_argument("--neural-steps", type=int, default=20_000)
    p.add_argument("--neural-batch", type=int, default=65536)
    p.add_argument("--neural-level-weighting", type=int, default=1, choices=[0, 1, 2],
                   help="training texture level l drawn with weight 2^(w*(5-l)): 2 by texel count, 1 by edge, 0 uniform")
    p.add_argument("--materials", type=int, default=64)
    p.add_argument("--no-combined", action="store_true")
    p.add_argument("--combined-copies", type=int, default=10, help="copies of the 100k-meshlet volume (10: 1M meshlets)")
    p.add_argument("--neural-width", type=int, default=2560)
    p.add_argument("--neural-height", type=int, default=1440)
    p.add_argument("--no-alpha", action="store_true")
    p.add_argument("--no-cone", action="store_true")
    p.add_argument("--frame-batch", type=int, default=0,
                   help="meshlets per draw call of the GPU frames (0: the whole node in one call; the frame is "
                        "also timed with the reference frame driver's 65,536)")
    p.add_argument("--e2e-lanes", type=int, default=2,
                   help="rasterizer/stream pairs that take the end-to-end frame's batches in turn")
    p.add_argument("--e2e-batches", default="16000,24000,30000",
                   help="meshlets per draw batch of the end-to-end frame, comma-separated; the last size repeats "
                        "until the scene is covered (each batch's upload overlaps the draws before it)")
    p.add_argument("--multiview-cameras", type=int, default=58,
                   help="cameras besides the 6 cube faces of the multi-view workload")
    p.add_argument("--only", default="all", choices=["all", "neural", "multiview"],
                   help="neural / multiview: only that section (for profiling runs; prints that section)")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


def build_scene(args):
    from glimpsw_gb300 import scenes
    return scenes.volume_scene(n=args.meshlets, width=args.width, height=args.height, texture_size=args.texture_size,
                               n_materials=args.materials)


def default_lights():
    d = -np.array([0.589494, 0.684509, 0.428906], dtype=np.float32)
    d = (d * np.float32(1.0 / np.sqrt(np.float64((d * d).sum())))).astype(np.float32)
    return d


def config_dict(args, sc, extra=None):
    d = {"workload": f"volume scene: {args.meshlets} meshlets x 124 tris, {len(sc.materials)} materials x 2 layers "
                     f"{args.texture_size}^2 RGBA8, {args.width}x{args.height}, full frame without a previous "
                     f"depth (frustum cull, draw unbinned, resolve, Hi-Z build)",
         "meshlets": args.meshlets, "triangles": int(args.meshlets * 124), "width": args.width, "height": args.height,
         "materials": int(len(sc.materials)), "texture_size": args.texture_size,
         "l2": "flushed between timed steps (256 MiB write outside the step events)"}
    if extra:
        d.update(extra)
    return d


# ----------------------------------------------------------------------------- textures
def make_gpu_textures(sc, api):
    """Seeded value-noise materials generated on the device (identical to scenes.value_noise_rgba)."""
    import torch

    from glimpsw_gb300 import scenes
    texs = []
    for i in range(len(sc.materials)):
        t = api.Texture2D(api.FORMAT_RGBA8U, sc.texture_size, sc.texture_size, 16, 2)
        for layer in range(2):
            px = scenes.value_noise_rgba_torch(sc.texture_size, sc.texture_seed + i, layer=layer, detail=sc.texture_detail,
                                               cutout=sc.texture_cutout(i, layer))
            t.set_pixels_device(px, layer)
            torch.cuda.synchronize()
        t.generate_mips()
        texs.append(t)
    env = api.Texture2D(api.FORMAT_R11G11B10F, sc.env_size, sc.env_size, 16, 1)
    env.set_pixels(scenes.env_map_r11g11b10(sc.env_size, sc.texture_seed + 999))
    env.generate_mips()
    return texs, env


# ----------------------------------------------------------------------------- CPU frame
class OracleFrame:
    """The same frame on the CPU oracle (test infrastructure, used here only as the timed baseline),
    in one of the reference's two rasterizer configurations:
    - "binned": Rasterizer(threads) with binning (Rasterizer.cpp:493-820): meshlets strided over the
      workers, 128x128 bins rasterized by their elected worker; the resolve's 4x4 tiles split over
      the same threads (Rasterizer::Dispatch, Rasterizer.cpp:822-845);
    - "unbinned1": Rasterizer(1) without binning (DrawMeshletsST, Rasterizer.cpp:153-254), the
      shape of the reference's RasterBench (RasterBench.cpp:75-86): one thread does everything.
    Culling and the Hi-Z build run on one thread, as the reference's frame driver calls them."""

    def __init__(self, sc, tex_data, env_data, threads, mode="binned"):
        from oracle import oracle as O
        from glimpsw_gb300 import scenes
        self.O, self.sc, self.mode = O, sc, mode
        self.threads = threads if mode == "binned" else 1
        v0, v1 = sc.views
        self.v0, self.v1 = v0, v1
        self.texs = []
        for data in tex_data:
            t = O.Texture(sc.texture_size, sc.texture_size, 16, 2)
            t.data[:] = data[: t.data.size]
            self.texs.append(t)
        self.env = O.Texture(sc.env_size, sc.env_size, 16, 1, fmt=1)
        self.env.data[:] = env_data[: self.env.data.size]
        hw, hh = O.hiz_texture_size(v0.width, v0.height)
        self.hiz_in = O.Texture(hw, hh, 16, 1, fmt=2)
        self.hiz_out = O.Texture(hw, hh, 16, 1, fmt=2)
        self.fb = O.Framebuffer(v0.width, v0.height, 3)
        lights = np.zeros(1, dtype=[("type", "<u4"), ("position", "<f4", 3), ("direction", "<f4", 3), ("color", "<f4", 3),
                                    ("intensity", "<f4"), ("radius", "<f4"), ("si", "<f4"), ("so", "<f4"), ("irs", "<f4"),
                                    ("ss", "<f4"), ("sof", "<f4")])
        lights["direction"], lights["color"], lights["intensity"] = default_lights(), 1.0, 1500.0
        self.lights = lights
        self.model = scenes.IDENTITY

    def frame(self, view, prev, hiz_in, hiz_out):
        O, sc = self.O, self.sc
        n = len(sc.meshlets)
        self.fb.clear(0xFF000000, 0.0)
        for off in range(0, n, BATCH):
            cnt = min(BATCH, n - off)
            bm, _ = O.cull_meshlets(sc.meshlets[off:off + cnt], cnt, view.proj, view.view, self.model, prev.view,
                                    view.width, view.height, hiz_in)
            ctx = O.Context(sc.meshlets, sc.materials, view.world_to_clip, meshlet_offset=off, cull_bitmap=bm)
            if self.mode == "binned":
                O.draw_meshlets_binned(self.fb, ctx, cnt, self.threads)
            else:
                O.draw_meshlets(self.fb, ctx, cnt, binning=False, threads=1)
        ctx = O.Context(sc.meshlets, sc.materials, view.world_to_clip, world_to_clip=view.world_to_clip,
                        textures=self.texs, lights=self.lights, skybox=self.env, view_pos=view.eye)
        O.resolve(self.fb, ctx, threads=self.threads)
        O.downsample_depth(self.fb, hiz_out)

    def timed(self, budget_s, max_frames=50, warmup=1):
        """Median-ready frame times of the headline frame (no previous depth) after `warmup`
        untimed frames, until budget_s seconds or max_frames frames."""
        for _ in range(warmup):
            self.frame(self.v0, self.v0, None, self.hiz_out)
        times = []
        t_end = time.perf_counter() + budget_s
        while True:
            t0 = time.perf_counter()
            self.frame(self.v0, self.v0, None, self.hiz_out)
            times.append(time.perf_counter() - t0)
            if time.perf_counter() > t_end or len(times) >= max_frames:
                return times


def host_description():
    import platform
    try:
        flags = open("/proc/cpuinfo").read()
    except OSError:
        flags = ""
    return {"machine": platform.machine(), "cores": cpu_threads(), "avx512": "avx512f" in flags,
            "note": "scalar C++ restatement of the reference's AVX-512 code (the reference needs clang vector "
                    "extensions and cannot be built here)"}


def cpu_baselines(sc, tex_data, env_data, steps, warmup, unbinned_seconds=10.0):
    """Both reference configurations on this host's cores: the binned Rasterizer(threads) frame
    (steps frames after warmup, the reported value) and a bounded sample of the one-thread
    unbinned frame."""
    threads = cpu_threads()
    binned = OracleFrame(sc, tex_data, env_data, threads, "binned")
    times = binned.timed(150.0, max_frames=steps, warmup=warmup)
    single = OracleFrame(sc, tex_data, env_data, 1, "unbinned1")
    t1 = single.timed(unbinned_seconds, max_frames=steps, warmup=0)
    return {"binned_ms": float(np.median(times) * 1e3), "binned_frames": len(times), "threads": threads,
            "unbinned_1_thread_ms": float(np.median(t1) * 1e3), "unbinned_frames": len(t1), "host": host_description()}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def oracle_textures_from_host(sc):
    """Texel storage for the oracle without a GPU: same generator, built on the CPU."""
    from oracle import oracle as O
    from glimpsw_gb300 import scenes
    data = []
    for i in range(len(sc.materials)):
        t = O.Texture(sc.texture_size, sc.texture_size, 16, 2)
        for layer in range(2):
            # torch on the CPU (multi-threaded) computes the same texels as scenes.value_noise_rgba
            px = scenes.value_noise_rgba_torch(sc.texture_size, sc.texture_seed + i, layer=layer, device="cpu",
                                               detail=sc.texture_detail, cutout=sc.texture_cutout(i, layer))
            t.set_pixels(px.numpy().view(np.uint32), layer)
        t.generate_mips()
        data.append(t.data.copy())
    env = O.Texture(sc.env_size, sc.env_size, 16, 1, fmt=1)
    env.set_pixels(scenes.env_map_r11g11b10(sc.env_size, sc.texture_seed + 999))
    env.generate_mips()
    return data, env.data.copy()


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sc = build_scene(args)
    tex_data, env_data = oracle_textures_from_host(sc)
    warmup = max(3, args.warmup)
    b = cpu_baselines(sc, tex_data, env_data, args.steps, warmup)
    ms = b["binned_ms"]
    line = {"impl": "reference", "metric": METRIC, "value": ms, "unit": UNIT, "n_gpus": args.gpus,
            "steps": b["binned_frames"], "warmup": warmup, "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+i32", "data": "synthetic (seeded)",
            "config": config_dict(args, sc, {"parallelism": PARALLELISM}),
            "cpu_baseline": cpu_baseline_entry(b),
            "e2e": {"value": ms, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


PARALLELISM = "replicas only (one GPU renders the frame)"


def cpu_baseline_entry(b):
    return {"value": b["binned_ms"], "unit": UNIT, "cores": b["threads"], "kind": "port",
            "sample": f"{b['binned_frames']} full frames of the same workload (median) through the oracle's "
                      f"restatement of Rasterizer({b['threads']}) with binning: meshlets strided over "
                      f"{b['threads']} workers, 128x128 bins rasterized by their elected worker, resolve tiles "
                      f"over the same threads",
            "unbinned_1_thread": {"value": b["unbinned_1_thread_ms"], "unit": UNIT, "frames": b["unbinned_frames"],
                                  "what": "Rasterizer(1) without binning (RasterBench's shape), one thread"},
            "host": b["host"]}


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, index=0):
        self.index, self.samples = index, []
        self._stop, self._t = threading.Event(), None

    def _run(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                  "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            return
        try:
            while not self._stop.is_set():
                line = p.stdout.readline()
                if not line:
                    break
                self.samples.append([x.strip() for x in line.split(",")])
        finally:
            p.terminate()

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        self._stop.set()
        self._t.join(timeout=3)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[1]) for s in self.samples if len(s) > 2 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 2 and s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples if len(s) >= 9 for i in range(4) if s[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of the frame's kernels, from
# one ncu capture of the default workload drawn in one call (100k meshlets, 1920x1080; the capture
# used 256^2 textures, which changes only the resolve's texel addresses): k_draw_meshlets 108.83 MB
# read + 22.18 MB written, k_raster_big 52.39 + 0.42 MB, k_resolve 27.26 MB.
NCU_DRAM_BYTES_PER_LAUNCH = {"k_draw_meshlets": 131.01e6, "k_raster_big": 52.81e6, "k_resolve": 27.26e6}
NCU_WORKLOAD = (100_000, 1920, 1080)


# ----------------------------------------------------------------------------- multi-view
def multiview_section(args, api, stream):
    """64 views (6 depth-only cube faces at 1024^2 + 58 cameras of log-uniform resolution) of a
    200k-meshlet grid: one batched graph launch (autotuned chunk size and shape / warps per block) against
    64 per-view sequences of clear + frustum cull + draw through the regular entry points."""
    import torch

    from glimpsw_gb300 import autotune, scenes
    sc = scenes.multiview_scene(n=args.multiview_meshlets, n_cameras=args.multiview_cameras)
    scene = api.Scene()
    scene.upload_meshlets(sc.meshlets)
    scene.set_materials(sc.materials)
    rast = api.Rasterizer()
    rast.EnableBinning = False
    n = len(sc.meshlets)
    fbs = [api.Framebuffer(v.width, v.height) for v in sc.views]
    views = [(fb, v.proj, v.view, scenes.IDENTITY, v.depth_only) for fb, v in zip(fbs, sc.views)]
    batch = api.Batch(rast, scene, views)
    gpu = torch.cuda.get_device_name()
    best, timings = autotune.tune(batch, key=autotune.workload_key(gpu, views, n), repeats=3)
    bms = [torch.zeros((n + 15) // 16, dtype=torch.int16, device="cuda") for _ in sc.views]
    ctxs = [api.ShadingContext(scene, v.world_to_clip, cull_bitmap=bm) for v, bm in zip(sc.views, bms)]
    visible = [api.cull_meshlets(scene, 0, n, bm, v.proj, v.view, scenes.IDENTITY, v.view, v.width, v.height, None,
                                 want_count=True) for v, bm in zip(sc.views, bms)]

    def per_view():
        for fb, v, bm, ctx in zip(fbs, sc.views, bms, ctxs):
            fb.clear(0xFF000000, 0.0)
            api.cull_meshlets(scene, 0, n, bm, v.proj, v.view, scenes.IDENTITY, v.view, v.width, v.height, None)
            rast.draw_meshlets(fb, n, ctx)

    def timed(fn, steps):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return float(np.median(ms))

    batched_ms = timed(batch.render, args.steps)
    per_view_ms = timed(per_view, args.steps)
    # every view of the batch against its own per-view draw (the depth-only views hold depth alone)
    batch.reset_counters()
    batch.render()
    c = batch.counters()
    batched_layers = [(fb.get_pixels(0) if not v.depth_only else None, fb.get_pixels(1)) for fb, v in zip(fbs, sc.views)]
    per_view()
    identical = 0
    for (ids, depth), fb, v in zip(batched_layers, fbs, sc.views):
        same = np.array_equal(depth, fb.get_pixels(1)) and (ids is None or np.array_equal(ids, fb.get_pixels(0)))
        identical += int(same)
    return {"views": len(sc.views), "meshlets": n, "pixels": int(sum(v.width * v.height for v in sc.views)),
            "views_bit_identical_to_per_view_draws": f"{identical}/{len(sc.views)}",
            "visible_meshlets_per_view": {"min": int(min(visible)), "max": int(max(visible)),
                                          "total": int(sum(visible))},
            "batched_ms": batched_ms, "per_view_ms": per_view_ms, "speedup": per_view_ms / batched_ms,
            "autotuned": {"chunk_px": [best[0] * 4, best[2] * 4], "warps_per_block": best[1],
                          "candidates_ms": {f"{cw * 4}x{ch * 4}px/{w}w": round(t, 4) for (cw, w, ch), t in timings.items()}},
            "triangles_processed": int(c[0]), "gtri_per_s": float(c[0]) / (batched_ms / 1e3) / 1e9}


# ----------------------------------------------------------------------------- combined stress
def combined_section(args, api, stream):
    """Combined stress workload: 1M meshlets (10 translated copies of the volume construction,
    124M triangles, 1.73 GB of meshlet records), 256 materials of two 2048^2 RGBA8 layers, 16 views
    of 1280x720..2880x1620. One batched graph launch (autotuned chunk size and shape, warps per block)
    draws every view; each view is then resolved with the learned decoder (trained on the 256
    materials). Reports the batched raster time, the neural resolve time of all views, Gtri/s,
    HBM GB/s of the raster (algorithmic bytes: 1168 B per drawn meshlet + 16 B per pixel) and
    whether two views are bit-identical to single-view draws."""
    import torch

    from glimpsw_gb300 import autotune, scenes
    t0 = time.perf_counter()
    sc = scenes.combined_scene(copies=args.combined_copies, texture_size=args.texture_size)
    scene_s = time.perf_counter() - t0
    n = len(sc.meshlets)
    scene = api.Scene()
    scene.upload_meshlets(sc.meshlets)
    texs, env = make_gpu_textures(sc, api)
    scene.set_materials(sc.materials, texs)
    rast = api.Rasterizer()
    rast.EnableBinning = False
    fbs = [api.Framebuffer(v.width, v.height, 3) for v in sc.views]
    views = [(fb, v.proj, v.view, scenes.IDENTITY, False) for fb, v in zip(fbs, sc.views)]
    batch = api.Batch(rast, scene, views)
    gpu = torch.cuda.get_device_name()
    best, _ = autotune.tune(batch, key=autotune.workload_key(gpu, views, n), repeats=2)

    def timed(fn, steps):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return float(np.median(ms))

    raster_ms = timed(batch.render, args.steps)
    batch.reset_counters()
    batch.render()
    c = batch.counters()
    pixels = sum(v.width * v.height for v in sc.views)
    drawn = int(c[0]) // 124
    raster_bytes = drawn * 1168 + pixels * 16
    # the learned decoder over the 256 materials, then the neural resolve of every view
    model = api.NeuralMaterials(texs, latent_levels=4, seed=1)
    t1 = time.perf_counter()
    model.train(args.neural_steps, batch=args.neural_batch, materials_per_step=8,
                level_weighting=args.neural_level_weighting)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t1
    lights = [api.SwrLight()]
    lights[0].type, lights[0].intensity = 0, 1500.0
    lights[0].direction[:] = default_lights().tolist()
    lights[0].color[:] = [1.0, 1.0, 1.0]
    ctxs = [api.ShadingContext(scene, v.world_to_clip, world_to_clip=v.world_to_clip, skybox=env, view_pos=v.eye,
                               lights=lights) for v in sc.views]

    def frame():
        batch.render()
        for ctx, fb in zip(ctxs, fbs):
            ctx.resolve_neural(rast, fb, model)

    frame_ms = timed(frame, args.steps)
    # two views against single-view draws (clear, frustum cull, draw)
    batch.render()
    exact = True
    for k in (0, len(sc.views) - 1):
        v, fb = sc.views[k], fbs[k]
        ref = api.Framebuffer(v.width, v.height)
        ref.clear(0xFF000000, 0.0)
        bm = torch.zeros((n + 15) // 16, dtype=torch.int16, device="cuda")
        api.cull_meshlets(scene, 0, n, bm, v.proj, v.view, scenes.IDENTITY, v.view, v.width, v.height, None)
        rast.draw_meshlets(ref, n, api.ShadingContext(scene, v.world_to_clip, cull_bitmap=bm))
        exact = exact and np.array_equal(fb.get_pixels(0), ref.get_pixels(0)) and \
            np.array_equal(fb.get_pixels(1), ref.get_pixels(1))
    peak, peak_kind = peaks()
    return {"meshlets": n, "triangles": n * 124, "meshlet_bytes": int(sc.meshlets.nbytes), "materials": len(sc.materials),
            "views": len(sc.views), "sizes": [[v.width, v.height] for v in sc.views], "pixels": pixels,
            "scene_build_s": scene_s, "autotuned": {"chunk_px": [best[0] * 4, best[2] * 4], "warps_per_block": best[1]},
            "batched_raster_ms": raster_ms, "frame_ms_raster_plus_neural_resolve": frame_ms,
            "triangles_processed": int(c[0]), "gtri_per_s": float(c[0]) / (raster_ms / 1e3) / 1e9,
            "raster_hbm_gbs": raster_bytes / (raster_ms / 1e3) / 1e9, "hbm_peak_gbs": peak, "peak_kind": peak_kind,
            "decoder_train_s": train_s, "views_bit_identical_to_single_view_draws": bool(exact)}


# ----------------------------------------------------------------------------- alpha-tested materials
def alpha_section(args, api, stream, sc, texs, env, lights, flush):
    """The headline frame with every second material alpha-tested (FS_EncodeSurfaceId<true>,
    Shading.cpp:309-331): cutoff 128, double-sided, a noise alpha channel in layer 0 (like foliage
    cards). Same meshlets, camera and frame (cull, draw, resolve, Hi-Z); reports the frame time,
    the per-kernel split and the share of pixels showing alpha-tested materials."""
    import torch

    from glimpsw_gb300 import scenes
    sca = scenes.volume_scene(n=args.meshlets, width=args.width, height=args.height, texture_size=args.texture_size,
                              n_materials=args.materials, alpha_every=2)
    texs_a = list(texs)
    for i in range(len(sca.materials)):
        if sca.texture_cutout(i, 0):
            t = api.Texture2D(api.FORMAT_RGBA8U, sca.texture_size, sca.texture_size, 16, 2)
            for layer in range(2):
                px = scenes.value_noise_rgba_torch(sca.texture_size, sca.texture_seed + i, layer=layer,
                                                   detail=sca.texture_detail, cutout=sca.texture_cutout(i, layer))
                t.set_pixels_device(px, layer)
                torch.cuda.synchronize()
            t.generate_mips()
            texs_a[i] = t
    scene = api.Scene()
    scene.upload_meshlets(sca.meshlets)
    scene.set_materials(sca.materials, texs_a)
    rast = api.Rasterizer()
    rast.EnableBinning = False
    v0 = sca.views[0]
    W, H = v0.width, v0.height
    fb = api.Framebuffer(W, H, 3)
    n = len(sca.meshlets)
    batches = gpu_batches(n, args.frame_batch)
    bitmaps = [torch.zeros((cnt + 15) // 16, dtype=torch.int16, device="cuda") for _, cnt in batches]
    hw, hh = api.hiz_texture_size(W, H)
    hiz = api.Texture2D(api.FORMAT_R32F, hw, hh, 16, 1)

    mats = (api.mat4(v0.proj), api.mat4(v0.view), api.mat4(scenes.IDENTITY), api.mat4(v0.view))
    ctxs = [api.ShadingContext(scene, v0.world_to_clip, meshlet_offset=off, cull_bitmap=bm)
            for (off, _), bm in zip(batches, bitmaps)]
    rctx = api.ShadingContext(scene, v0.world_to_clip, world_to_clip=v0.world_to_clip, skybox=env, view_pos=v0.eye,
                              lights=lights)

    def draw():
        fb.clear(0xFF000000, 0.0)
        for (off, cnt), bm, ctx in zip(batches, bitmaps, ctxs):
            api.cull_meshlets(scene, off, cnt, bm, *mats, W, H, None)
            rast.draw_meshlets(fb, cnt, ctx)

    def frame():
        draw()
        rctx.resolve(rast, fb)
        api.downsample_depth(fb, hiz)

    for _ in range(max(3, args.warmup)):
        frame()
    torch.cuda.synchronize()
    rast.reset_counters()
    frame()
    c = rast.counters()
    ms = []
    for _ in range(args.steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        frame()
        b.record(stream)
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    api.profile_enable(True)  # per-kernel times from a second pass (events around every launch)
    for _ in range(args.steps):
        flush.zero_()
        frame()
    torch.cuda.synchronize()
    api.profile_enable(False)
    per = {}
    for name, t in api.profile_collect():
        per[name] = per.get(name, 0.0) + t / args.steps
    draw()  # the vis-buffer ids (the resolve overwrites layer 0 with colour)
    ids = fb.get_pixels(0)
    shown = ids != 0xFF000000
    mat = sca.meshlets["MaterialId"].astype(np.int64)[np.minimum(ids, n * 128 - 1) // 128]
    alpha_px = int((shown & (sca.materials["alpha_cutoff"][mat] < 255)).sum())
    return {"frame_ms": float(np.mean(ms)), "kernels_ms_per_step": dict(sorted(per.items())),
            "alpha_materials": int((sca.materials["alpha_cutoff"] < 255).sum()), "materials": len(sca.materials),
            "cutoff": 128, "triangles_processed": int(c[0]), "triangles_rasterized": int(c[1]),
            "pixels_showing_alpha_materials": alpha_px, "pixels_covered": int(shown.sum())}


# ----------------------------------------------------------------------------- backface-cone culling
def cone_section(args, api, stream, texs, env, lights, flush):
    """Backface-cone culling (swr_cull_meshlets_ex, SWR_CULL_BACKFACE_CONE) on the headline frame's
    construction with open sphere patches instead of closed hulls (scenes.patch_scene: same count,
    volume, scales, materials and camera; each patch carries its normal cone). The frame (cull,
    draw, resolve, Hi-Z) is timed with frustum culling alone and with the cone test added; reports
    both times, the meshlets each keeps and whether the two vis-buffers are identical. (The closed
    meshlets of the headline scene have degenerate cones: the test culls none of them.)"""
    import torch

    from glimpsw_gb300 import scenes
    sc = scenes.patch_scene(n=args.meshlets, width=args.width, height=args.height, texture_size=args.texture_size,
                            n_materials=args.materials)
    scene = api.Scene()
    scene.upload_meshlets(sc.meshlets)
    scene.set_materials(sc.materials, texs)
    rast = api.Rasterizer()
    rast.EnableBinning = False
    v0 = sc.views[0]
    W, H = v0.width, v0.height
    fb = api.Framebuffer(W, H, 3)
    n = len(sc.meshlets)
    batches = gpu_batches(n, args.frame_batch)
    bitmaps = [torch.zeros((cnt + 15) // 16, dtype=torch.int16, device="cuda") for _, cnt in batches]
    hw, hh = api.hiz_texture_size(W, H)
    hiz = api.Texture2D(api.FORMAT_R32F, hw, hh, 16, 1)
    mats = (api.mat4(v0.proj), api.mat4(v0.view), api.mat4(scenes.IDENTITY), api.mat4(v0.view))
    ctxs = [api.ShadingContext(scene, v0.world_to_clip, meshlet_offset=off, cull_bitmap=bm)
            for (off, _), bm in zip(batches, bitmaps)]
    rctx = api.ShadingContext(scene, v0.world_to_clip, world_to_clip=v0.world_to_clip, skybox=env, view_pos=v0.eye,
                              lights=lights)

    def draw(cone):
        fb.clear(0xFF000000, 0.0)
        for (off, cnt), bm, ctx in zip(batches, bitmaps, ctxs):
            api.cull_meshlets(scene, off, cnt, bm, *mats, W, H, None, cone=cone)
            rast.draw_meshlets(fb, cnt, ctx)

    def frame(cone):
        draw(cone)
        rctx.resolve(rast, fb)
        api.downsample_depth(fb, hiz)

    out = {"meshlets": n, "scene": "open sphere patches (20-degree caps, 64 vertices, 113 triangles) with normal cones"}
    layers = {}
    for cone in (False, True):
        for _ in range(max(3, args.warmup)):
            frame(cone)
        torch.cuda.synchronize()
        ms = []
        for _ in range(args.steps):
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            frame(cone)
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        kept = sum(api.cull_meshlets(scene, off, cnt, bm, *mats, W, H, None, want_count=True, cone=cone)
                   for (off, cnt), bm in zip(batches, bitmaps))
        draw(cone)
        layers[cone] = (fb.get_pixels(0), fb.get_pixels(1))
        key = "frustum_and_cone" if cone else "frustum_only"
        out[key] = {"frame_ms": float(np.mean(ms)), "meshlets_kept": int(kept)}
    out["cone_culled_share_of_frustum_visible"] = 1.0 - out["frustum_and_cone"]["meshlets_kept"] / max(
        1, out["frustum_only"]["meshlets_kept"])
    out["visbuffer_identical"] = bool(np.array_equal(layers[False][0], layers[True][0]) and
                                      np.array_equal(layers[False][1], layers[True][1]))
    return out


# ----------------------------------------------------------------------------- learned decoder
def texel_accuracy(api, model, texs, materials=4, n=65536, seed=7):
    """Decoded texels against the plain texels they replace, per channel group, over n random texels
    of each decoded level (levels weighted by edge length) of the first `materials` materials; the
    AO channel (no source texels) is compared with its constant target 1."""
    import torch
    rng = np.random.default_rng(seed)
    levels = np.arange(model.latent_levels + 2)
    w = 2.0 ** -levels.astype(np.float64)
    got, ref = [], []
    for mat in range(min(materials, len(texs))):
        t = texs[mat]
        data = t.get_data()
        row_shift = int(np.log2(max(t.width, 8)))
        lvl = rng.choice(levels, n, p=w / w.sum())
        x, y = rng.integers(0, t.width >> lvl), rng.integers(0, t.height >> lvl)
        off = np.asarray(t.mip_offsets, np.int64)[lvl] + ((y & 7) | (x << 3) | ((y & ~7) << (row_shift - lvl)))
        a0, a1 = data[off].astype(np.int64), data[t.layer_stride + off].astype(np.int64)
        ref.append(np.stack([a0 & 255, (a0 >> 8) & 255, (a0 >> 16) & 255, a1 & 255, (a1 >> 8) & 255, (a1 >> 16) & 255,
                             a1 >> 24, np.full(n, 255)], axis=1))
        packed = api.pack_texel(lvl, x, y).astype(np.uint32)
        out = torch.zeros(2 * n, dtype=torch.int32, device="cuda")
        model.decode(mat, torch.from_numpy(packed.view(np.int32)).cuda(), n, out)
        d = out.cpu().numpy().view(np.uint32).reshape(-1, 2).astype(np.int64)
        got.append(np.stack([d[:, 0] & 255, (d[:, 0] >> 8) & 255, (d[:, 0] >> 16) & 255, d[:, 1] & 255,
                             (d[:, 1] >> 8) & 255, (d[:, 1] >> 16) & 255, d[:, 1] >> 24, d[:, 0] >> 24], axis=1))
    got, ref = np.concatenate(got), np.concatenate(ref)

    def psnr(cols):
        mse = float(((got[:, cols] - ref[:, cols]) ** 2).mean()) / 255.0 ** 2
        return 10 * np.log10(1.0 / mse) if mse > 0 else float("inf")
    err = np.abs(got - ref)
    return {"texels": int(len(got)), "albedo_psnr_db": psnr([0, 1, 2]), "normal_xy_psnr_db": psnr([3, 4]),
            "metal_rough_psnr_db": psnr([5, 6]), "max_abs_255": {"albedo": int(err[:, :3].max()),
                                                                  "normal_xy": int(err[:, 3:5].max()),
                                                                  "metal_rough": int(err[:, 5:7].max())},
            "ao": {"target": 255, "mean": float(got[:, 7].mean()), "max_abs_255": int(err[:, 7].max())}}


def neural_section(args, api, stream, sc, texs, env, scene, rast, lights):
    """Learned texture decoder over the scene's 64 materials: trained on the device (Adam, lr 1e-3,
    `neural_steps` steps of `neural_batch` texels spread over 8 materials per step), then the scene
    is resolved at 2560x1440 with the plain sampler and with the decoder (texture levels 0-3 decoded,
    coarser levels sampled), from the headline camera and from a camera inside the volume where
    more pixels use the decoded levels. Reports training time and loss, both resolves' device time,
    PSNR / max-abs of the neural frame against the plain frame, decoded texels and memory."""
    import torch

    from glimpsw_gb300 import scenes
    model = api.NeuralMaterials(texs, latent_levels=4, seed=1)
    mps, lw = 8, args.neural_level_weighting
    loss0 = model.train(1, batch=args.neural_batch, materials_per_step=mps, want_loss=True, level_weighting=lw)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    model.train(max(args.neural_steps - 2, 0), batch=args.neural_batch, materials_per_step=mps, level_weighting=lw)
    b.record(stream)
    loss1 = model.train(1, batch=args.neural_batch, materials_per_step=mps, want_loss=True, level_weighting=lw)
    train_ms = a.elapsed_time(b)
    api.profile_enable(True)
    api.profile_collect()
    model.train(4, batch=args.neural_batch, materials_per_step=mps, level_weighting=lw)
    step_kernels = {}
    for k, t in api.profile_collect():
        step_kernels[k] = step_kernels.get(k, 0.0) + t / 4
    api.profile_enable(False)
    texel = texel_accuracy(api, model, texs)
    W, H = args.neural_width, args.neural_height
    n = len(sc.meshlets)
    batches = gpu_batches(n, args.frame_batch)
    bms = [torch.zeros((cnt + 15) // 16, dtype=torch.int16, device="cuda") for _, cnt in batches]
    fbs = [api.Framebuffer(W, H, 3), api.Framebuffer(W, H, 3)]
    eye = sc.views[0].eye
    cams = {"headline_camera": scenes.make_view(W, H, eye=eye, target=(0.0, 0.0, 0.0)),
            "interior_camera": scenes.make_view(W, H, eye=(3.0, 2.0, -20.0), target=(0.0, 0.0, 40.0))}

    def render(fb, view):
        fb.clear(0xFF000000, 0.0)
        for (off, cnt), bm in zip(batches, bms):
            api.cull_meshlets(scene, off, cnt, bm, view.proj, view.view, scenes.IDENTITY, view.view, W, H, None)
            rast.draw_meshlets(fb, cnt, api.ShadingContext(scene, view.world_to_clip, meshlet_offset=off, cull_bitmap=bm))

    out = {"training": {"steps": args.neural_steps, "batch": args.neural_batch, "materials_per_step": mps,
                        "level_weighting": lw,
                        "lr": 1e-3, "loss_first_step": loss0, "loss_last_step": loss1, "train_ms": train_ms,
                        "ms_per_step": train_ms / max(args.neural_steps - 2, 1),
                        "step_kernels_ms": {k: round(v, 4) for k, v in step_kernels.items()},
                        "samples_per_s": (args.neural_steps - 2) * args.neural_batch / (train_ms / 1e3)}}
    mem = model.memory()
    neural_bytes = mem["latent_bytes"] + mem["weight_bytes"] + mem["fallback_bytes"]
    out["memory"] = {**mem, "neural_total_bytes": neural_bytes, "ratio_plain_over_neural": mem["plain_bytes"] / neural_bytes}
    out["texel_accuracy"] = texel
    for name, view in cams.items():
        ctx = api.ShadingContext(scene, view.world_to_clip, world_to_clip=view.world_to_clip, skybox=env,
                                 view_pos=view.eye, lights=lights)
        ms = {"plain": [], "neural": []}
        for i in range(args.warmup + args.steps):
            for kind, fb in zip(("plain", "neural"), fbs):
                render(fb, view)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                if kind == "plain":
                    ctx.resolve(rast, fb)
                else:
                    ctx.resolve_neural(rast, fb, model)
                e1.record(stream)
                torch.cuda.synchronize()
                if i >= args.warmup:
                    ms[kind].append(e0.elapsed_time(e1))
        render(fbs[1], view)
        depth = fbs[1].get_pixels(1)
        covered = int((depth != 0).sum())
        requests, tiles, per_level = ctx.resolve_neural(rast, fbs[1], model, want_stats=True)
        render(fbs[0], view)
        ctx.resolve(rast, fbs[0])
        pa = fbs[0].get_pixels(0).view(np.uint8).reshape(H, W, 4)[..., :3].astype(np.float64) / 255.0
        pb = fbs[1].get_pixels(0).view(np.uint8).reshape(H, W, 4)[..., :3].astype(np.float64) / 255.0
        diff = np.abs(pa - pb)
        mse = float((diff ** 2).mean())
        cov = (depth != 0)
        mse_cov = float((diff[cov] ** 2).mean()) if covered else 0.0
        out[name] = {"plain_resolve_ms": float(np.median(ms["plain"])), "neural_resolve_ms": float(np.median(ms["neural"])),
                     "psnr_db": 10 * np.log10(1.0 / mse) if mse > 0 else float("inf"),
                     "psnr_covered_pixels_db": 10 * np.log10(1.0 / mse_cov) if mse_cov > 0 else float("inf"),
                     "max_abs_255": int(round(diff.max() * 255)), "pixels_differing": int((diff.max(axis=2) > 0).sum()),
                     "covered_pixels": covered, "decoded_texels": int(requests), "decode_tiles": int(tiles),
                     "decoded_texels_per_level": [int(v) for v in per_level],
                     "plain_gpix_per_s": W * H / (np.median(ms["plain"]) / 1e3) / 1e9,
                     "neural_gpix_per_s": W * H / (np.median(ms["neural"]) / 1e3) / 1e9}
    api.profile_enable(True)
    render(fbs[1], cams["interior_camera"])
    ctx = api.ShadingContext(scene, cams["interior_camera"].world_to_clip, world_to_clip=cams["interior_camera"].world_to_clip,
                             skybox=env, view_pos=cams["interior_camera"].eye, lights=lights)
    api.profile_collect()
    ctx.resolve_neural(rast, fbs[1], model)
    out["interior_camera"]["neural_kernels_ms"] = {k: round(t, 4) for k, t in api.profile_collect()}
    api.profile_enable(False)
    return out


# ----------------------------------------------------------------------------- GPU
def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from glimpsw_gb300 import api, scenes
    api.load_library()
    if args.only == "multiview":  # the multi-view section alone (profiling runs)
        stream = torch.cuda.current_stream()
        api.set_stream(stream.cuda_stream)
        out = multiview_section(args, api, stream)
        if rank == 0:
            print(json.dumps({"multiview": out}), flush=True)
        return

    sc = build_scene(args)
    v0, v1 = sc.views
    W, H = v0.width, v0.height
    stream = torch.cuda.current_stream()
    api.set_stream(stream.cuda_stream)

    texs, env = make_gpu_textures(sc, api)
    scene = api.Scene()
    scene.upload_meshlets(sc.meshlets)
    scene.set_materials(sc.materials, texs)
    rast = api.Rasterizer()
    rast.EnableBinning = False  # the reference frame driver's setting (Main.cpp:76)
    fb = api.Framebuffer(W, H, 3)
    n = len(sc.meshlets)
    batches = gpu_batches(n, args.frame_batch)
    bitmaps = [torch.zeros((cnt + 15) // 16, dtype=torch.int16, device="cuda") for _, cnt in batches]
    hw, hh = api.hiz_texture_size(W, H)
    hiz = [api.Texture2D(api.FORMAT_R32F, hw, hh, 16, 1) for _ in range(2)]
    model = scenes.IDENTITY
    lights = [api.SwrLight()]
    lights[0].type, lights[0].intensity = 0, 1500.0
    lights[0].direction[:] = default_lights().tolist()
    lights[0].color[:] = [1.0, 1.0, 1.0]
    if args.only == "neural":  # the learned-decoder section alone (profiling runs)
        out = neural_section(args, api, stream, sc, texs, env, scene, rast, lights)
        if rank == 0:
            print(json.dumps({"neural": out, "config": config_dict(args, sc)}), flush=True)
        return

    def frame_fn(view, prev, hiz_in, hiz_out, blist=None):
        """The frame driver's sequence (Main.cpp:203-260) for one camera, drawing the meshlets in
        the batches blist (default: gpu_batches). Matrices and shading contexts are parameter
        blocks, built once per camera as a renderer keeps them."""
        blist = batches if blist is None else blist
        bms = bitmaps if blist is batches else [torch.zeros((cnt + 15) // 16, dtype=torch.int16, device="cuda")
                                                for _, cnt in blist]
        mats = (api.mat4(view.proj), api.mat4(view.view), api.mat4(model), api.mat4(prev.view))
        ctxs = [api.ShadingContext(scene, view.world_to_clip, meshlet_offset=off, cull_bitmap=bm)
                for (off, _), bm in zip(blist, bms)]
        rctx = api.ShadingContext(scene, view.world_to_clip, world_to_clip=view.world_to_clip, skybox=env,
                                  view_pos=view.eye, lights=lights)

        def run(uploaded=None, resolved=None, lanes=None):
            """uploaded: per batch, an event after which its records are on the device, or None
            (their upload then overlaps the culling and drawing of the batches before). resolved:
            an event recorded once the colour image is complete (before the Hi-Z build). lanes:
            (rasterizer, stream, event) triples that take the batches in turn, so that one batch's
            chunk stage overlaps the next batch's mesh stage (keys are order-independent); the
            first is the frame's own (rast, stream)."""
            lanes = lanes or [(rast, stream, None)]
            fb.clear(0xFF000000, 0.0)
            for r, s, ev in lanes[1:]:  # the other lanes start after the clear
                ev.record(stream)
                s.wait_event(ev)
            for k, ((off, cnt), bm, ctx) in enumerate(zip(blist, bms, ctxs)):
                r, s, _ = lanes[k % len(lanes)]
                if s is not stream:
                    api.set_stream(s)
                if uploaded is not None and uploaded[k] is not None:
                    s.wait_event(uploaded[k])
                api.cull_meshlets(scene, off, cnt, bm, *mats, W, H, hiz_in)
                r.draw_meshlets(fb, cnt, ctx)
                if s is not stream:
                    api.set_stream(stream)
            for r, s, ev in lanes[1:]:  # the resolve waits for every lane's draws
                ev.record(s)
                stream.wait_event(ev)
            rctx.resolve(rast, fb)
            if resolved is not None:
                resolved.record(stream)
            api.downsample_depth(fb, hiz_out)
        return run

    # headline frame: no previous depth (frustum culling only), so all 12.4M triangles are set up;
    # the second figure is the next frame, culled against the first frame's Hi-Z
    headline = frame_fn(v0, v0, None, hiz[0])
    hiz_frame = frame_fn(v1, v0, hiz[0], hiz[1])

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def timed(fn, steps):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for i in range(steps):
            flush.zero_()
            ev[i][0].record(stream)
            fn()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in ev]

    for _ in range(max(3, args.warmup)):
        headline()
    torch.cuda.synchronize()
    rast.reset_counters()
    headline()
    counters = rast.counters()
    rast.reset_counters()
    hiz_frame()
    hiz_counters = rast.counters()

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = api.launch_count()
    with ClockSampler(local) as clocks:
        step_ms = timed(headline, args.steps)
    launches = api.launch_count() - launches0
    ms = float(np.mean(step_ms))
    # per-kernel times: a second pass of the same steps with an event pair around every launch
    # (the events add a few microseconds per launch, so the frame time comes from the pass without)
    api.profile_enable(True)
    prof_ms = float(np.mean(timed(headline, args.steps)))
    api.profile_enable(False)
    prof = api.profile_collect()
    hiz_ms = float(np.mean(timed(hiz_frame, args.steps)))
    api.profile_enable(True)
    timed(hiz_frame, args.steps)
    api.profile_enable(False)
    hiz_per = {}
    for name, t in api.profile_collect():
        hiz_per[name] = hiz_per.get(name, 0.0) + t / args.steps
    # the same frame drawn as the reference frame driver calls it (Main.cpp:221-242)
    ref_batches = [(off, min(BATCH, n - off)) for off in range(0, n, BATCH)]
    ref_batch_frame = frame_fn(v0, v0, None, hiz[0], ref_batches)
    for _ in range(2):
        ref_batch_frame()
    ref_batch_ms = float(np.mean(timed(ref_batch_frame, args.steps)))
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())

    per = {}
    for name, t in prof:
        c, s = per.get(name, (0, 0.0))
        per[name] = (c + 1, s + t)
    peak, peak_kind = peaks()
    ids = fb.get_pixels(1)  # depth layer: sky pixels keep the clear depth 0
    covered = int((ids != 0).sum())
    # algorithmic bytes per launch (what each kernel must move at minimum)
    algo = {
        "k_draw_meshlets": (n * (1152 + 16)) / len(batches) + W * H * 16 / len(batches),
        "k_resolve": W * H * (8 + 4) + covered * 60 + covered * 2 * 4 + (W * H - covered) * 4 * 4,
        "k_raster_big": W * H * 16 / len(batches),
    }
    top_name = max((k for k in per if k in algo), key=lambda k: per[k][1])
    top_avg_s = per[top_name][1] / per[top_name][0] / 1e3
    achieved = algo[top_name] / top_avg_s / 1e9
    roofline = {"bound": "hbm", "kernel": top_name, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": NCU_DRAM_BYTES_PER_LAUNCH.get(top_name) if (n, W, H) == NCU_WORKLOAD else None,
                "algorithmic_bytes_per_launch": algo[top_name], "avg_launch_ms": top_avg_s * 1e3}

    # end to end through the public API: pinned host scene upload + frame + colour readback
    pinned = torch.empty(sc.meshlets.nbytes, dtype=torch.uint8).pin_memory()
    pinned.numpy()[:] = sc.meshlets.view(np.uint8).reshape(-1)
    host_img = torch.empty((H, W), dtype=torch.int32).pin_memory()
    # The frame draws in batches (--e2e-batches). The first batch's records go up on the frame's
    # stream; the others' on a copy stream behind it (the host link is the limit, so sharing it
    # would only delay the first batch), each followed by an event that its batch's culling waits
    # for, so each upload overlaps the culling and drawing of the batches before (every byte of the
    # scene is still copied every step). The colour image goes back on the copy stream while the
    # frame's stream builds the Hi-Z pyramid.
    sizes = [int(x) for x in args.e2e_batches.split(",")]
    eb, off = [], 0
    while off < n:
        cnt = min(sizes[min(len(eb), len(sizes) - 1)], n - off)
        eb.append((off, cnt))
        off += cnt
    e2e_frame = frame_fn(v0, v0, None, hiz[0], eb)
    copy_stream = torch.cuda.Stream()
    first_up, resolved = torch.cuda.Event(), torch.cuda.Event()
    lanes = [(rast, stream, None)]
    for _ in range(args.e2e_lanes - 1):
        r2 = api.Rasterizer()
        r2.EnableBinning = False
        lanes.append((r2, torch.cuda.Stream(), torch.cuda.Event()))
    uploaded = [None] + [torch.cuda.Event() for _ in eb[1:]]
    headline()
    expected = fb.get_pixels(0)  # the image the overlapped upload must reproduce
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        off0, cnt0 = eb[0]
        api._check(api._lib.swr_scene_upload_meshlets(scene.h, C.c_void_p(pinned.data_ptr() + off0 * MESHLET_BYTES),
                                                      off0, cnt0))
        first_up.record(stream)
        copy_stream.wait_event(first_up)
        api.set_stream(copy_stream.cuda_stream)
        for (off, cnt), ev in zip(eb[1:], uploaded[1:]):
            api._check(api._lib.swr_scene_upload_meshlets(scene.h, C.c_void_p(pinned.data_ptr() + off * MESHLET_BYTES),
                                                          off, cnt))
            ev.record(copy_stream)
        api.set_stream(stream.cuda_stream)
        e2e_frame(uploaded, resolved, lanes)
        copy_stream.wait_event(resolved)
        api.set_stream(copy_stream.cuda_stream)
        api._check(api._lib.swr_framebuffer_get_pixels(fb.h, 0, C.c_void_p(host_img.data_ptr()), W))
        api.set_stream(stream.cuda_stream)
        stream.synchronize()  # the Hi-Z build
        if i >= args.warmup:
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
    if not np.array_equal(host_img.numpy().view(np.uint32).reshape(-1), np.asarray(expected).view(np.uint32).reshape(-1)):
        raise RuntimeError("end-to-end frame differs from the device-resident frame")

    del pinned, host_img
    alpha = None
    if not args.no_alpha:
        alpha = alpha_section(args, api, stream, sc, texs, env, lights, flush)
    cone = None
    if not args.no_cone:
        cone = cone_section(args, api, stream, texs, env, lights, flush)
    neural = None
    if not args.no_neural:
        neural = neural_section(args, api, stream, sc, texs, env, scene, rast, lights)
    multiview = None
    if not args.no_multiview:
        multiview = multiview_section(args, api, stream)
    combined = None
    if not args.no_combined:
        combined = combined_section(args, api, stream)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_baseline_entry(cpu_baselines(sc, [t.get_data() for t in texs], env.get_data(), args.steps, 1,
                                               unbinned_seconds=args.cpu_seconds))

    if rank == 0:
        line = {"metric": METRIC, "value": ms, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32+i32", "data": "synthetic (seeded)",
                "config": config_dict(args, sc, {"parallelism": PARALLELISM}),
                "gtri_per_s": int(counters[0]) / (ms / 1e3) / 1e9,
                "gpix_per_s": W * H / (ms / 1e3) / 1e9,
                "counters": {"triangles_processed": int(counters[0]), "triangles_rasterized": int(counters[1]),
                             "triangles_clipped": int(counters[2])},
                "draw_calls": len(batches),
                "frame_driver_batches": {"meshlets_per_draw": BATCH, "draw_calls": len(ref_batches),
                                         "ms": ref_batch_ms},
                "hiz_frame": {"ms": hiz_ms, "note": "next frame culled against this frame's Hi-Z (Main.cpp:229-232)",
                              "triangles_processed": int(hiz_counters[0]),
                              "triangles_rasterized": int(hiz_counters[1]),
                              "kernels_ms_per_step": dict(sorted(hiz_per.items()))},
                "kernels_ms_per_step": {k: s / args.steps for k, (c, s) in sorted(per.items())},
                "kernels_pass_ms_per_step": prof_ms,
                "roofline": roofline,
                "e2e": {"value": float(np.median(e2e_ms)), "unit": UNIT, "h2d_bytes_per_step": int(sc.meshlets.nbytes),
                        "d2h_bytes_per_step": int(W * H * 4), "draw_batches_meshlets": [c for _, c in eb],
                        "lanes": args.e2e_lanes},
                "gpu_launches": int(launches), "clocks": clocks.summary(), "cpu_baseline": cpu,
                "alpha": alpha, "cone": cone, "multiview": multiview, "neural": neural, "combined": combined}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
