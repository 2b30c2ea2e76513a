#!/usr/bin/env python3
"""Benchmark of the GB300 meshlet raster pipeline on the reference's large plain-path scene.

Workload (the headline configuration): 100k meshlets of 64 vertices / 124 triangles (12.4M
triangles), seeded, scattered in a 200^3 volume with log-uniform scale 0.1-10, 64 materials,
rendered at 1920x1080 by one camera, unbinned rasterizer semantics (clipping on), as the
reference's frame driver does (Main.cpp:97-305): clear, meshlet culling, draw in 65536-meshlet
batches, and the stages of the frame that are available in this build.

One "step" = one frame. Timed on the device with CUDA events on the library's stream (set to
torch's current stream); L2 is flushed between timed steps by a 256 MiB write outside the step's
events. `e2e` measures the same frame through the public API with the scene uploaded from pinned
host memory and the id layer read back to host memory inside the timed region.

`--impl reference` times the reference's CPU algorithm (the oracle restatement; the reference
itself cannot be compiled here) on the host cores for the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "1080p frame time (100k meshlets, 12.4M triangles)"
UNIT = "ms/frame"
BATCH = 65536  # Main.cpp:222


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--meshlets", type=int, default=100_000)
    p.add_argument("--width", type=int, default=1920)
    p.add_argument("--height", type=int, default=1080)
    p.add_argument("--cpu-seconds", type=float, default=12.0, help="budget of the CPU baseline sample")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def build_scene(args):
    from glimpsw_gb300 import scenes
    return scenes.volume_scene(n=args.meshlets, width=args.width, height=args.height, texture_size=2048)


def config_dict(args, sc, extra=None):
    d = {"workload": f"volume scene: {args.meshlets} meshlets x 124 tris @ {args.width}x{args.height}, "
                     f"unbinned (clipping on), 1 view",
         "meshlets": args.meshlets, "triangles": int(args.meshlets * 124), "width": args.width,
         "height": args.height, "materials": int(len(sc.materials)),
         "l2": "flushed between timed steps (256 MiB write outside the step events)"}
    if extra:
        d.update(extra)
    return d


# ----------------------------------------------------------------------------- CPU baseline
def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def time_cpu_frames(sc, budget_s, threads):
    """Oracle frames (draw of all meshlets, unbinned semantics) until the budget is used."""
    from oracle import oracle as O
    v = sc.views[0]
    fb = O.Framebuffer(v.width, v.height)
    ctx = O.Context(sc.meshlets, sc.materials, v.world_to_clip)
    times = []
    t_end = time.perf_counter() + budget_s
    while True:
        t0 = time.perf_counter()
        fb.clear(0xFF000000, 0.0)
        for off in range(0, len(sc.meshlets), BATCH):
            n = min(BATCH, len(sc.meshlets) - off)
            ctx2 = O.Context(sc.meshlets, sc.materials, v.world_to_clip, meshlet_offset=off)
            O.draw_meshlets(fb, ctx2, n, binning=False, threads=threads)
        times.append(time.perf_counter() - t0)
        if time.perf_counter() > t_end or len(times) >= 50:
            break
    _ = ctx
    return times


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    sc = build_scene(args)
    threads = cpu_threads()
    times = []
    for _ in range(max(1, args.warmup and 1)):
        time_cpu_frames(sc, 0.0, threads)  # one warm-up frame
    for _ in range(args.steps):
        times += time_cpu_frames(sc, 0.0, threads)
        if sum(times) > 120:
            break
    ms = float(np.median(times) * 1e3)
    line = {"impl": "reference", "metric": METRIC, "value": ms, "unit": UNIT, "n_gpus": args.gpus,
            "steps": len(times), "warmup": 1, "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+i32", "data": "synthetic (seeded)",
            "config": config_dict(args, sc),
            "cpu_baseline": {"value": ms, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{len(times)} full frames (median); oracle restatement of the reference's "
                                       f"CPU rasterizer, rows split over {threads} threads"},
            "e2e": {"value": ms, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, index=0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._t = None

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


# ----------------------------------------------------------------------------- GPU
def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def run_ours(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    from glimpsw_gb300 import api
    api.load_library()

    sc = build_scene(args)
    v = sc.views[0]
    stream = torch.cuda.current_stream()
    api.set_stream(stream.cuda_stream)

    scene = api.Scene()
    scene.upload_meshlets(sc.meshlets)
    scene.set_materials(sc.materials)
    rast = api.Rasterizer()
    rast.EnableBinning = False  # the reference frame driver's setting (Main.cpp:76)
    fb = api.Framebuffer(v.width, v.height, 3)
    n = len(sc.meshlets)
    ctxs = [api.ShadingContext(scene, v.world_to_clip, world_to_clip=v.world_to_clip, meshlet_offset=off)
            for off in range(0, n, BATCH)]

    def frame():
        fb.clear(0xFF000000, 0.0)
        for i, off in enumerate(range(0, n, BATCH)):
            rast.draw_meshlets(fb, min(BATCH, n - off), ctxs[i])

    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    for _ in range(max(3, args.warmup)):
        frame()
    torch.cuda.synchronize()
    rast.reset_counters()
    frame()
    counters = rast.counters()
    rast.reset_counters()

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches0 = api.launch_count()
    api.profile_enable(True)
    with ClockSampler(local) as clocks:
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            frame()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    api.profile_enable(False)
    prof = api.profile_collect()
    launches = api.launch_count() - launches0
    step_ms = [a.elapsed_time(b) for a, b in ev]
    ms = float(np.mean(step_ms))
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())

    # per-kernel device time over the timed region
    per = {}
    for name, t in prof:
        c, s = per.get(name, (0, 0.0))
        per[name] = (c + 1, s + t)
    top = max(per.items(), key=lambda kv: kv[1][1])
    top_name, (top_count, top_total) = top
    top_avg_ms = top_total / top_count

    # algorithmic bytes of the draw kernel: positions + indices of every drawn meshlet (1152 B),
    # the 12-byte meshlet header, and one read+write of the 8-byte vis-buffer key per pixel
    batches = len(ctxs)
    draw_bytes = (n * (1152 + 16)) / batches + v.width * v.height * 16 / batches
    peak, peak_kind = peaks()
    achieved = draw_bytes / (per["k_draw_meshlets"][1] / per["k_draw_meshlets"][0] / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": "k_draw_meshlets", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind, "traffic": None,
                "algorithmic_bytes_per_launch": draw_bytes}

    # end to end through the public API: pinned host scene upload + frame + id layer readback
    pinned = torch.empty(sc.meshlets.nbytes, dtype=torch.uint8).pin_memory()
    pinned.numpy()[:] = sc.meshlets.view(np.uint8).reshape(-1)
    host_ids = torch.empty((v.height, v.width), dtype=torch.int32).pin_memory()
    import ctypes as C
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        api._check(api._lib.swr_scene_upload_meshlets(scene.h, C.c_void_p(pinned.data_ptr()), 0, n))
        frame()
        api._check(api._lib.swr_framebuffer_get_pixels(fb.h, 0, C.c_void_p(host_ids.data_ptr()), v.width))
        dt = (time.perf_counter() - t0) * 1e3
        if i >= args.warmup:
            e2e_ms.append(dt)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = cpu_threads()
        times = time_cpu_frames(sc, args.cpu_seconds, threads)
        cpu = {"value": float(np.median(times) * 1e3), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{len(times)} full frames of the same workload (median), oracle restatement, "
                         f"rows split over {threads} threads"}

    tris_drawn = int(counters[0])
    if rank == 0:
        line = {"metric": METRIC, "value": ms, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": False, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32+i32", "data": "synthetic (seeded)",
                "config": config_dict(args, sc, {"parallelism": "replicas only (one GPU renders the frame)"}),
                "gtri_per_s": tris_drawn / (ms / 1e3) / 1e9,
                "gpix_per_s": v.width * v.height / (ms / 1e3) / 1e9,
                "counters": {"triangles_processed": int(counters[0]), "triangles_rasterized": int(counters[1]),
                             "triangles_clipped": int(counters[2])},
                "kernels_ms_per_step": {k: s / args.steps for k, (c, s) in sorted(per.items())},
                "roofline": roofline,
                "e2e": {"value": float(np.median(e2e_ms)), "unit": UNIT, "h2d_bytes_per_step": int(sc.meshlets.nbytes),
                        "d2h_bytes_per_step": int(v.width * v.height * 4)},
                "gpu_launches": int(launches), "clocks": clocks.summary(), "cpu_baseline": cpu}
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
