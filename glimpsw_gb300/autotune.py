"""Autotuner for batched multi-view rendering: picks the chunk (bin) size, the chunk shape and the
warps per mesh-stage block by timing the batch itself, and caches the choice per (GPU, workload
class).

Candidates, in two stages: square chunks of 2/4/8/16 tiles (8/16/32/64-pixel bins) x 4/8/16 warps
per block, then, for the best of those, the rectangular chunks of half and twice its width or
height (2 to 16 tiles a side). Each candidate re-captures the batch's CUDA graph and is timed with
CUDA events on the batch's stream (median of `repeats` renders after one warm-up). The image never
depends on the choice. A choice is (chunk width, warps per block, chunk height) in tiles.
"""
from __future__ import annotations

import json
import math
import os

CANDIDATES = [(c, w) for c in (2, 4, 8, 16) for w in (4, 8, 16)]


def cache_path() -> str:
    p = os.environ.get("SWR_AUTOTUNE_CACHE")
    if p:
        return p
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "glimpsw_gb300", "autotune.json")


def workload_key(gpu_name: str, views, meshlets: int) -> str:
    """GPU name, number of views, total pixels and meshlets, both rounded to a power of two."""
    pixels = sum(fb.width * fb.height for fb, *_ in views)
    return f"{gpu_name}|views={len(views)}|px=2^{round(math.log2(max(pixels, 1)))}|meshlets=2^{round(math.log2(max(meshlets, 1)))}"


def _load(path):
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


def shape_candidates(c: int) -> list[tuple[int, int]]:
    """Rectangular chunks next to the square chunk of c tiles: half or twice one side."""
    out = []
    for w, h in ((c // 2, c), (c * 2, c), (c, c // 2), (c, c * 2)):
        if 2 <= w <= 16 and 2 <= h <= 16:
            out.append((w, h))
    return out


def apply(batch, choice) -> None:
    c, w, h = choice
    batch.set_tuning(c, w)
    if h != c:
        batch.set_chunk_shape(c, h)


def tune(batch, key: str | None = None, repeats: int = 3, use_cache: bool = True):
    """Returns ((chunk_w, warps_per_block, chunk_h), {candidate: ms}) and applies the best choice."""
    import torch

    path = cache_path()
    cache = _load(path) if use_cache else {}
    if key and key in cache and len(cache[key]["choice"]) == 3:
        choice = tuple(cache[key]["choice"])
        apply(batch, choice)
        return choice, {tuple(map(int, k.split("x"))): v for k, v in cache[key]["ms"].items()}
    stream = torch.cuda.current_stream()

    def time_choice(choice):
        apply(batch, choice)
        batch.render()  # captures the graph for this choice, warms caches
        torch.cuda.synchronize()
        ms = []
        for _ in range(repeats):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            batch.render()
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return sorted(ms)[len(ms) // 2]

    timings = {(c, w, c): time_choice((c, w, c)) for c, w in CANDIDATES}
    c0, w0, _ = min(timings, key=timings.get)
    for cw, ch in shape_candidates(c0):
        timings[(cw, w0, ch)] = time_choice((cw, w0, ch))
    best = min(timings, key=timings.get)
    apply(batch, best)
    if key:
        cache[key] = {"choice": list(best), "ms": {f"{c}x{w}x{h}": v for (c, w, h), v in timings.items()}}
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            with open(path, "w") as f:
                json.dump(cache, f, indent=1, sort_keys=True)
        except OSError:
            pass
    return best, timings
