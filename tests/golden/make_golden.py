"""Generates the golden fixtures of tests/golden/ from the CPU oracle (run from the repository root:
`python tests/golden/make_golden.py [fixture names]`).

The reference ships no golden vectors for this path and cannot be built here, so these fixtures
are frozen outputs of the oracle on small seeded scenes. They pin the oracle against drift
(CPU tests) and give the GPU tests a fixed target. Each fixture stores a hash of the scene it was
rendered from, so a change of the scene generators is reported as such instead of as a mismatch.

Fixtures (all at 160x96 unless noted):
  raster_grid.npz     C1 construction (32x32 patch grid), vis-buffer (depth + surface ids), binned
                      and unbinned semantics
  raster_inside.npz   camera inside a dense volume (near-plane clipping, guard band): unbinned with
                      clipping, unbinned without guard band, binned
  resolve_volume.npz  volume scene with 4 materials of 32^2 textures, one light and a sky: resolved
                      RGBA8, the Hi-Z pyramid of the frame, and the cull bitmap of the next camera
  neural_fwd_bwd.npz  learned decoder: forward outputs and parameter / input gradients for fixed
                      parameters, inputs and targets (oracle/neural.py)
  alpha_debug.npz     camera inside a volume whose every second material is alpha-tested: the
                      vis-buffer, the OverdrawShader's counters and depth, and the ResolveDebug
                      layers base colour, meshlet id and overdraw-quad
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from glimpsw_gb300 import scenes  # noqa: E402

W, H = 160, 96


def scene_hash(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).view(np.uint8).tobytes())
    return h.hexdigest()


def grid_scene():
    return scenes.grid_scene(n_side=32, width=W, height=H)


def inside_scene():
    sc = scenes.volume_scene(n=3000, width=W, height=H, n_materials=4, extent=12.0, texture_size=32, env_size=32)
    mats = sc.materials.copy()
    mats["is_double_sided"][::2] = 1
    view = scenes.make_view(W, H, eye=(0.0, 0.0, 0.0), target=(0.3, 0.1, 1.0))
    return sc, mats, view


def resolve_scene():
    return scenes.volume_scene(n=4000, width=W, height=H, n_materials=4, extent=30.0, texture_size=32, env_size=32)


def default_lights():
    from tests.helpers import default_lights as dl
    return dl()


def make_raster_grid(O):
    from tests.helpers import render_oracle
    sc = grid_scene()
    v = sc.views[0]
    out = {"scene_hash": scene_hash(sc.meshlets, sc.materials, v.world_to_clip)}
    for name, binning in (("binned", True), ("unbinned", False)):
        fb, counters = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, W, H, binning=binning)
        out[f"{name}_ids"], out[f"{name}_depth"] = fb.get_pixels(0), fb.get_pixels(1)
        out[f"{name}_counters"] = np.asarray(counters[:3], np.uint64)
    return out


def make_raster_inside(O):
    from tests.helpers import render_oracle
    sc, mats, view = inside_scene()
    out = {"scene_hash": scene_hash(sc.meshlets, mats, view.world_to_clip)}
    for name, (binning, clipping, guardband) in (("clip", (False, True, True)), ("noguard", (False, True, False)),
                                                 ("binned", (True, True, True))):
        fb, counters = render_oracle(sc.meshlets, mats, view.world_to_clip, W, H, binning=binning, clipping=clipping,
                                     guardband=guardband)
        out[f"{name}_ids"], out[f"{name}_depth"] = fb.get_pixels(0), fb.get_pixels(1)
        out[f"{name}_counters"] = np.asarray(counters[:3], np.uint64)
    return out


def make_resolve_volume(O):
    from tests.helpers import TexturePair, render_oracle
    sc = resolve_scene()
    v0, v1 = sc.views
    texs = [TexturePair([sc.texture_pixels(i, 0), sc.texture_pixels(i, 1)], sc.texture_size, gpu=False) for i in range(4)]
    env = TexturePair([scenes.env_map_r11g11b10(32, 5)], 32, fmt=1, gpu=False)
    fb, _ = render_oracle(sc.meshlets, sc.materials, v0.world_to_clip, W, H)
    hw, hh = O.hiz_texture_size(W, H)
    hiz = O.Texture(hw, hh, 16, 1, fmt=2)
    hiz.data[:] = 0x7F7FFFFE
    O.downsample_depth(fb, hiz)
    bm, visible = O.cull_meshlets(sc.meshlets, len(sc.meshlets), v1.proj, v1.view, scenes.IDENTITY, v0.view, W, H, hiz)
    ctx = O.Context(sc.meshlets, sc.materials, v0.world_to_clip, world_to_clip=v0.world_to_clip,
                    textures=[t.o for t in texs], lights=default_lights(), skybox=env.o, view_pos=v0.eye)
    O.resolve(fb, ctx)
    return {"scene_hash": scene_hash(sc.meshlets, sc.materials, v0.world_to_clip, v1.world_to_clip,
                                     *[t.o.data for t in texs], env.o.data),
            "color": fb.get_pixels(0), "hiz": hiz.data.copy(), "cull_bitmap": bm, "cull_visible": np.uint32(visible)}


def alpha_scene():
    sc = scenes.volume_scene(n=3000, width=W, height=H, n_materials=4, extent=12.0, texture_size=32, env_size=32,
                             alpha_every=2)
    view = scenes.make_view(W, H, eye=(0.0, 0.0, 0.0), target=(0.3, 0.1, 1.0))
    return sc, view


def make_alpha_debug(O):
    from tests.helpers import TexturePair, render_oracle
    sc, view = alpha_scene()
    texs = [TexturePair([sc.texture_pixels(i, 0), sc.texture_pixels(i, 1)], sc.texture_size, gpu=False) for i in range(4)]
    tex = [t.o for t in texs]
    out = {"scene_hash": scene_hash(sc.meshlets, sc.materials, view.world_to_clip, *[t.data for t in tex])}
    fb, counters = render_oracle(sc.meshlets, sc.materials, view.world_to_clip, W, H, textures=tex)
    out["alpha_ids"], out["alpha_depth"] = fb.get_pixels(0), fb.get_pixels(1)
    out["alpha_counters"] = np.asarray(counters[:3], np.uint64)
    ctx = O.Context(sc.meshlets, sc.materials, view.world_to_clip, textures=tex)
    for layer in (1, 4):
        fb, _ = render_oracle(sc.meshlets, sc.materials, view.world_to_clip, W, H, textures=tex)
        O.resolve_debug(fb, ctx, layer)
        out[f"debug{layer}"] = fb.get_pixels(0)
    fb, _ = render_oracle(sc.meshlets, sc.materials, view.world_to_clip, W, H, textures=tex, clear=(0, 0.0),
                          shader=O.SHADER_OVERDRAW)
    out["overdraw_counts"], out["overdraw_depth"] = fb.get_pixels(0), fb.get_pixels(1)
    O.resolve_debug(fb, ctx, 7)
    out["debug7"] = fb.get_pixels(0)
    return out


def neural_case():
    """Fixed parameters, inputs, levels and targets of the decoder check."""
    rng = np.random.default_rng(2024)
    from oracle import neural as N
    p = np.zeros(N.PARAMS, np.float32)
    w1 = rng.normal(0, 0.4, (64, 16)).astype(np.float32)
    w1[:, 11:] = 0
    p[N.PW1:N.PW2] = w1.reshape(-1)
    p[N.PW2:N.PB2] = rng.normal(0, 0.2, 4096)
    p[N.PB2:N.PW3] = rng.normal(0, 0.1, 64)
    p[N.PW3:N.PB3] = rng.normal(0, 0.2, 512)
    p[N.PB3:] = rng.normal(0.5, 0.1, 8)
    x0 = rng.normal(0, 0.7, (256, 8)).astype(np.float32)
    lvl = rng.integers(0, 6, 256)
    t = rng.uniform(0, 1, (256, 8)).astype(np.float32)
    return p, x0, lvl, t


def make_neural(O):
    from oracle import neural as N
    p, x0, lvl, t = neural_case()
    cache = N.forward(p, x0, lvl)
    g, dx0, loss = N.backward(p, cache, t)
    return {"y": cache["y"], "param_grad": g, "dx0": dx0, "loss": np.float64(loss)}


MAKERS = {"raster_grid": make_raster_grid, "raster_inside": make_raster_inside, "resolve_volume": make_resolve_volume,
          "neural_fwd_bwd": make_neural, "alpha_debug": make_alpha_debug}


def main():
    from oracle import oracle as O
    O.lib()
    O.set_approx_mode(0)  # the portable rcp14/rsqrt14 model, as on the GPU
    names = sys.argv[1:] or list(MAKERS)  # regenerate the named fixtures (default: all)
    for name in names:
        out = MAKERS[name](O)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, {k: (v.shape if hasattr(v, "shape") else v) for k, v in out.items()})


if __name__ == "__main__":
    main()
