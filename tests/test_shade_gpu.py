"""GPU parity of textures, the Hi-Z pyramid, meshlet culling and the vis-buffer resolve against
the CPU oracle (both sides run rcp14/rsqrt14 through the exact tables of include/swr/approx14.h).

Mips, Hi-Z texels and cull bitmaps must be bit-exact; the resolved RGBA8 colour must be within
1/255 per channel (the contract), and the test also reports how many pixels match exactly.
"""
import numpy as np
import pytest

from glimpsw_gb300 import scenes
from tests.helpers import LIGHT_DTYPE, GpuRenderer, TexturePair, default_lights, gpu_lights, make_light, render_oracle

pytestmark = pytest.mark.gpu


def test_texture_mips_bit_exact():
    from glimpsw_gb300 import api
    api.load_library()
    rgba = [scenes.value_noise_rgba(256, 7, layer=0), scenes.value_noise_rgba(256, 7, layer=1)]
    t = TexturePair(rgba, 256, fmt=0)
    assert np.array_equal(t.g.get_data()[: t.o.data.size], t.o.data)
    env = TexturePair([scenes.env_map_r11g11b10(128, 3)], 128, fmt=1)
    assert np.array_equal(env.g.get_data()[: env.o.data.size], env.o.data)


@pytest.fixture(scope="module")
def shaded():
    from glimpsw_gb300 import api
    api.load_library()
    sc = scenes.volume_scene(n=6000, width=640, height=360, n_materials=4, extent=40.0, texture_size=256, env_size=128)
    texs = [TexturePair([sc.texture_pixels(i, 0), sc.texture_pixels(i, 1)], 256) for i in range(4)]
    env = TexturePair([scenes.env_map_r11g11b10(128, 5)], 128, fmt=1)
    g = GpuRenderer(sc.meshlets, sc.materials, [t.g for t in texs])
    return sc, texs, env, g


def _hiz_textures(w, h):
    from oracle import oracle as O
    from glimpsw_gb300 import api
    hw, hh = O.hiz_texture_size(w, h)
    o = O.Texture(hw, hh, 16, 1, fmt=2)
    g = api.Texture2D(api.FORMAT_R32F, hw, hh, 16, 1)
    o.data[:] = 0x7F7FFFFE  # same sentinel on both sides: texels the reference never writes keep it
    g.set_data(o.data)
    return o, g


@pytest.mark.parametrize("size", [(640, 360), (1280, 720), (64, 48)])
def test_hiz_bit_exact(shaded, size):
    from glimpsw_gb300 import api
    from oracle import oracle as O
    sc, _, _, g = shaded
    w, h = size
    v = scenes.make_view(w, h, eye=sc.views[0].eye, target=(0.0, 0.0, 0.0))
    gfb, _ = g.render(v.world_to_clip, w, h)
    ofb, _ = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, w, h)
    ot, gt = _hiz_textures(w, h)
    O.downsample_depth(ofb, ot)
    api.downsample_depth(gfb, gt)
    got = gt.get_data()[: ot.data.size]
    assert np.array_equal(got, ot.data), f"{(got != ot.data).sum()} texels differ"
    assert (ot.data != 0x7F7FFFFE).sum() > 0


@pytest.mark.parametrize("use_hiz", [False, True])
def test_cull_bit_exact(shaded, use_hiz):
    import torch
    from glimpsw_gb300 import api
    from oracle import oracle as O
    sc, _, _, g = shaded
    v0, v1 = sc.views
    w, h = v0.width, v0.height
    n = len(sc.meshlets)
    ot = gt = None
    if use_hiz:
        gfb, _ = g.render(v0.world_to_clip, w, h)
        ofb, _ = render_oracle(sc.meshlets, sc.materials, v0.world_to_clip, w, h)
        ot, gt = _hiz_textures(w, h)
        O.downsample_depth(ofb, ot)
        api.downsample_depth(gfb, gt)
    model = scenes.IDENTITY
    obm, ocount = O.cull_meshlets(sc.meshlets, n, v1.proj, v1.view, model, v0.view, w, h, ot)
    dbm = torch.zeros((n + 15) // 16, dtype=torch.int16, device="cuda")
    gcount = api.cull_meshlets(g.scene, 0, n, dbm, v1.proj, v1.view, model, v0.view, w, h, gt, want_count=True)
    gbm = dbm.cpu().numpy().view(np.uint16)
    assert np.array_equal(gbm, obm), f"{np.unpackbits((gbm ^ obm).view(np.uint8)).sum()} meshlets differ"
    assert gcount == ocount
    assert 0 < ocount < n


def test_resolve_within_one_lsb(shaded):
    from glimpsw_gb300 import api
    from oracle import oracle as O
    sc, texs, env, g = shaded
    v = sc.views[0]
    w, h = v.width, v.height
    lights = default_lights()
    gfb, _ = g.render(v.world_to_clip, w, h)
    ofb, _ = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, w, h)
    octx = O.Context(sc.meshlets, sc.materials, v.world_to_clip, world_to_clip=v.world_to_clip,
                     textures=[t.o for t in texs], lights=lights, skybox=env.o, view_pos=v.eye)
    O.resolve(ofb, octx)
    gctx = api.ShadingContext(g.scene, v.world_to_clip, world_to_clip=v.world_to_clip, skybox=env.g, view_pos=v.eye,
                              lights=gpu_lights(lights))
    gctx.resolve(g.rast, gfb)
    a = gfb.get_pixels(0).view(np.uint8).reshape(h, w, 4).astype(np.int32)
    b = ofb.get_pixels(0).view(np.uint8).reshape(h, w, 4).astype(np.int32)
    diff = np.abs(a - b)
    exact = (diff.max(axis=2) == 0).mean()
    print(f"resolve: max abs {diff.max()} / 255, exact pixels {exact:.6f}")
    assert diff.max() <= 1
    assert exact > 0.999


def test_resolve_point_and_spot_lights_within_one_lsb(shaded):
    """EvalLighting's loop over several lights with GetLightAttenuation's three branches
    (Shading.cpp:581-645): one directional, two point and two spot lights with their own colours,
    ranges and cone angles. Each light alone visibly changes the oracle's image (so every branch is
    exercised), and the GPU resolve with all five is within 1/255 of the oracle's."""
    from glimpsw_gb300 import api
    from oracle import oracle as O
    sc, texs, env, g = shaded
    v = sc.views[0]
    w, h = v.width, v.height
    lights = np.concatenate([
        make_light(0, direction=(0.3, -0.8, 0.5), color=(1.0, 0.85, 0.6), intensity=900.0),
        make_light(1, position=(-8.0, 6.0, -30.0), color=(1.0, 0.45, 0.25), intensity=3.0e5, radius=45.0),
        make_light(1, position=(12.0, -4.0, -18.0), color=(0.3, 0.6, 1.0), intensity=1.5e5, radius=30.0),
        make_light(2, position=(0.0, 20.0, -50.0), direction=(0.0, -20.0, 20.0), color=(0.8, 1.0, 0.7),
                   intensity=4.0e5, radius=100.0, inner=0.2, outer=0.6),
        make_light(2, position=(5.0, -10.0, -50.0), direction=(-5.0, 10.0, 20.0), color=(1.0, 0.7, 0.9),
                   intensity=4.0e5, radius=100.0, inner=0.25, outer=0.5),
    ])

    def oracle_image(ls):
        ofb, _ = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, w, h)
        octx = O.Context(sc.meshlets, sc.materials, v.world_to_clip, world_to_clip=v.world_to_clip,
                         textures=[t.o for t in texs], lights=ls, skybox=env.o, view_pos=v.eye)
        O.resolve(ofb, octx, threads=8)
        return ofb.get_pixels(0).view(np.uint8).reshape(h, w, 4).astype(np.int32)

    ambient = oracle_image(np.zeros(0, dtype=LIGHT_DTYPE))
    for i in range(len(lights)):
        changed = (np.abs(oracle_image(lights[i:i + 1]) - ambient).max(axis=2) > 2).sum()
        assert changed > 1000, f"light {i} changes only {changed} pixels"
    ref = oracle_image(lights)
    gfb, _ = g.render(v.world_to_clip, w, h)
    gctx = api.ShadingContext(g.scene, v.world_to_clip, world_to_clip=v.world_to_clip, skybox=env.g, view_pos=v.eye,
                              lights=gpu_lights(lights))
    gctx.resolve(g.rast, gfb)
    got = gfb.get_pixels(0).view(np.uint8).reshape(h, w, 4).astype(np.int32)
    diff = np.abs(got - ref)
    exact = (diff.max(axis=2) == 0).mean()
    print(f"resolve, 5 lights: max abs {diff.max()} / 255, exact pixels {exact:.6f}")
    assert diff.max() <= 1
    assert exact > 0.999


def test_resolve_follows_rcp14_tables(shaded):
    """On the pixels where the reference's rcp14/rsqrt14 give a different colour than correctly
    rounded IEEE reciprocals would, the GPU gives the reference's colour exactly: the device runs
    the instructions' tables, not an IEEE stand-in."""
    from glimpsw_gb300 import api
    from oracle import oracle as O
    sc, texs, env, g = shaded
    v = sc.views[0]
    w, h = v.width, v.height
    lights = default_lights()
    gfb, _ = g.render(v.world_to_clip, w, h)
    gctx = api.ShadingContext(g.scene, v.world_to_clip, world_to_clip=v.world_to_clip, skybox=env.g, view_pos=v.eye,
                              lights=gpu_lights(lights))
    gctx.resolve(g.rast, gfb)
    got = gfb.get_pixels(0).view(np.uint8).reshape(h, w, 4).astype(np.int32)
    out = {}
    for mode in (0, 2):
        ofb, _ = render_oracle(sc.meshlets, sc.materials, v.world_to_clip, w, h)
        octx = O.Context(sc.meshlets, sc.materials, v.world_to_clip, world_to_clip=v.world_to_clip,
                         textures=[t.o for t in texs], lights=lights, skybox=env.o, view_pos=v.eye)
        assert O.set_approx_mode(mode)
        try:
            O.resolve(ofb, octx)
        finally:
            O.set_approx_mode(0)
        out[mode] = ofb.get_pixels(0).view(np.uint8).reshape(h, w, 4).astype(np.int32)
    sensitive = (out[0] != out[2]).any(axis=2)
    print(f"pixels whose colour depends on rcp14/rsqrt14: {int(sensitive.sum())}")
    assert sensitive.sum() > 0
    assert np.array_equal(got[sensitive], out[0][sensitive])

