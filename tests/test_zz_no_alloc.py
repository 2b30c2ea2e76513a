"""swr_draw_meshlets_noalloc, the draw for callers that cannot allocate device memory, must give
the same vis-buffer as swr_draw_meshlets on the same inputs, call after call.

Such callers hand over device pointers they own and cannot let the library call cudaMalloc; the
test plays that caller: it allocates the inputs and outputs itself (with torch) and calls the
entry point through the C ABI. The comparison is exact, the tolerance of every vis-buffer test.
Cases: the grid scene, and a camera inside a volume scene (triangles across the near plane and the
guard band) under every combination of the rasterizer flags, with and without a cull bitmap;
alpha-tested materials, which this entry point draws as opaque. This file sorts last so that a run
stopping at the first failure has run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from glimpsw_gb300 import scenes

pytestmark = pytest.mark.gpu


def detile(layer: np.ndarray, width: int, height: int) -> np.ndarray:
    """Row-major copy of a 4x4-tiled layer (the reference's Framebuffer::GetPixelOffset)."""
    y, x = np.mgrid[0:height, 0:width]
    off = ((x & ~3) << 2) + (y & ~3) * width + (x & 3) + (y & 3) * 4
    return layer[off]


def regular_draw(meshlets, mats, world_to_clip, W, H, binning, clipping, guardband, bitmap=None):
    """swr_draw_meshlets into a fresh cleared framebuffer: (surface ids, depth, counters)."""
    from glimpsw_gb300 import api

    scene = api.Scene()
    scene.upload_meshlets(meshlets)
    scene.set_materials(mats)
    rast = api.Rasterizer()
    rast.EnableBinning, rast.EnableClipping, rast.EnableGuardband = binning, clipping, guardband
    fb = api.Framebuffer(W, H)
    fb.clear(0xFF000000, 0.0)
    rast.reset_counters()
    rast.draw_meshlets(fb, len(meshlets), api.ShadingContext(scene, world_to_clip, cull_bitmap=bitmap))
    return fb.get_pixels(0), fb.get_pixels(1)


def noalloc_draws(meshlets, flags, world_to_clip, W, H, binning, clipping, guardband, bitmap=None, calls=2):
    """The allocation-free draw on caller-owned device memory, `calls` times in a row into freshly
    cleared layers; yields (surface ids, depth) per call."""
    import torch

    from glimpsw_gb300 import api

    lib = api.load_library()
    d_meshlets = torch.from_numpy(meshlets.view(np.uint8).copy()).cuda()
    d_flags = torch.from_numpy(flags.astype(np.uint8)).cuda()
    ids = torch.empty(W * H, dtype=torch.int32, device="cuda")
    depth = torch.empty(W * H, dtype=torch.float32, device="cuda")
    m = (C.c_float * 16)(*np.asarray(world_to_clip, dtype=np.float32).tolist())
    bm = bitmap.data_ptr() if bitmap is not None else None
    api.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        for _ in range(calls):
            ids.fill_(-16777216)  # 0xFF000000 as int32: Framebuffer::Clear(0xFF000000, 0.0)
            depth.zero_()
            st = lib.swr_draw_meshlets_noalloc(d_meshlets.data_ptr(), 0, len(meshlets), d_flags.data_ptr(), len(flags),
                                               bm, m, ids.data_ptr(), depth.data_ptr(), W, H, int(binning),
                                               int(clipping), int(guardband))
            assert st == api.SWR_OK, lib.swr_last_error().decode()
            torch.cuda.synchronize()
            yield (detile(ids.cpu().numpy().view(np.uint32), W, H), detile(depth.cpu().numpy().view(np.uint32), W, H))
    finally:
        api.set_stream(None)


def assert_calls_match(ref, calls):
    ref_ids, ref_depth = ref
    assert np.any(ref_depth)
    for call, (ids, depth) in enumerate(calls):
        assert np.array_equal(ids, ref_ids), f"call {call}: surface ids differ"
        assert np.array_equal(depth, ref_depth), f"call {call}: depth differs"


def test_noalloc_draw_matches_regular_draw_on_consecutive_calls():
    sc = scenes.grid_scene(n_side=32, width=640, height=360)
    v = sc.views[0]
    mats = sc.materials.copy()
    mats["is_double_sided"][0] = 0
    ref = regular_draw(sc.meshlets, mats, v.world_to_clip, v.width, v.height, False, True, True)
    assert_calls_match(ref, noalloc_draws(sc.meshlets, mats["is_double_sided"], v.world_to_clip, v.width, v.height,
                                          False, True, True))


@pytest.fixture(scope="module")
def inside():
    """A camera inside a volume of meshlets: triangles cross the near plane and the guard band."""
    sc = scenes.volume_scene(n=3000, width=480, height=272, n_materials=4, extent=12.0, texture_size=8)
    mats = sc.materials.copy()
    mats["is_double_sided"][::2] = 1
    view = scenes.make_view(480, 272, eye=np.zeros(3), target=(0.3, 0.1, 1.0))
    return sc.meshlets, mats, view


@pytest.mark.parametrize("binning,clipping,guardband", [(True, True, True), (True, False, False), (False, True, True),
                                                        (False, False, True), (False, True, False),
                                                        (False, False, False)])
@pytest.mark.parametrize("with_bitmap", [False, True])
def test_noalloc_flags_and_cull_bitmap(inside, binning, clipping, guardband, with_bitmap):
    import torch

    meshlets, mats, view = inside
    bitmap = None
    if with_bitmap:
        bm = np.random.default_rng(5).integers(0, 1 << 16, (len(meshlets) + 15) // 16).astype(np.uint16)
        bitmap = torch.from_numpy(bm.view(np.int16)).cuda()
    ref = regular_draw(meshlets, mats, view.world_to_clip, 480, 272, binning, clipping, guardband, bitmap)
    assert_calls_match(ref, noalloc_draws(meshlets, mats["is_double_sided"], view.world_to_clip, 480, 272, binning,
                                          clipping, guardband, bitmap))


def test_noalloc_draws_alpha_tested_materials_as_opaque():
    """The entry point takes no textures: a material that swr_draw_meshlets alpha-tests draws opaque,
    the image swr_draw_meshlets gives for the same materials with alpha_cutoff 255."""
    from glimpsw_gb300 import api

    sc = scenes.grid_scene(n_side=16, width=320, height=180)
    v = sc.views[0]
    meshlets = sc.meshlets.copy()
    meshlets["MaterialId"] = np.arange(len(meshlets)) % 2
    mats = np.zeros(2, dtype=scenes.MATERIAL_DTYPE)
    mats["texture"] = [0, 1]
    mats["alpha_cutoff"] = [255, 128]
    mats["is_double_sided"] = [0, 1]
    opaque = mats.copy()
    opaque["alpha_cutoff"] = 255
    ref = regular_draw(meshlets, opaque, v.world_to_clip, v.width, v.height, False, True, True)
    assert_calls_match(ref, noalloc_draws(meshlets, mats["is_double_sided"], v.world_to_clip, v.width, v.height,
                                          False, True, True, calls=1))

    # and swr_draw_meshlets with the textures does alpha-test them (the images differ)
    px = scenes.value_noise_rgba(64, 4, cells=8, layer=0, cutout=True)
    texs = []
    for _ in range(2):
        t = api.Texture2D(api.FORMAT_RGBA8U, 64, 64, 16, 1)
        t.set_pixels(px, 0)
        t.generate_mips()
        texs.append(t)
    scene = api.Scene()
    scene.upload_meshlets(meshlets)
    scene.set_materials(mats, texs)
    rast = api.Rasterizer()
    rast.EnableBinning = False
    fb = api.Framebuffer(v.width, v.height)
    fb.clear(0xFF000000, 0.0)
    rast.draw_meshlets(fb, len(meshlets), api.ShadingContext(scene, v.world_to_clip))
    assert not np.array_equal(fb.get_pixels(0), ref[0])


def test_noalloc_draw_rejects_sizes_above_its_limit():
    from glimpsw_gb300 import api

    lib = api.load_library()
    m = (C.c_float * 16)(*([0.0] * 16))
    dummy = 1 << 20  # never dereferenced: the size check comes first
    st = lib.swr_draw_meshlets_noalloc(dummy, 0, 1, None, 0, None, m, dummy, dummy, 1920, 1080, 0, 1, 1)
    assert st == api.SWR_ECAPACITY
    assert "1048576" in lib.swr_last_error().decode()
