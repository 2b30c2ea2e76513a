"""swr_draw_meshlets_noalloc, the draw for callers that cannot allocate device memory, must give
the same vis-buffer as swr_draw_meshlets on the same inputs, call after call.

Such callers hand over device pointers they own and cannot let the library call cudaMalloc; the
test plays that caller: it allocates the inputs and outputs itself (with torch) and calls the
entry point through the C ABI. The comparison is exact, the tolerance of every vis-buffer test.
This file sorts last so that a run stopping at the first failure has run every other test.
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


def test_noalloc_draw_matches_regular_draw_on_consecutive_calls():
    import torch

    from glimpsw_gb300 import api

    lib = api.load_library()
    sc = scenes.grid_scene(n_side=32, width=640, height=360)
    v = sc.views[0]
    W, H, n = v.width, v.height, len(sc.meshlets)
    mats = sc.materials.copy()
    mats["is_double_sided"][0] = 0

    # regular entry point
    scene = api.Scene()
    scene.upload_meshlets(sc.meshlets)
    scene.set_materials(mats)
    rast = api.Rasterizer()
    rast.EnableBinning = False
    fb = api.Framebuffer(W, H)
    fb.clear(0xFF000000, 0.0)
    rast.draw_meshlets(fb, n, api.ShadingContext(scene, v.world_to_clip))
    ref_ids, ref_depth = fb.get_pixels(0), fb.get_pixels(1)
    assert np.any(ref_depth)

    # caller-owned device memory for the allocation-free entry point
    meshlets = torch.from_numpy(sc.meshlets.view(np.uint8).copy()).cuda()
    flags = torch.from_numpy(mats["is_double_sided"].astype(np.uint8)).cuda()
    ids = torch.empty(W * H, dtype=torch.int32, device="cuda")
    depth = torch.empty(W * H, dtype=torch.float32, device="cuda")
    m = (C.c_float * 16)(*np.asarray(v.world_to_clip, dtype=np.float32).tolist())
    api.set_stream(torch.cuda.current_stream().cuda_stream)
    try:
        for call in range(2):
            ids.fill_(-16777216)  # 0xFF000000 as int32: Framebuffer::Clear(0xFF000000, 0.0)
            depth.zero_()
            st = lib.swr_draw_meshlets_noalloc(meshlets.data_ptr(), 0, n, flags.data_ptr(), len(mats), None, m,
                                               ids.data_ptr(), depth.data_ptr(), W, H, 0, 1, 1)
            assert st == api.SWR_OK, lib.swr_last_error().decode()
            torch.cuda.synchronize()
            got_ids = detile(ids.cpu().numpy().view(np.uint32), W, H)
            got_depth = detile(depth.cpu().numpy().view(np.uint32), W, H)
            assert np.array_equal(got_ids, ref_ids), f"call {call}: surface ids differ"
            assert np.array_equal(got_depth, ref_depth), f"call {call}: depth differs"
    finally:
        api.set_stream(None)


def test_noalloc_draw_rejects_sizes_above_its_limit():
    from glimpsw_gb300 import api

    lib = api.load_library()
    m = (C.c_float * 16)(*([0.0] * 16))
    dummy = 1 << 20  # never dereferenced: the size check comes first
    st = lib.swr_draw_meshlets_noalloc(dummy, 0, 1, None, 0, None, m, dummy, dummy, 1920, 1080, 0, 1, 1)
    assert st == api.SWR_ECAPACITY
    assert "1048576" in lib.swr_last_error().decode()
