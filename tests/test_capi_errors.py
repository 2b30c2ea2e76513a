"""The C ABI's argument checks, without a GPU: every call below fails validation before it reaches
CUDA, returns its status code (no exception crosses the boundary) and leaves a message for
swr_last_error. The size rules are the reference's: framebuffers are non-zero multiples of 4 up
to MaxRenderSize 2896 (Rasterizer.h:66-78), textures power-of-two sized (Texture.h:599-636)."""
import ctypes as C

import pytest

from glimpsw_gb300 import api

EINVAL = 1


@pytest.fixture(scope="module")
def lib():
    return api.load_library()


def _fails(lib, status, *words):
    assert status == EINVAL
    msg = lib.swr_last_error().decode()
    for w in words:
        assert w in msg, msg


@pytest.mark.parametrize("w,h", [(0, 4), (4, 0), (6, 4), (4, 10), (2900, 4), (4, 2900)])
def test_framebuffer_sizes(lib, w, h):
    out = C.c_void_p()
    _fails(lib, lib.swr_framebuffer_create(w, h, 2, C.byref(out)), "swr_framebuffer_create")
    assert not out.value


@pytest.mark.parametrize("fmt,w,h,levels,layers", [(9, 64, 64, 1, 1), (0, 48, 64, 1, 1), (0, 64, 2, 1, 1),
                                                   (0, 64, 64, 0, 1), (0, 64, 64, 17, 1), (0, 64, 64, 1, 0)])
def test_texture_arguments(lib, fmt, w, h, levels, layers):
    out = C.c_void_p()
    _fails(lib, lib.swr_texture_create(fmt, w, h, levels, layers, C.byref(out)), "swr_texture_create")


def test_null_handles(lib):
    _fails(lib, lib.swr_rasterizer_set_flags(None, 1, 1, 1), "NULL")
    _fails(lib, lib.swr_batch_set_tuning(None, 8, 8), "NULL")
    _fails(lib, lib.swr_batch_set_chunk_shape(None, 8, 8), "NULL")
    _fails(lib, lib.swr_batch_render(None), "NULL")
    _fails(lib, lib.swr_scene_upload_meshlets(None, None, 0, 1), "swr_scene_upload_meshlets")
    _fails(lib, lib.swr_framebuffer_create(64, 64, 2, None), "NULL")


def test_self_test_limit_range(lib):
    _fails(lib, lib.swr_selftest_bounded_wait(0), "1 ns to 1 s")
    _fails(lib, lib.swr_selftest_bounded_wait(2_000_000_000), "1 ns to 1 s")


def test_unknown_shader_table(lib):
    _fails(lib, lib.swr_draw_meshlets(None, None, 1, 7, None), "unknown shader table")
