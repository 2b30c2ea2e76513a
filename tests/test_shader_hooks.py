"""The shader hooks on the CPU: user shaders compile against include/swr/shader.cuh for sm_103a into
their own library, which links against libswr_gb300 (nvcc runs without a GPU), and the library
exports the entry points the hooks drive."""
import ctypes as C


def test_user_shaders_build_and_export():
    from tests.user_shader import build
    lib = C.CDLL(build.build())
    for name in ("hook_draw_texcoords", "hook_draw_custom_mesh"):
        assert hasattr(lib, name)


def test_library_exports_hook_entry_points():
    from glimpsw_gb300 import api
    lib = api.load_library()
    for name in ("swr_draw_shaded_meshlets", "swr_draw_meshlets_hooked", "swr_fragment_source_get",
                 "swr_scene_meshlets_device"):
        assert hasattr(lib, name)


def test_shaded_meshlet_layout_matches_reference():
    """swr_shaded_meshlet keeps ShadedMeshlet's layout (Rasterizer.h:82-99): 3 header bytes, Indices
    at 64, Position at 448 (both 64-byte aligned), 1472 bytes."""
    import subprocess
    import tempfile
    import os
    from glimpsw_gb300 import build as lib_build
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = ('#include <stddef.h>\n#include "swr_gb300.h"\n'
           'int main(void) { return !(sizeof(swr_shaded_meshlet) == 1472 && offsetof(swr_shaded_meshlet, indices) == 64'
           ' && offsetof(swr_shaded_meshlet, position) == 448 && offsetof(swr_shaded_meshlet, fragment_shader_id) == 2); }\n')
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "t")
        subprocess.run(["gcc", "-I", os.path.join(root, "include"), c, "-o", exe], check=True)
        assert subprocess.run([exe]).returncode == 0
