"""An imported glTF model drawn on the GPU through gltf.upload / gltf.draw against the oracle fed
the same meshlets, instance by instance: the vis-buffer bit for bit (the plane's material is
alpha-masked, so the alpha pass runs with the model's own texcoords) and the resolve within 1/255,
lit by the frame driver's default light and the model's own point light."""
import numpy as np
import pytest

from glimpsw_gb300 import gltf, scenes
from tests import gltf_fixtures
from tests.helpers import TexturePair, assert_visbuffer_equal, default_lights, gpu_lights, model_lights

pytestmark = pytest.mark.gpu


def test_imported_model_matches_oracle(tmp_path):
    from glimpsw_gb300 import api
    from oracle import oracle as O
    m = gltf.load(gltf_fixtures.build(str(tmp_path))[1])
    assert not m.warnings
    lights = np.concatenate([default_lights(), model_lights(m)])
    assert len(m.lights) == 1 and int(lights["type"][1]) == 1
    scene, texs = gltf.upload(m)
    otex = [TexturePair(layers, layers[0].shape[0], gpu=False) for layers in m.textures]
    rast = api.Rasterizer()
    rast.EnableBinning = False
    for eye, target in (((0.0, 3.0, -6.0), (0.5, 0.5, 0.0)), ((0.3, 0.4, 0.2), (3.0, 0.0, 4.0))):
        v = scenes.make_view(480, 272, eye=eye, target=target)
        fb = api.Framebuffer(v.width, v.height)
        fb.clear(0xFF000000, 0.0)
        gltf.draw(m, scene, rast, fb, v.proj, v.view)
        ofb = O.Framebuffer(v.width, v.height)
        ofb.clear(0xFF000000, 0.0)
        for inst in m.instances:
            bm, _ = O.cull_meshlets(m.meshlets[inst.meshlet_offset:], inst.meshlet_count, v.proj, v.view, inst.transform,
                                    v.view, v.width, v.height)
            ctx = O.Context(m.meshlets, m.materials, scenes.mat_mul(v.world_to_clip, inst.transform),
                            world_to_clip=v.world_to_clip, meshlet_offset=inst.meshlet_offset, cull_bitmap=bm,
                            textures=[t.o for t in otex])
            O.draw_meshlets(ofb, ctx, inst.meshlet_count)
        assert_visbuffer_equal(fb, ofb)
        ids = fb.get_pixels(0)
        assert (ids != 0xFF000000).sum() > 3000
        # resolve (one instance's object transform is the reference frame driver's choice: identity)
        octx = O.Context(m.meshlets, m.materials, v.world_to_clip, world_to_clip=v.world_to_clip,
                         textures=[t.o for t in otex], lights=lights, view_pos=v.eye)
        O.resolve(ofb, octx, threads=8)
        gctx = api.ShadingContext(scene, v.world_to_clip, world_to_clip=v.world_to_clip, view_pos=v.eye,
                                  lights=gpu_lights(lights))
        gctx.resolve(rast, fb)
        a = fb.get_pixels(0).view(np.uint8).astype(np.int32)
        b = ofb.get_pixels(0).view(np.uint8).astype(np.int32)
        assert np.abs(a - b).max() <= 1
