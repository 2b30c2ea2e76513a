// Shaders a user of the library would write, compiled against include/swr/shader.cuh into their own
// shared library (tests/user_shader/build.py) and driven from the tests through the C functions at
// the end. They exercise both hooks:
//  - TexcoordFS: a fragment shader writing the surface id (layer 0) and the bits of the
//    perspective-correct interpolated texcoords (layers 2 and 3), the reference's
//    FragmentVars::Interpolate of Mesh::TexCoords[VertexId];
//  - CustomMesh: a mesh shader that transforms like ShadeMeshlet by a matrix of its own context,
//    culls every meshlet whose index is 4 mod 5 (PrimCount 0), draws the ones that are 0 mod 3
//    double-sided, and selects fragment entry point idx & 1 (entry point 1 marks its surface ids with
//    bit 30).
#include <cuda_fp16.h>
#include <swr/shader.cuh>

#include <cstring>

namespace {

struct HookCtx {
    const uint8_t* meshlets;  // the scene's records (swr_scene_meshlets_device)
    uint32_t meshletOffset;   // the draw's first meshlet
    float objectToClip[16];   // CustomMesh's transform
};

template <uint32_t kMark>
struct TexcoordFS {
    __device__ void operator()(const HookCtx& c, const swr::FragmentFramebuffer& fb, swr::FragmentVars& v) const {
        const uint8_t* rec = c.meshlets + (size_t)v.MeshletId * 1728u;
        float2 t[3];
        for (int k = 0; k < 3; k++) {  // Mesh::TexCoords[VertexId] (words past the array: the record's next fields)
            const uint32_t off = 832u + 4u * v.VertexId[k];
            const uint32_t w = off < 1728u ? *(const uint32_t*)(rec + off) : 0u;
            t[k] = make_float2(__half2float(__ushort_as_half((unsigned short)(w & 0xFFFF))),
                               __half2float(__ushort_as_half((unsigned short)(w >> 16))));
        }
        const float2 uv = v.Interpolate(t[0], t[1], t[2]);
        v.StoreTile(fb.GetColorBuffer(), (v.MeshletId * 128u + v.PrimId) | kMark);
        v.StoreTile(fb.GetLayerData(2), __float_as_uint(uv.x));
        v.StoreTile(fb.GetLayerData(3), __float_as_uint(uv.y));
    }
};

struct CustomMesh {
    __device__ void operator()(const HookCtx& c, uint32_t idx, swr::ShadedMeshlet& out) const {
        const uint32_t lane = swr::mesh_lane();
        const uint8_t* rec = c.meshlets + (size_t)(c.meshletOffset + idx) * 1728u;
        const float* P = (const float*)(rec + 64);
        const uint32_t nv = rec[44], nvr = min((nv + 15u) & ~15u, 64u);  // ShadeMeshlet's 16-vertex chunks
        for (uint32_t v = lane; v < 64; v += 32) {
            const float4 p = v < nvr ? swr::clip_transform(P[v], P[64 + v], P[128 + v], c.objectToClip)
                                     : make_float4(0.f, 0.f, 0.f, 0.f);
            out.position[0][v] = p.x, out.position[1][v] = p.y, out.position[2][v] = p.z, out.position[3][v] = p.w;
        }
        for (uint32_t i = lane; i < 3 * 128; i += 32) (&out.indices[0][0])[i] = rec[1344 + i];
        if (lane == 0) {
            out.prim_count = (idx % 5 == 4) ? 0 : rec[45];
            out.cull_mode = (idx % 3 == 0) ? swr::kFaceCullNone : swr::kFaceCullFrontCCW;
            out.fragment_shader_id = (uint8_t)(idx & 1);
        }
    }
};

HookCtx make_ctx(const swr_shading_context* sctx) {
    HookCtx c = {};
    swr_scene_meshlets_device(sctx->scene, (const void**)&c.meshlets);
    c.meshletOffset = sctx->meshlet_offset;
    memcpy(c.objectToClip, sctx->object_to_clip, sizeof(c.objectToClip));
    return c;
}

}  // namespace

// The library's ShadeMeshlet with TexcoordFS for every entry point.
extern "C" swr_status hook_draw_texcoords(swr_rasterizer r, swr_framebuffer fb, uint32_t count, const swr_shading_context* sctx) {
    return swr::DrawMeshlets<swr::ShadeMeshletFn, HookCtx, TexcoordFS<0u>>(r, fb, count, sctx, make_ctx(sctx));
}

// CustomMesh (transform by object_to_clip) with TexcoordFS at entry point 0 and its marked variant at 1.
extern "C" swr_status hook_draw_custom_mesh(swr_rasterizer r, swr_framebuffer fb, uint32_t count,
                                            const swr_shading_context* sctx) {
    return swr::DrawMeshlets<CustomMesh, HookCtx, TexcoordFS<0u>, TexcoordFS<0x40000000u>>(r, fb, count, sctx,
                                                                                         make_ctx(sctx));
}
