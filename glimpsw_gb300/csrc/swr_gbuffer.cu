// ShadingContext::DeferredShader (Shading.cpp:655): the mesh shader ShadeMeshlet with the fragment
// shader FS_EncodeGBuffer (Shading.cpp:344-414) as the first client of the shader hooks
// (include/swr/shader.cuh). Visibility runs the library's raster with FS_EncodeGBuffer's alpha test
// (every textured material, texel alpha >= AlphaCutoff); the fragment stage then shades the visible
// fragment of each pixel: base colour into layer 0 and the packed normal / metal / roughness into
// layer 2 (the depth is already in layer 1).
#include <cstring>

#include "../../include/swr/shader.cuh"
#include "swr_internal.h"
#include "swr_sample.cuh"
#include "swr_surface.cuh"

namespace swr {
namespace {

struct GBufferCtx {
    const uint8_t* meshlets;
    const DevMaterial* materials;
    uint32_t numMaterials;
    float objectToWorld[9];  // ShadingContext::ObjectToWorldMat (glm::mat3)
};

// Mesh::TexCoords / NormalTangents [VertexId]: the index byte is not bounded by the reference; words
// past the array are the record's following fields, and past the record (the next record in the
// reference) 0 here.
__device__ __forceinline__ uint32_t record_word(const uint8_t* rec, uint32_t offset, uint32_t idx) {
    return offset + 4 * idx < kMeshletSize ? *(const uint32_t*)(rec + offset + 4 * idx) : 0u;
}

// FS_EncodeGBuffer without its depth and alpha tests (done by visibility) for the 16 lanes of a tile.
struct EncodeGBuffer {
    __device__ void operator()(const GBufferCtx& c, const FragmentFramebuffer& fb, FragmentVars& v) const {
        const uint8_t* rec = c.meshlets + (size_t)v.MeshletId * kMeshletSize;
        const uint32_t matId = *(const uint32_t*)(rec + kOffMaterialId);
        if (matId == 0xFFFFFFFFu || matId >= c.numMaterials) return;  // depth only (Shading.cpp:350-353)
        const DevMaterial& mt = c.materials[matId];
        uint32_t baseColor = 0xFFFFFFFFu, ch2 = 0;
        if (mt.has_texture) {
            const DevTexture& tex = mt.tex;
            float2 t[3];
#pragma unroll
            for (int k = 0; k < 3; k++) {  // UnpackHalf2x16 (Shading.cpp:228-231)
                const uint32_t w = record_word(rec, kOffTexCoords, v.VertexId[k]);
                t[k] = make_float2(h2f(w & 0xFFFF), h2f(w >> 16));
            }
            const float2 uv = v.Interpolate(t[0], t[1], t[2]);
            // SampleImplicitLod (Texture.h:403-410): CalcMipLevel of the 2x2 differences of the scaled
            // sample position, minus LerpFracBits; the filter is chosen over the whole tile
            const float su = fmul(uv.x, tex.scale_lerp_u), sv = fmul(uv.y, tex.scale_lerp_v);
            const float gx = v.dFdx(su), gy = v.dFdx(sv), gz = v.dFdy(su), gw = v.dFdy(sv);
            const float dx = ffma(gx, gx, fmul(gy, gy)), dy = ffma(gz, gz, fmul(gw, gw));
            const int32_t mip = (ilog2_x86(vmax(dx, dy)) >> 1) - 8;
            const bool nearest = v.TileAny(mip > 0);
            baseColor = sample_rgba8(tex, uv.x, uv.y, 0, mip, nearest);
            if (tex.num_layers >= 2) {
                const uint32_t nmr = sample_rgba8(tex, uv.x, uv.y, 1, mip, nearest);  // Nx Ny M R
                // Z from the 2-channel normal map (Shading.cpp:365-367)
                const float tx = (float)(nmr & 255) * (1.0f / 127.5f) - 1.0f;
                const float ty = (float)((nmr >> 8) & 255) * (1.0f / 127.5f) - 1.0f;
                const float tz = approx_sqrt(1.0f - (tx * tx + ty * ty));
                F3 n[3], g[3];
#pragma unroll
                for (int k = 0; k < 3; k++) unpack_normal_tangent(record_word(rec, kOffNormalTangents, v.VertexId[k]), n[k], g[k]);
                auto lerp3 = [&](const F3* a) {
                    return F3{ v.Interpolate(a[0].x, a[1].x, a[2].x), v.Interpolate(a[0].y, a[1].y, a[2].y),
                               v.Interpolate(a[0].z, a[1].z, a[2].z) };
                };
                const F3 N = normalize3(mul3(c.objectToWorld, lerp3(n)));
                const F3 T = normalize3(mul3(c.objectToWorld, lerp3(g)));
                // TangentHandedness >> VertexId[0]: a 64-bit shift takes its count modulo 64
                const unsigned long long hand64 = *(const unsigned long long*)(rec + kOffHandedness);
                const uint32_t hand = (uint32_t)((hand64 >> (v.VertexId[0] & 63)) & 1) << 31;
                F3 B = cross3(N, T);
                B = { __uint_as_float(__float_as_uint(B.x) ^ hand), __uint_as_float(__float_as_uint(B.y) ^ hand),
                      __uint_as_float(__float_as_uint(B.z) ^ hand) };
                const F3 R = normalize3({ tx * T.x + ty * B.x + tz * N.x, tx * T.y + ty * B.y + tz * N.y,
                                          tx * T.z + ty * B.z + tz * N.z });
                float ou, ov;
                map_oct(R, ou, ov);
                ch2 = __float2uint_rz(ou * 1023.0f + 0.5f);
                ch2 |= __float2uint_rz(ov * 1023.0f + 0.5f) << 10;
                ch2 |= ((nmr >> 18) & 0x3F) << 20;
                ch2 |= ((nmr >> 26) & 0x3F) << 26;
            }
        }
        v.StoreTile(fb.GetColorBuffer(), baseColor);
        v.StoreTile(fb.GetLayerData(2), ch2);
    }
};

}  // namespace
}  // namespace swr

using namespace swr;

swr_status swr_internal_draw_deferred(swr_rasterizer r, swr_framebuffer fb, uint32_t count, const swr_shading_context* ctx) {
    if (!r || !fb || !ctx || !ctx->scene) return swr_internal_fail(SWR_EINVAL, "swr_draw_meshlets: NULL argument");
    if (fb->num_layers < 3)
        return swr_internal_fail(SWR_EINVAL, "swr_draw_meshlets: DeferredShader writes layer 2; the framebuffer has fewer layers");
    swr_status s = swr_draw_meshlets_hooked(r, fb, count, ctx, 1);
    if (s != SWR_OK || count == 0) return s;
    swr_fragment_source src;
    s = swr_fragment_source_get(r, fb, count, nullptr, ctx, &src);
    if (s != SWR_OK) return s;
    GBufferCtx g = {};
    g.meshlets = ctx->scene->meshlets;
    g.materials = ctx->scene->materials;
    g.numMaterials = ctx->scene->num_materials;
    memcpy(g.objectToWorld, ctx->object_to_world, sizeof(g.objectToWorld));
    cudaStream_t st = swr_internal_stream();
    {
        LaunchScope ls("k_shade_fragments_gbuffer", st);
        s = ShadeFragments<GBufferCtx, EncodeGBuffer>(src, g, st);
    }
    if (s != SWR_OK) return swr_internal_fail(SWR_ECUDA, "swr_draw_meshlets: FS_EncodeGBuffer launch failed");
    return SWR_OK;
}
