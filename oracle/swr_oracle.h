// Oracle for the meshlet raster pipeline: a single-threaded CPU restatement of
// GLimpSW's own CPU code (src/SwRast/*), written for this project.
//
// THIS IS TEST INFRASTRUCTURE. Only tests/, __graft_entry__.smoke() and the
// CPU-baseline legs of bench.py may load it, and only as the checker or the
// timed CPU baseline. The product (libswr_gb300.so) never calls into it.
//
// Parity status: UNPINNED against the reference binary. The reference cannot
// be compiled in this environment (clang-only vector extensions in
// src/SwRast/SIMD.h:19,194,256 and absent CPM dependencies), and the reference
// ships no tests or golden vectors. Every function here cites the reference
// file:line it restates; known-answer tests in tests/ pin hand-derived values.
//
// Float semantics: source order, IEEE round-to-nearest, no contraction
// (built with -ffp-contract=off); only the reference's explicit simd::fma calls
// are fused (std::fma). AVX-512 rcp14/rsqrt14 (SIMD.h:294-296) are reproduced
// bit for bit by the integer tables of include/swr/approx14.h (mode 0, every
// host); mode 1 runs the instructions on an AVX-512 host, mode 2 substitutes the
// correctly rounded 1/x and 1/sqrt(x).
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

// Framebuffer (Rasterizer.h:10-78): 4x4-tiled 32-bit layers.
typedef struct {
    uint32_t width, height, tile_stride, layer_stride, num_layers;
    uint32_t* data;  // num_layers * layer_stride words
} orc_framebuffer;

// Material (Scene.h:7-14). texture indexes orc_scene.textures (UINT32_MAX = none).
typedef struct {
    uint32_t texture;
    uint8_t is_double_sided;
    uint8_t alpha_cutoff;
    uint8_t pad[2];
} orc_material;

// Texture2D<Texel, TiledY8> (Texture.h:314-329) with data held out of line.
typedef struct {
    uint32_t width, height, mip_levels, num_layers;
    uint32_t row_shift, layer_stride;
    float scale_u, scale_v, scale_lerp_u, scale_lerp_v;
    int32_t mask_u, mask_v, mask_lerp_u, mask_lerp_v;
    uint32_t mip_offsets[16];
    uint32_t* data;
} orc_texture;

// Light (Scene.h:52-75).
typedef struct {
    uint32_t type;  // 0 directional, 1 point, 2 spot
    float position[3], direction[3], color[3];
    float intensity, radius, spot_inner, spot_outer;
    float inv_radius_sq, spot_scale, spot_offset;
} orc_light;

// ShadingContext (Shading.h:12-39), matrices column-major like glm.
typedef struct {
    const void* meshlets;           // Meshlet[] (1728-byte records)
    const orc_material* materials;
    const orc_texture* textures;    // indexed by orc_material.texture
    const orc_light* lights;
    uint32_t num_lights;
    uint32_t meshlet_offset;
    const uint16_t* cull_bitmap;    // one 16-bit mask per 16 meshlets, or NULL
    float world_to_clip[16];
    float object_to_clip[16];
    float object_to_world[9];       // glm::mat3, column-major
    const orc_texture* skybox;      // R11G11B10 octahedral map or NULL
    float view_pos[3];
    float exposure;
    uint32_t num_meshlets;          // size of the meshlet pool (bounds surface ids in the resolve)
} orc_shading_context;

// Rasterizer flags (Rasterizer.h:205-208) and the shader table of the draw: 0 VisBufferShader,
// 1 DeferredShader, 2 OverdrawShader (Shading.cpp:649-656), and 3, the texcoord shader of the
// shader-hook tests (depth test; depth, surface id, and the bits of the interpolated texcoords in
// layers 2 and 3).
typedef struct {
    int enable_binning, enable_clipping, enable_guardband;
    int shader;
} orc_raster_flags;
enum { ORC_SHADER_VISBUFFER = 0, ORC_SHADER_DEFERRED = 1, ORC_SHADER_OVERDRAW = 2, ORC_SHADER_TEXCOORD = 3 };

// PerfCounter (Rasterizer.h:366-370): processed, rasterized, clipped, bin flushes.
enum { ORC_TRIS_PROCESSED = 0, ORC_TRIS_RASTERIZED = 1, ORC_TRIS_CLIPPED = 2, ORC_BIN_FLUSHES = 3 };

uint32_t orc_meshlet_size(void);
void orc_set_approx_mode(int mode);  // 0: exact tables, 1: AVX-512 hardware (x86 only), 2: IEEE
int orc_approx_mode_available(int mode);
int64_t orc_approx14_mismatches(int which, uint64_t first, uint64_t count);
void orc_approx_eval(int which, const uint32_t* in, uint32_t* out, uint64_t n);

void orc_fb_init(orc_framebuffer* fb, uint32_t width, uint32_t height, uint32_t num_layers, uint32_t* storage);
uint32_t orc_fb_layer_stride(uint32_t width, uint32_t height);
void orc_fb_clear(orc_framebuffer* fb, uint32_t color, float depth);
void orc_fb_clear_layer(orc_framebuffer* fb, uint32_t layer, uint32_t value);
void orc_fb_get_pixels(const orc_framebuffer* fb, uint32_t layer, uint32_t* dest, uint32_t stride);

// Rasterizer::DrawMeshlets with the VisBufferShader table (Shading.cpp:649-654).
// Single-threaded: draw order is meshlet, packet, accepted lanes, clipped outputs.
void orc_draw_meshlets(orc_framebuffer* fb, uint32_t count, const orc_shading_context* ctx,
                       const orc_raster_flags* flags, uint64_t counters[4]);

// Same, restricted to framebuffer rows [row_begin, row_end) (used to split the CPU baseline
// across threads by screen strips; results equal the full draw on those rows).
void orc_draw_meshlets_rows(orc_framebuffer* fb, uint32_t count, const orc_shading_context* ctx,
                            const orc_raster_flags* flags, uint64_t counters[4],
                            uint32_t row_begin, uint32_t row_end);

// Multi-threaded CPU baseline: splits rows over num_threads std::threads.
void orc_draw_meshlets_mt(orc_framebuffer* fb, uint32_t count, const orc_shading_context* ctx,
                          const orc_raster_flags* flags, uint32_t num_threads);

// Rasterizer(num_threads)::DrawMeshlets with binning on (Rasterizer.cpp:493-820), threaded in the
// reference's shape: meshlets strided over workers, 128x128 bins, each bin rasterized by its elected
// worker. The timed CPU baseline; non-trivial triangles are dropped (binned semantics).
void orc_draw_meshlets_binned(orc_framebuffer* fb, uint32_t count, const orc_shading_context* ctx, uint32_t num_threads,
                              uint64_t counters[4]);

// ShadingContext::CullMeshlets (Shading.cpp:775-869).
uint32_t orc_cull_meshlets(uint16_t* bitmap, const void* meshlets, uint32_t count,
                           const float proj[16], const float view[16], const float model[16],
                           const float prev_view[16], float frame_w, float frame_h,
                           const orc_texture* depth_map);

// Texture creation (Texture.h:599-636), SetPixels (336-354), GenerateMips (382-388, 577-596).
// format: 0 RGBA8u, 1 R11G11B10f, 2 R32f.
uint64_t orc_texture_storage_words(uint32_t width, uint32_t height, uint32_t max_levels, uint32_t num_layers);
void orc_texture_init(orc_texture* tex, uint32_t width, uint32_t height, uint32_t max_levels,
                      uint32_t num_layers, uint32_t* storage);
void orc_texture_set_pixels(orc_texture* tex, const uint32_t* pixels, uint32_t stride, uint32_t layer, uint32_t mip);
void orc_texture_generate_mips(orc_texture* tex, uint32_t format);

// texutil::DownsampleDepth (ImageHelpers.cpp:150-247).
void orc_downsample_depth(const orc_framebuffer* fb, orc_texture* dest);

// ShadingContext::Resolve (Shading.cpp:658-690), light-sprite overlay excluded.
void orc_resolve(orc_framebuffer* fb, const orc_shading_context* ctx);
void orc_resolve_rows(orc_framebuffer* fb, const orc_shading_context* ctx, uint32_t row_begin, uint32_t row_end);
void orc_resolve_mt(orc_framebuffer* fb, const orc_shading_context* ctx, uint32_t num_threads);

// ShadingContext::ResolveDebug (Shading.cpp:734-773); layer is a DebugLayer (Shading.h:8):
// 0 None, 1 BaseColor, 2 Normals, 3 MetallicRoughness, 4 MeshletId, 5 TriangleId,
// 6 OverdrawPixel, 7 OverdrawQuad.
void orc_resolve_debug_rows(orc_framebuffer* fb, const orc_shading_context* ctx, uint32_t layer,
                            uint32_t row_begin, uint32_t row_end);
void orc_resolve_debug_mt(orc_framebuffer* fb, const orc_shading_context* ctx, uint32_t layer, uint32_t num_threads);

// Image-based lighting precompute (Shading.cpp:35-219), one output texel each:
// PrefilterDiffuseIrradiance of texel (x, y) of a w x h map (packed R11G11B10), PrefilterEnvMap of
// texel (x, y) of mip `level` of a `levels`-mip map with level 0 of w0 x h0 (R11G11B10), and
// IntegrateBRDF of texel (x, y) of a w x h table (packed RG16f). env: an R11G11B10 octahedral map.
uint32_t orc_ibl_irradiance_texel(const orc_texture* env, uint32_t x, uint32_t y, uint32_t w, uint32_t h);
uint32_t orc_ibl_radiance_texel(const orc_texture* env, uint32_t level, uint32_t levels, uint32_t x, uint32_t y,
                                uint32_t w0, uint32_t h0);
uint32_t orc_ibl_env_brdf_texel(uint32_t x, uint32_t y, uint32_t w, uint32_t h);

#ifdef __cplusplus
}
#endif
