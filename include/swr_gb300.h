/*
 * libswr_gb300 — C ABI of the GB300 (sm_103a) meshlet raster pipeline.
 *
 * Each entry point replaces one entry point of GLimpSW's C++ API (src/SwRast/..., cited per
 * function). Handles own device memory; callers keep their host copies. No exception crosses
 * this boundary: every function returns an swr_status and swr_last_error() describes the last
 * failure on the calling thread.
 *
 * Execution model: work is enqueued on the calling thread's current stream (swr_set_stream;
 * default: the per-thread default stream) and runs asynchronously, in stream order. Functions
 * that return data to host memory (swr_framebuffer_get_pixels, swr_cull_meshlets' count,
 * swr_rasterizer_get_counters, swr_texture_get_data) synchronise that stream first, which gives
 * the reference's blocking semantics at the points where it matters.
 */
#ifndef SWR_GB300_H
#define SWR_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    SWR_OK = 0,
    SWR_EINVAL = 1,      /* bad argument: size above 2896 or not a multiple of 4, bad handle, ... */
    SWR_ECAPACITY = 2,   /* an internal bound was exceeded (message says which) */
    SWR_ETIMEOUT = 3,    /* a bounded device-side wait gave up */
    SWR_ECUDA = 4,       /* CUDA runtime error (message carries the CUDA error string) */
    SWR_ENOMEM = 5       /* device allocation failed */
} swr_status;

typedef struct swr_rasterizer_t* swr_rasterizer;
typedef struct swr_framebuffer_t* swr_framebuffer;
typedef struct swr_scene_t* swr_scene;
typedef struct swr_texture_t* swr_texture;

/* Limits: Rasterizer::MaxRenderSize (Rasterizer.h:203); the vis-buffer tie-break rank packs
 * the global meshlet index into 21 bits. */
#define SWR_MAX_RENDER_SIZE 2896u
#define SWR_MAX_MESHLETS (1u << 21)
#define SWR_MESHLET_SIZE 1728u

/* ShadingContext::VisBufferShader (Shading.cpp:649-654): mesh shader ShadeMeshlet with fragment
 * entry points FS_EncodeSurfaceId<false> (0) and FS_EncodeSurfaceId<true> (1). */
#define SWR_SHADER_VISBUFFER 0u
/* ShadingContext::DeferredShader (Shading.cpp:655): ShadeMeshlet with FS_EncodeGBuffer (344-414) for
 * every fragment entry point. A fragment survives the depth test and, when its material has a
 * texture, the alpha test texel alpha >= AlphaCutoff (for every material, cutoff 255 included); the
 * front-most survivor writes depth (layer 1), its base colour (layer 0) and, for two-layer
 * textures, the packed octahedral normal and metal/roughness (layer 2; 0 otherwise). Needs a
 * framebuffer of 3 layers. Shading runs after visibility (the fragment stage of the shader hooks,
 * swr/shader.cuh), so only the visible fragment of each pixel is shaded. Defined deviations: a
 * material without a texture (the reference dereferences it) passes the alpha test with base colour
 * 0xFFFFFFFF and layer 2 = 0; a visible surface without a material stores its depth and leaves
 * layers 0 and 2 as they were (where the reference keeps the colour of the last material fragment
 * drawn there, which may lie behind it). */
#define SWR_SHADER_DEFERRED 1u
/* ShadingContext::OverdrawShader (Shading.cpp:656): FS_Overdraw (333-342) for every fragment entry
 * point. No depth test: each 4x4 tile a triangle covers adds 1 to the high 16 bits of its covered
 * pixels' layer-0 words and 1 to the low 16 bits of the others (saturating), and layer 1 keeps the
 * maximum depth of all 16 samples. Clear layer 0 to 0 first (Main.cpp:213). */
#define SWR_SHADER_OVERDRAW 2u

/* DebugLayer (Shading.h:8) for swr_resolve_debug. */
#define SWR_DEBUG_NONE 0u
#define SWR_DEBUG_BASE_COLOR 1u
#define SWR_DEBUG_NORMALS 2u
#define SWR_DEBUG_METALLIC_ROUGHNESS 3u
#define SWR_DEBUG_MESHLET_ID 4u
#define SWR_DEBUG_TRIANGLE_ID 5u
#define SWR_DEBUG_OVERDRAW_PIXEL 6u
#define SWR_DEBUG_OVERDRAW_QUAD 7u

/* Texel formats (pixfmt::*, Texture.h:23-200). */
#define SWR_FORMAT_RGBA8U 0u
#define SWR_FORMAT_R11G11B10F 1u
#define SWR_FORMAT_R32F 2u
#define SWR_FORMAT_RG16F 3u  /* pixfmt::RG16f (Texture.h:105-133): two IEEE halves, R in the low 16 bits */

/* Perf counters (PerfCounter, Rasterizer.h:366-370). */
#define SWR_COUNTER_TRIANGLES_PROCESSED 0
#define SWR_COUNTER_TRIANGLES_RASTERIZED 1
#define SWR_COUNTER_TRIANGLES_CLIPPED 2
#define SWR_COUNTER_BIN_QUEUE_FLUSHES 3
#define SWR_NUM_COUNTERS 4

/* Material (Scene.h:7-14); texture may be NULL. alpha_cutoff < 255 selects the alpha-tested
 * vis-buffer shader (FS_EncodeSurfaceId<true>, Shading.cpp:302-331): a fragment is kept if the
 * texture's layer-0 texel at its implicit LOD has alpha >= alpha_cutoff. A material without a
 * texture (which the reference would dereference) keeps every fragment. */
typedef struct {
    swr_texture texture;
    uint8_t is_double_sided;
    uint8_t alpha_cutoff;
} swr_material;

/* Light (Scene.h:52-75), with the precomputed InvRadiusSq/SpotScale/SpotOffset. */
typedef struct {
    uint32_t type; /* 0 directional, 1 point, 2 spot */
    float position[3], direction[3], color[3];
    float intensity, radius, spot_inner_angle, spot_outer_angle;
    float inv_radius_sq, spot_scale, spot_offset;
} swr_light;

/* ShadingContext (Shading.h:12-39). Matrices are column-major (glm layout). */
typedef struct {
    swr_scene scene;                 /* Meshlets + Materials */
    uint32_t meshlet_offset;         /* MeshletOffset */
    const uint16_t* cull_bitmap;     /* device pointer, one bit per meshlet of the draw, or NULL */
    float world_to_clip[16];
    float object_to_clip[16];
    float object_to_world[9];        /* glm::mat3 */
    swr_texture skybox;              /* R11G11B10 octahedral map, or NULL */
    float view_pos[3];
    float exposure;
    const swr_light* lights;         /* host array, copied at call time */
    uint32_t num_lights;
} swr_shading_context;

/* ---- errors and streams ---- */
const char* swr_last_error(void);
swr_status swr_set_stream(void* cuda_stream);      /* cudaStream_t; NULL = per-thread default */
void* swr_get_stream(void);
swr_status swr_synchronize(void);

/* ---- tracing: the reference's Tracy zones and SWR_PERF timers (Rasterizer.cpp:494-643,
 * Rasterizer.h:397-399) become per-kernel CUDA events ---- */
uint64_t swr_launch_count(void);                   /* kernels launched by this library so far */
swr_status swr_profile_enable(int enable);         /* record events around each launch (this thread) */
/* Synchronises, returns up to max_records (kernel name, milliseconds) pairs recorded since the
 * last collect, and clears the record list; *count receives the number recorded. */
swr_status swr_profile_collect(uint32_t max_records, const char** names, float* ms, uint32_t* count);

/* ---- Rasterizer (Rasterizer.h:202-213) ---- */
/* Rasterizer::Rasterizer(uint32_t numThreads): numThreads has no GPU meaning and is ignored. */
swr_status swr_rasterizer_create(uint32_t num_threads, swr_rasterizer* out);
swr_status swr_rasterizer_destroy(swr_rasterizer r);
/* EnableBinning / EnableClipping / EnableGuardband (Rasterizer.h:205-208). Binning selects the
 * reference's binned semantics (non-trivial triangles dropped, guard band always on); otherwise
 * non-trivial triangles are clipped when clipping is enabled. */
swr_status swr_rasterizer_set_flags(swr_rasterizer r, int enable_binning, int enable_clipping,
                                    int enable_guardband);
/* Capacity (triangles) of the device queue that carries large and clipped triangles from the
 * mesh stage to the chunk rasterizer; 0 (default) sizes it per draw. The reference bounds the
 * equivalent per-bin queues at compile time (MaxBinSize/MaxWorkerBatch, Rasterizer.cpp:14) and
 * flushes early when they fill; here a full queue makes the mesh stage rasterize the triangle
 * itself, so any capacity gives the same image. Used to exercise that path in tests. */
swr_status swr_rasterizer_set_queue_capacity(swr_rasterizer r, uint32_t triangles);
/* perf::GetCurrent / perf::Reset (Rasterizer.h:381-395): device-side counters. */
swr_status swr_rasterizer_get_counters(swr_rasterizer r, uint64_t out[SWR_NUM_COUNTERS]);
swr_status swr_rasterizer_reset_counters(swr_rasterizer r);

/* Rasterizer::DrawMeshlets(Framebuffer&, count, ShaderBinding) (Rasterizer.h:213,
 * Rasterizer.cpp:493-644) with ShaderBinding{VisBufferShader, &ctx}: FragmentShaderId 0 (opaque)
 * or 1 (alpha-tested) per meshlet material. Depth test GREATER with equal depths resolved to the
 * first-submitted triangle of a single-threaded draw. */
swr_status swr_draw_meshlets(swr_rasterizer r, swr_framebuffer fb, uint32_t count, uint32_t shader_table,
                             const swr_shading_context* ctx);

/* ---- Shader hooks (Rasterizer.h:82-138, 178-196) ----
 * The reference binds a mesh shader MeshFn(ctx, idx, ShadedMeshlet&) and up to four fragment
 * shaders FragFn(ctx, Framebuffer&, FragmentVars&) as CPU function pointers. On the GPU they are
 * __device__ functors instantiated into the kernels of the header-only swr/shader.cuh
 * (swr::DrawMeshlets<MeshFn, FragFn...>), which drives the entry points below. */

/* ShadedMeshlet (Rasterizer.h:82-99), the reference's layout: 1472 bytes, 64-byte aligned. */
typedef struct {
    uint8_t prim_count;          /* PrimCount (0: nothing is drawn) */
    uint8_t cull_mode;           /* FaceCullMode: 0 None, 1 FrontCCW, 2 FrontCW */
    uint8_t fragment_shader_id;  /* FragmentShaderId: entry point 0-3 of the fragment stage */
    uint8_t pad[61];
    uint8_t indices[3][128];     /* Indices: vertex slots of each primitive */
    float position[4][64];       /* Position: clip-space x, y, z, w of each vertex slot */
} swr_shaded_meshlet;

/* Rasterizer::DrawMeshlets for meshlets a mesh shader has already shaded: shaded_device holds count
 * swr_shaded_meshlet records (device memory), record i standing for meshlet ctx->meshlet_offset + i of
 * the scene (whose texcoords and material the alpha test of FragmentShaderId 1 reads). Visibility
 * only: the depth test, alpha test and tie rules of swr_draw_meshlets; the keys stay pending for
 * swr_fragment_source_get. ctx->cull_bitmap and ctx->object_to_clip are not used (the mesh shader
 * culls by PrimCount 0 and transforms). Single view. */
swr_status swr_draw_shaded_meshlets(swr_rasterizer r, swr_framebuffer fb, uint32_t count, const void* shaded_device,
                                    const swr_shading_context* ctx);

/* Everything the fragment stage of swr/shader.cuh needs to rebuild the visible fragments of one
 * draw, in device memory. */
typedef struct {
    uint64_t* keys;                  /* per-pixel vis-buffer keys (4x4-tiled like the layers) */
    uint32_t* layers;                /* layer k at layers + k * layer_stride */
    uint32_t width, height, layer_stride, num_layers;
    const void* meshlets;            /* the scene's Meshlet records */
    const void* shaded;              /* the draw's swr_shaded_meshlet records, or NULL (built-in ShadeMeshlet) */
    const uint8_t* material_fs_ids;  /* FragmentShaderId of each material under ShadeMeshlet (0 or 1) */
    uint32_t num_materials;
    uint32_t meshlet_offset, count;  /* the draw's meshlets: [meshlet_offset, meshlet_offset + count) */
    float object_to_clip[16];        /* ShadeMeshlet's transform (built-in mesh shader) */
    float guard_x, guard_y;          /* guard-band factors of the clipper */
    int32_t half_w, half_h;
    uint32_t clip_mode;              /* non-trivial triangles were clipped (1) or dropped (0) */
} swr_fragment_source;

/* Writes the depth of the draw's visible fragments to layer 1 and fills *out for the fragment stage
 * of the draw just made with swr_draw_meshlets_hooked or swr_draw_shaded_meshlets (count meshlets
 * from ctx->meshlet_offset; shaded_device as given to the draw, or NULL). The fragment stage then
 * shades every pixel whose visible fragment belongs to the draw and marks the pixel done. */
swr_status swr_fragment_source_get(swr_rasterizer r, swr_framebuffer fb, uint32_t count, const void* shaded_device,
                                   const swr_shading_context* ctx, swr_fragment_source* out);

/* The visibility part of swr_draw_meshlets for a draw whose fragment stage is user code
 * (swr/shader.cuh): mesh shader ShadeMeshlet, depth and alpha tests as SWR_SHADER_VISBUFFER (with
 * alpha_test_all, as SWR_SHADER_DEFERRED: every textured material's texel alpha >= its cutoff). */
swr_status swr_draw_meshlets_hooked(swr_rasterizer r, swr_framebuffer fb, uint32_t count,
                                    const swr_shading_context* ctx, int alpha_test_all);

/* No counterpart in the reference. The vis-buffer draw of swr_draw_meshlets for callers that
 * cannot allocate device memory (their memory belongs to another allocator, or they run where
 * cudaMalloc is not allowed): every input and output is a caller-owned device pointer and the call
 * allocates nothing. meshlets: Meshlet records (device); material_flags: one byte per material,
 * bit 0 = double-sided, other bits reserved (device, or NULL with num_materials 0). It takes no
 * textures, so materials are never alpha-tested: every meshlet draws with the opaque shader
 * (FragmentShaderId 0), where swr_draw_meshlets would alpha-test the meshlets of a material with
 * alpha_cutoff < 255 and a texture. cull_bitmap as in
 * swr_shading_context; object_to_clip: host. surface_ids and depth are the framebuffer's layers 0
 * and 1 in the 4x4-tiled layout (width*height words each, device): they are read for the depth
 * test and updated like the layers of a framebuffer. Limits: width*height <= 1048576 pixels and
 * at most 1024 materials, else SWR_ECAPACITY. Working memory is one fixed device array (about
 * 9.3 MiB, held by every GPU that loads the library until the process exits), shared by every
 * call: calls whose work overlaps on the GPU race, so serialise them (one stream). The first call
 * on each device (and the first after a cudaDeviceReset) looks up that array's device address; make
 * it before any stream capture. */
swr_status swr_draw_meshlets_noalloc(const void* meshlets, uint32_t meshlet_offset, uint32_t count,
                                     const uint8_t* material_flags, uint32_t num_materials,
                                     const uint16_t* cull_bitmap, const float object_to_clip[16],
                                     uint32_t* surface_ids, float* depth, uint32_t width, uint32_t height,
                                     int enable_binning, int enable_clipping, int enable_guardband);

/* ---- Batched multi-view rendering (no reference counterpart: the reference issues one
 * DrawMeshlets per view, Main.cpp:216-245) ----
 * A batch renders the meshlets [first, first+count) of a scene into many framebuffers of any
 * sizes. Each view's result equals, bit for bit, swr_framebuffer_clear(fb, 0xFF000000, 0) +
 * swr_cull_meshlets (frustum only, when frustum_cull) + swr_draw_meshlets with the rasterizer's
 * flags. The frame runs as one CUDA graph (batched clear, batched cull, one persistent mesh-stage
 * launch over every (view, meshlet), the chunk rasterizer, batched finalize), captured at the first
 * render and replayed on the calling thread's stream. */
typedef struct swr_batch_t* swr_batch;
typedef struct {
    swr_framebuffer fb;
    float proj[16], view[16], model[16];   /* object_to_clip = proj * view * model */
    uint32_t depth_only;                   /* keep only the depth layer (shadow-map style views) */
} swr_view_desc;
/* frustum_cull: bit 0 (SWR_CULL_FRUSTUM) culls each view's frustum as swr_cull_meshlets does; bit 1
 * (SWR_CULL_BACKFACE_CONE) adds the backface-cone test of swr_cull_meshlets_ex. */
#define SWR_CULL_FRUSTUM 1u
swr_status swr_batch_create(swr_rasterizer r, swr_scene s, uint32_t first, uint32_t count, const swr_view_desc* views,
                            uint32_t num_views, int frustum_cull, swr_batch* out);
/* New matrices for the same framebuffers (takes effect at the next render; no re-capture). */
swr_status swr_batch_set_views(swr_batch b, const swr_view_desc* views, uint32_t num_views);
/* Chunk (bin) edge in 4x4 tiles: 2, 4, 8, 16 (8-64 pixels); warps per mesh-stage block: 4, 8, 16;
 * 0 = default (8, 8). Changing them re-captures the graph at the next render. */
swr_status swr_batch_set_tuning(swr_batch b, uint32_t chunk_tiles, uint32_t warps_per_block);
/* Rectangular chunks (bins) of the chunk rasterizer: chunk_w_tiles x chunk_h_tiles 4x4 tiles, each
 * 2, 4, 8 or 16 (8-64 pixels); keeps the warps per block. swr_batch_set_tuning sets square chunks.
 * The image never depends on the shape. */
swr_status swr_batch_set_chunk_shape(swr_batch b, uint32_t chunk_w_tiles, uint32_t chunk_h_tiles);
swr_status swr_batch_render(swr_batch b);
swr_status swr_batch_get_counters(swr_batch b, uint64_t out[SWR_NUM_COUNTERS]);
swr_status swr_batch_reset_counters(swr_batch b);
swr_status swr_batch_destroy(swr_batch b);

/* ---- Framebuffer (Rasterizer.h:10-78, ImageHelpers.cpp:109-147) ---- */
/* CreateFramebuffer(width, height, numLayers): width/height multiples of 4, at most 2896. */
swr_status swr_framebuffer_create(uint32_t width, uint32_t height, uint32_t num_layers, swr_framebuffer* out);
swr_status swr_framebuffer_destroy(swr_framebuffer fb);
swr_status swr_framebuffer_clear(swr_framebuffer fb, uint32_t color, float depth);       /* Clear */
swr_status swr_framebuffer_clear_layer(swr_framebuffer fb, uint32_t layer, uint32_t value); /* ClearLayer */
/* GetPixels(layer, dest, stride): de-tiles a layer into host memory (stride in pixels). Pinned
 * (page-locked) destinations are written by the de-tiling kernel directly over the host link. */
swr_status swr_framebuffer_get_pixels(swr_framebuffer fb, uint32_t layer, uint32_t* dest, uint32_t stride);
/* Device copy of a de-tiled layer (row-major, width*height words); no host synchronisation. */
swr_status swr_framebuffer_get_pixels_device(swr_framebuffer fb, uint32_t layer, uint32_t* dest_device);
/* Raw tiled layer storage (GetLayerData, Rasterizer.h:24-33), device pointer. Draws write layers 0
 * and 1 when they are next read, so the storage holds the draws made before this call: call it again
 * after later draws before reading or writing through the pointer. Writing through it must be
 * followed by swr_framebuffer_invalidate (which first writes any draws still pending). */
swr_status swr_framebuffer_layer_data(swr_framebuffer fb, uint32_t layer, void** out_device_ptr);
swr_status swr_framebuffer_invalidate(swr_framebuffer fb);
swr_status swr_framebuffer_size(swr_framebuffer fb, uint32_t* width, uint32_t* height, uint32_t* layer_stride,
                                uint32_t* num_layers);

/* ---- Meshlet building for imported meshes (Scene::ImportGltf, Scene.cpp:196-276) ----
 * One primitive's triangles grouped into Meshlet records of at most 64 vertices and 128
 * triangles, with bounds (sphere and normal cone). The reference uses meshoptimizer here; the
 * grouping of this library is its own (greedy growth over shared vertices in Morton order), so
 * the meshlets differ from the reference's for the same mesh. Per-vertex words are copied as
 * given: texcoords as packed half2 (glm::packHalf2x16), normal/tangent as
 * packUnorm4x8(oct(normal), oct(tangent)) (Scene.cpp:262-272). */
typedef struct {
    const float* positions;           /* x, y, z per vertex (mesh space) */
    const uint32_t* texcoords;        /* per vertex, or NULL */
    const uint32_t* normal_tangents;  /* per vertex, or NULL */
    const uint8_t* tangent_signs;     /* per vertex, 1 where the tangent's w < 0, or NULL */
    uint32_t num_vertices;
    const uint32_t* indices;          /* 3 per triangle */
    uint32_t num_triangles;
    uint32_t material_id;             /* UINT32_MAX: none */
    uint8_t alpha_cutoff;             /* Meshlet::AlphaCutoff */
} swr_mesh_desc;
/* An upper bound of the meshlets swr_build_meshlets makes for num_triangles triangles. */
uint32_t swr_meshlet_bound(uint32_t num_triangles);
/* Writes *count SWR_MESHLET_SIZE-byte records to host memory out (capacity records). */
swr_status swr_build_meshlets(const swr_mesh_desc* mesh, void* out, uint32_t capacity, uint32_t* count);

/* ---- Scene: Meshlet and Material pools (Scene.h:117-128) ---- */
swr_status swr_scene_create(swr_scene* out);
swr_status swr_scene_destroy(swr_scene s);
/* Copies count 1728-byte Meshlet records (Scene.h:15-30) from host memory to the device pool,
 * starting at record first (the pool grows as needed). */
swr_status swr_scene_upload_meshlets(swr_scene s, const void* meshlets, uint32_t first, uint32_t count);
swr_status swr_scene_set_materials(swr_scene s, const swr_material* materials, uint32_t count);
swr_status swr_scene_meshlet_count(swr_scene s, uint32_t* out);
/* The device copy of the records (ShadingContext::Meshlets, Shading.h:13), for user shaders
 * (swr/shader.cuh) that read the meshlets' attributes; valid until the next upload grows the pool. */
swr_status swr_scene_meshlets_device(swr_scene s, const void** out);

/* ---- Textures (Texture.h:314-636) ---- */
/* CreateTexture2D<format>(width, height, maxLevels, numLayers): power-of-two sizes. */
swr_status swr_texture_create(uint32_t format, uint32_t width, uint32_t height, uint32_t max_levels,
                              uint32_t num_layers, swr_texture* out);
swr_status swr_texture_destroy(swr_texture t);
/* SetPixels(pixels, stride, layer, 0): row-major host texels into mip 0 of a layer. */
swr_status swr_texture_set_pixels(swr_texture t, const uint32_t* pixels, uint32_t stride, uint32_t layer);
/* The same from row-major texels already in device memory (stream-ordered, no host sync). */
swr_status swr_texture_set_pixels_device(swr_texture t, const uint32_t* pixels_device, uint32_t stride, uint32_t layer);
swr_status swr_texture_generate_mips(swr_texture t);                                     /* GenerateMips */
/* Raw storage (Data[], MipOffsets[16], levels) for inspection; words = layer_stride*layers. */
swr_status swr_texture_info(swr_texture t, uint32_t* mip_levels, uint32_t* layer_stride, uint32_t mip_offsets[16]);
swr_status swr_texture_get_data(swr_texture t, uint32_t* dest, size_t words);
swr_status swr_texture_set_data(swr_texture t, const uint32_t* src, size_t words);

/* ---- Culling, Hi-Z, resolve ---- */
/* ShadingContext::CullMeshlets (Shading.cpp:775-869). bitmap_device receives one uint16 per 16
 * meshlets of [first, first+count) of the scene. depth_map (R32f Hi-Z from
 * swr_downsample_depth) may be NULL. If visible_count is not NULL the stream is synchronised and
 * the number of visible meshlets is returned. */
swr_status swr_cull_meshlets(swr_scene s, uint32_t first, uint32_t count, uint16_t* bitmap_device,
                             const float proj[16], const float view[16], const float model[16],
                             const float prev_view[16], float frame_width, float frame_height,
                             swr_texture depth_map, uint32_t* visible_count);
/* swr_cull_meshlets with options. SWR_CULL_BACKFACE_CONE (no counterpart in the reference, whose
 * records carry the cone but whose CullMeshlets never reads it) also drops meshlets that face away
 * from the camera as a whole: dot(normalize(ConeApex - eye), ConeAxis) >= ConeCutoff
 * (meshoptimizer's cone, Scene.h:18-19), tested with a margin so that it never removes a triangle
 * the rasterizer would draw; the vis-buffer is the same with and without it. Meshlets of
 * double-sided materials are kept; a projection that mirrors the screen or has no camera centre
 * (orthographic) turns the test off. */
#define SWR_CULL_BACKFACE_CONE 2u
swr_status swr_cull_meshlets_ex(swr_scene s, uint32_t first, uint32_t count, uint16_t* bitmap_device,
                                const float proj[16], const float view[16], const float model[16],
                                const float prev_view[16], float frame_width, float frame_height,
                                swr_texture depth_map, uint32_t* visible_count, uint32_t flags);
/* texutil::DownsampleDepth(Framebuffer&, Texture2D<R32f>&) (Texture.h:243, ImageHelpers.cpp:150-247). */
swr_status swr_downsample_depth(swr_framebuffer fb, swr_texture dest);
/* ShadingContext::Resolve(Rasterizer&, Framebuffer&) (Shading.cpp:658-690): shades the vis-buffer
 * into RGBA8 colour written over layer 0. The light-sprite overlay (691-731) is not drawn. */
swr_status swr_resolve(swr_rasterizer r, swr_framebuffer fb, const swr_shading_context* ctx);
/* ShadingContext::ResolveDebug(Rasterizer&, Framebuffer&, DebugLayer) (Shading.cpp:734-773): the
 * selected SWR_DEBUG_* layer as RGBA8 over layer 0: surface base colour, normal or metal/rough
 * (from the vis-buffer), hashed meshlet or triangle ids, or the OverdrawShader's counters through
 * the Turbo colormap; sky pixels (depth <= 0) get a grey/white checkerboard of 4x4 tiles. */
swr_status swr_resolve_debug(swr_rasterizer r, swr_framebuffer fb, const swr_shading_context* ctx, uint32_t layer);

/* ---- Image-based lighting precompute (Shading.cpp:35-219; the reference's frame driver never
 * calls it) ----
 * GenerateIrradianceMap: the cosine-weighted diffuse irradiance of an R11G11B10 octahedral
 * environment map (with at least 3 mips; the integral reads level 2) over 360 x 90 angle steps, into
 * level 0 of out (R11G11B10; the reference's is 64x64). */
swr_status swr_ibl_irradiance_map(swr_texture env, swr_texture out);
/* GenerateRadianceMap: every mip level L of out (R11G11B10 with mips; the reference's is 256x256,
 * 8 levels) prefiltered with 128 GGX importance samples at roughness L / (levels - 1) (Karis 2014). */
swr_status swr_ibl_radiance_map(swr_texture env, swr_texture out);
/* GenerateEnvBRDFLut: the split-sum scale and bias of the environment BRDF at NoV = u, roughness = v
 * (1024 importance samples) into level 0 of out (RG16f; the reference's is 128x128). */
swr_status swr_ibl_env_brdf_lut(swr_texture out);

/* ---- Learned texture decoder (no counterpart in the reference) ----
 * One model holds, per material, an FP16 latent pyramid of 8 channels (latent level k has the size
 * of texture level k+2, k < latent_levels) and an MLP of 11 inputs (8 latent channels, bias, two
 * level flags) -> 64 -> 64 -> 8 (GELU; 5384 parameters) decoding a texel's albedo RGB, normal XY,
 * metallic, roughness and AO. Texture levels 2..latent_levels+1 decode from their latent level's
 * texel, levels 1 and 0 from latent level 0 magnified 2x / 4x. It is trained on the device (BF16
 * tensor cores, FP32 accumulation, Adam) towards the plain sampler's texels, and
 * swr_resolve_neural decodes the texture levels it covers instead of sampling them; coarser
 * levels keep the plain sampler. Textures: RGBA8, 1 or 2 layers, width and height multiples of
 * 4 << (latent_levels-1), at least latent_levels+2 mips. The textures must outlive the model. */
typedef struct swr_neural_t* swr_neural;
enum { SWR_NEURAL_PARAMS = 5704 };   /* padded FP32 parameter block per material (see swr_neural_get_params) */
typedef struct {
    uint32_t num_materials, latent_levels;
    uint32_t texels_per_material;     /* latent texels over all levels */
    uint32_t level_offset[4], level_width[4], level_height[4];
    uint64_t latent_bytes;            /* FP16 latents of all materials */
    uint64_t weight_bytes;            /* inference weights of all materials (BF16 + FP32 biases) */
    uint64_t fallback_bytes;          /* texture levels >= latent_levels+2 kept for the plain sampler */
    uint64_t plain_bytes;             /* all levels of the plain textures */
} swr_neural_info;
typedef struct {
    uint32_t requests;                /* texels decoded by the network */
    uint32_t tiles;                   /* 128-texel tensor-core tiles */
    uint32_t level_texels[6];         /* decoded texels per texture level */
} swr_neural_stats;

/* textures[i] is the texture of material i (NULL: the material has none and is never decoded). */
swr_status swr_neural_create(const swr_texture* textures, uint32_t num_materials, uint32_t latent_levels, uint64_t seed,
                             swr_neural* out);
swr_status swr_neural_destroy(swr_neural n);
swr_status swr_neural_get_info(swr_neural n, swr_neural_info* info);
/* `steps` Adam steps (lr, beta1 0.9, beta2 0.999, eps 1e-8). Each step draws batch samples spread
 * evenly over materials_per_step materials taken round-robin; a sample is a texel and its target
 * the plain texel. Texture level l is drawn with weight 2^(level_weighting * (latent_levels+1-l)):
 * 2 = proportional to the level's texel count, 1 = to its edge, 0 = uniform. batch /
 * materials_per_step must be a multiple of 128. mean_loss (optional, synchronises) receives the
 * mean squared error per output of the last step. */
swr_status swr_neural_train(swr_neural n, uint32_t steps, uint32_t batch, uint32_t materials_per_step,
                            uint32_t level_weighting, float learning_rate, float* mean_loss);
/* Gradients for explicit samples of one material without updating anything: samples_device holds
 * count (multiple of 128) packed texels level<<28 | y<<14 | x. param_grad (host, SWR_NEURAL_PARAMS)
 * receives the parameter gradient of the loss sum over 128-sample tiles of mean squared error,
 * latent_grad (host, texels_per_material*8, may be NULL) the latent gradient, loss (may be NULL)
 * the summed squared error. */
swr_status swr_neural_gradients(swr_neural n, uint32_t material, const uint32_t* samples_device, uint32_t count,
                                float* param_grad, float* latent_grad, float* loss);
/* FP32 parameters / latents (texels_per_material*8 floats, [texel][channel]) of one material. */
swr_status swr_neural_get_params(swr_neural n, uint32_t material, float* params);
swr_status swr_neural_set_params(swr_neural n, uint32_t material, const float* params);
swr_status swr_neural_get_latents(swr_neural n, uint32_t material, float* latents);
swr_status swr_neural_set_latents(swr_neural n, uint32_t material, const float* latents);
/* Training checkpoint: the model's whole training state (per-material Adam step counts, the
 * sampler's seed and step counter, FP32 parameters and latents with their Adam moments) as one
 * versioned blob, so training can stop and resume on the same trajectory. swr_neural_save with
 * dst NULL returns the size only; swr_neural_load takes a blob of a model of the same shape
 * (materials, latent levels, texture sizes) and rebuilds the inference weights and latents. */
swr_status swr_neural_save(swr_neural n, void* dst, size_t capacity, size_t* size);
swr_status swr_neural_load(swr_neural n, const void* src, size_t size);
/* Decodes count texels (packed as for swr_neural_gradients) of one material into out_device
 * (2 words per texel: layer-0 RGBA8 with AO in alpha, layer-1 RGBA8). */
swr_status swr_neural_decode(swr_neural n, uint32_t material, const uint32_t* texels_device, uint32_t count,
                             uint32_t* out_device);
/* Time limit of each bounded device-side wait of the model's kernels (copy and tensor-core
 * completion; default 1 s, 1 ns to 60 s). A wait that reaches it makes the call return
 * SWR_ETIMEOUT; the kernel first lets the operation it waited for land, then frees its TMEM. */
swr_status swr_neural_set_wait_limit(swr_neural n, uint64_t limit_ns);
/* Exercises the bounded-wait path on the device: one CTA allocates TMEM, arms an mbarrier for a
 * 16-byte copy that is never issued and waits at most limit_ns (1 ns to 1 s); the wait gives up,
 * the CTA frees its TMEM and exits, and the call returns SWR_ETIMEOUT. The context stays usable. */
swr_status swr_selftest_bounded_wait(uint64_t limit_ns);
/* swr_resolve with the texture levels below latent_levels decoded by the model (the scene's
 * material i must use the model's texture i); stats may be NULL (else the stream is synchronised). */
swr_status swr_resolve_neural(swr_rasterizer r, swr_framebuffer fb, const swr_shading_context* ctx, swr_neural n,
                              swr_neural_stats* stats);

#ifdef __cplusplus
}
#endif
#endif /* SWR_GB300_H */
