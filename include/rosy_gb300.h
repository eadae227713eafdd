/*
 * rosy_gb300 — C ABI of the GB300 (sm_103a) frame renderer that replaces Rosy's
 * shadow depth pass + mesh forward pass.
 *
 * The reference interface is `rosy::graphics` (src/Engine/Graphics.h:11-21) and
 * the inner seams of its Vulkan backend `graphics_device`:
 *   set_asset           src/Engine/Graphics.cpp:3525   -> rz_set_asset
 *   set_graphic_objects src/Engine/Graphics.cpp:4691   -> rz_set_objects
 *   (go_update upload)  src/Engine/Graphics.cpp:5120-5138 -> rz_update_objects
 *   update              src/Engine/Graphics.cpp:6016   -> rz_update
 *   render              src/Engine/Graphics.cpp:4934   -> rz_render
 *   init / deinit       src/Engine/Graphics.cpp:6119-6170, 6217-6228 -> rz_create / rz_destroy
 *   resize              src/Engine/Graphics.cpp:6200   -> rz_resize
 *   (DRAW DEBUG)        src/Engine/Graphics.cpp:5694-5738 -> rz_set_debug_objects
 *
 * Windowing, swapchain and imgui are not part of this path: the
 * frame is rendered into headless device buffers (RGBA8 sRGB colour, D32 depth,
 * a 64-bit visibility buffer and the D32 shadow map) that the caller reads with
 * rz_get_frame (device pointers) or rz_read_frame (copy to host memory).
 *
 * Every entry point returns an rz_result (the numeric values 0..15 are those of
 * rosy::result, src/Engine/Types.h:13-31). No entry point throws. One context
 * is used by one host thread at a time; there is no global mutable state except
 * the CUDA runtime's own.
 */
#ifndef ROSY_GB300_H
#define ROSY_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RZ_ABI_VERSION 2u

/* Opaque renderer context (one per host thread). */
struct rz_ctx;
typedef struct rz_ctx rz_ctx;
#define RZ_INVALID_INDEX 0xFFFFFFFFu /* UINT32_MAX == absent, src/shaders/data.slang:135-137 */

typedef enum rz_result {
    RZ_OK = 0,
    RZ_STATE_CHANGED = 1,
    RZ_ERROR = 2,
    RZ_INVALID_ARGUMENT = 3,
    RZ_ALLOCATION_FAILURE = 4,
    RZ_GRAPHICS_INIT_FAILURE = 5,
    RZ_GRAPHICS_FRAME_FAILURE = 6,
    RZ_GRAPHICS_SWAPCHAIN_FAILURE = 7,
    RZ_OPEN_FAILED = 8,
    RZ_WRITE_FAILED = 9,
    RZ_COPY_FAILED = 10,
    RZ_READ_FAILED = 11,
    RZ_CREATE_FAILED = 12,
    RZ_UPDATE_FAILED = 13,
    RZ_OVERFLOW = 14,
    RZ_INVALID_STATE = 15,
    /* Added by this library: rz_sync gave up waiting (the reference waits on a
     * fence with a timeout at src/Engine/Graphics.cpp:4940). */
    RZ_TIMEOUT = 16
} rz_result;

/* One vertex: rosy_asset::position (src/Asset/Asset.h:92-99), read by the shaders
 * as BasicInputVertex (src/shaders/data.slang:24-30). 64 bytes, tightly packed. */
typedef struct rz_vertex {
    float position[3];
    float normal[3];
    float tangent[4];
    float color[4];
    float uv[2];
} rz_vertex;

/* A mesh: its vertices and mesh-local u32 indices (rosy_asset::mesh,
 * src/Asset/Asset.h:101-106). The renderer concatenates all meshes the way
 * set_asset does (src/Engine/Graphics.cpp:4310-4334); indices stay mesh-local. */
typedef struct rz_mesh {
    const rz_vertex* positions;
    uint32_t position_count;
    uint32_t index_count;
    const uint32_t* indices;
} rz_mesh;

/* Asset material (rosy_asset::material, src/Asset/Asset.h:27-46). rz_set_asset
 * packs it into the 64-byte gpu_material (src/Engine/Graphics.cpp:345-360) with
 * the index mapping of src/Engine/Graphics.cpp:4071-4150: an image index that
 * is out of range becomes "absent"; a sampler index that is out of range (or
 * given for an absent image) selects the default sampler. */
typedef struct rz_material {
    float base_color_factor[4];
    float metallic_factor;
    float roughness_factor;
    float alpha_cutoff;
    uint32_t alpha_mode;     /* 0 opaque, 1 mask, 2 blend (any non-zero => blended list) */
    uint32_t double_sided;   /* carried, unused by the path (as in the reference) */
    uint32_t color_image_index;
    uint32_t color_sampler_index;
    uint32_t normal_image_index;
    uint32_t normal_sampler_index;
    uint32_t metallic_image_index;
    uint32_t metallic_sampler_index;
    uint32_t mixmap_image_index;
    uint32_t mixmap_sampler_index;
} rz_material;

/* Asset sampler (rosy_asset::sampler, src/Asset/Asset.h:48-54). Filter codes
 * 0..2 => nearest, anything else => linear (src/Engine/Graphics.cpp:250-262);
 * wrap codes 0 clamp-to-edge, 1 mirrored repeat, else repeat (264-278). The
 * mip mode of asset samplers is linear (src/Engine/Graphics.cpp:3996-4014). */
typedef struct rz_sampler {
    uint16_t min_filter;
    uint16_t mag_filter;
    uint16_t wrap_s;
    uint16_t wrap_t;
} rz_sampler;

/* Image types (src/Asset/Asset.h:108-112). Colour, metallic-roughness and mixmap
 * images are sampled as sRGB, normal maps as UNORM (Graphics.cpp:3632-3647). */
#define RZ_IMAGE_COLOR 0u
#define RZ_IMAGE_NORMAL_MAP 1u
#define RZ_IMAGE_METALLIC_ROUGHNESS 2u
#define RZ_IMAGE_MIXMAP 3u

/* Texel formats of rz_texture.format. */
#define RZ_TEXELS_RGBA8 0u /* 4 bytes per texel */
#define RZ_TEXELS_BC7 1u   /* BC7 blocks: what the reference's .dds images hold */

/* A texture of `levels` mip levels, concatenated level 0 first; level l is
 * max(1, width>>l) x max(1, height>>l) texels, rows top to bottom.
 * RZ_TEXELS_RGBA8: 4 bytes per texel. RZ_TEXELS_BC7: 16-byte BC7 blocks, level
 * l is max(1, (w_l+3)/4) x max(1, (h_l+3)/4) blocks in rows top to bottom, the
 * layout of a .dds file's mips (src/libs/dds.hpp:550-566) — the reference
 * uploads these as VK_FORMAT_BC7_{SRGB,UNORM}_BLOCK images
 * (src/Engine/Graphics.cpp:3632-3647); rz_set_asset decodes them on the
 * device into RGBA8 (rz_bc7_decode), which the shading samples. */
typedef struct rz_texture {
    uint32_t width;
    uint32_t height;
    uint32_t levels;
    uint32_t image_type;
    const void* texels;
    uint32_t format;   /* RZ_TEXELS_RGBA8 (0) or RZ_TEXELS_BC7 */
    uint32_t reserved; /* 0 */
} rz_texture;

/* Per-object transforms: graphic_object_data (src/Engine/Graphics.cpp:422-427),
 * BasicGraphicsData in the shaders (src/shaders/data.slang:32-36). Column-major
 * (glm) matrices, 164 bytes. */
typedef struct rz_object {
    float transform[16];
    float to_object_space_transform[16];
    float normal_transform[9];
} rz_object;

/* One draw: rosy::surface_graphics_data (src/Engine/Types.h:39-48), with u32 in
 * place of size_t. Surfaces are given in scene order; the shadow list is all of
 * them, the opaque list those with blended == 0, the blended list the others
 * (src/Engine/Graphics.cpp:4715-4735). */
typedef struct rz_surface {
    uint32_t mesh_index;
    uint32_t graphic_objects_offset;
    uint32_t graphics_object_index;
    uint32_t material_index; /* RZ_INVALID_INDEX => no material */
    uint32_t index_count;
    uint32_t start_index;
    uint32_t blended;
} rz_surface;

/* Scene constants: byte-identical to gpu_scene_data (src/Engine/Graphics.cpp:
 * 281-306) / SceneData (src/shaders/data.slang:45-70), 408 bytes. */
typedef struct rz_scene_data {
    float view[16];
    float proj[16];
    float view_projection[16];
    float shadow_projection_near[16];
    float sun_position[4];
    float camera_position[4];
    float ambient_color[4];
    float sunlight_color[4];
    uint32_t flip_lights[4];
    uint32_t flip_tangents[4];
    float draw_extent[2];
    float light_intensity;
    uint32_t csm_index_sampler; /* ignored: the shadow map is the one this frame rendered */
    uint32_t csm_index_near;    /* ignored */
    uint32_t fragment_output;
    uint32_t light_enabled;
    uint32_t tangent_space_enabled;
    uint32_t shadows_enabled;
    uint32_t normal_maps_enabled;
    uint32_t inverse_bnt;
    uint32_t ignore_asset_tangent_sign;
    uint32_t ensure_orthogonal_bitangent;
    uint32_t brdf_lighting_enabled;
} rz_scene_data;

/* PCF kernels for the shadow lookup. */
#define RZ_PCF_5TAP 0u /* the reference's pattern, src/shaders/pcf.slang:1-11 */
#define RZ_PCF_3X3 1u  /* 3x3 grid, one texel apart (option) */

/* Fixed-function state that the reference takes from read_level_state rather
 * than from gpu_scene_data: draw_config (src/Engine/Graphics.cpp:5010-5015) and
 * the light's depth bias (5222-5231). Defaults: src/Engine/Level.cpp:1246-1255. */
typedef struct rz_draw_config {
    uint32_t cull_enabled;                  /* 1 => cull FRONT faces */
    uint32_t reverse_winding_order_enabled; /* 1 => front face is counter-clockwise */
    uint32_t depth_bias_enabled;            /* shadow pass only */
    float depth_bias_constant;
    float depth_bias_clamp;
    float depth_bias_slope_factor;
    uint32_t pcf_mode;                      /* RZ_PCF_* */
    uint32_t shadow_cascades;               /* 0 or 1: the reference's single "near" map; 2..4: nested
                                               cascades (see below) */
} rz_draw_config;

/* Shadow cascades (the reference allocates three layers and renders only the
 * "near" one, src/Engine/Graphics.cpp:2545, 5203). With shadow_cascades = n > 1
 * the shadow pass renders n maps of shadow_map_size^2, stored one after the
 * other: cascade k uses shadowProjNear with clip x and y scaled by 2^-k (the
 * light's orthographic extent times 2^k). A fragment uses the finest cascade k
 * whose coordinates (csm.xy - 0.5) * 2^-k + 0.5 (csm.xy itself for k = 0) lie in
 * [2 / size, 1 - 2 / size], else the coarsest. */

/* Context creation: the headless analogue of graphics::init's config
 * (src/Engine/Types.h:33-37). */
typedef struct rz_config {
    uint32_t width;            /* colour/depth extent */
    uint32_t height;
    uint32_t shadow_map_size;  /* square D32 shadow map (the reference uses 4096, Graphics.cpp:2524) */
    uint32_t samples;          /* rasterisation samples per pixel: 1 */
    int32_t device;            /* CUDA device ordinal */
    uint32_t queue_chunks;     /* raster work-queue depth per pass, in chunks of 32
                                  8x4-pixel stamps; 0 = sized from the scene. A frame
                                  that needs more reports RZ_OVERFLOW and the queue
                                  grows for the next frame. */
    uint32_t reserved[2];
} rz_config;

/* Device pointers of the last rendered frame. colour: RGBA8, sRGB-encoded RGB
 * (the B8G8R8A8_SRGB swapchain blit of src/Engine/Graphics.cpp:5845-5879, with
 * R in byte 0); depth: f32 reverse-Z (cleared to 0); visibility: per pixel
 * (depth_bits << 32) | (triangle_id + 1), 0 = background; shadow map: f32. */
typedef struct rz_frame_out {
    void* color_rgba8;
    void* depth_f32;
    void* visibility_u64;
    void* shadow_map_f32;
    uint32_t width;
    uint32_t height;
    uint32_t shadow_map_size;
    uint32_t triangle_id_base; /* ids in the visibility buffer are triangle_id_base + (index of the
                                  triangle in the view's opaque list) + 1; 0 for view 0 */
} rz_frame_out;

/* Counters of the last frame (graphics_stats, src/Engine/DebugUI.h:7-13). */
typedef struct rz_stats {
    uint32_t draw_call_count;
    uint32_t triangle_count;
    uint32_t shadow_setup_records;  /* raster setup records written, shadow pass */
    uint32_t camera_setup_records;  /* raster setup records written, camera pass */
    uint64_t shadow_stamps;         /* 8x4-pixel stamps rasterised, shadow pass */
    uint64_t camera_stamps;         /* 8x4-pixel stamps rasterised, camera pass */
    uint32_t error_flags;           /* device-side error bits of the last frame */
    uint32_t kernel_launches;       /* kernels the last rz_render launched (counted as its frame was built) */
} rz_stats;

/* graphics::init (src/Engine/Graphics.h:17): creates the CUDA stream and the
 * frame buffers on cfg->device. */
int rz_create(struct rz_ctx** out_ctx, const rz_config* cfg);

/* graphics::deinit (src/Engine/Graphics.h:21). Accepts NULL. */
void rz_destroy(struct rz_ctx* ctx);

/* graphics::resize (src/Engine/Graphics.h:20): new colour/depth extent. */
int rz_resize(struct rz_ctx* ctx, uint32_t width, uint32_t height);

/* graphics_device::set_asset (src/Engine/Graphics.cpp:3525): copies meshes,
 * materials, textures and samplers into device memory. Blocks until the copy is
 * done (the reference waits on an immediate-submit fence). */
int rz_set_asset(struct rz_ctx* ctx,
                 const rz_mesh* meshes, uint32_t mesh_count,
                 const rz_material* materials, uint32_t material_count,
                 const rz_texture* textures, uint32_t texture_count,
                 const rz_sampler* samplers, uint32_t sampler_count);

/* graphics_device::set_graphic_objects (src/Engine/Graphics.cpp:4691): the
 * object transforms and the surface list in scene order. Rejects an empty
 * scene (RZ_INVALID_ARGUMENT, as 4693-4697), out-of-range mesh/object/material
 * indices or index ranges, and non-blended surfaces whose material has a
 * non-zero alpha_mode (the opaque list never holds those in the engine,
 * src/Engine/Level.cpp:1056-1061, and this renderer's visibility pass relies on it). */
int rz_set_objects(struct rz_ctx* ctx,
                   const rz_object* objects, uint32_t object_count,
                   const rz_surface* surfaces, uint32_t surface_count);

/* Mob transform update (src/Engine/Graphics.cpp:5120-5138): overwrite
 * objects [offset, offset+count) before the next frame. Staged in pinned memory
 * and copied to the device by rz_render, like the scene constants. */
int rz_update_objects(struct rz_ctx* ctx, uint32_t offset, const rz_object* objects, uint32_t count);

/* Fixed-function state of the next frames (see rz_draw_config). */
int rz_set_draw_config(struct rz_ctx* ctx, const rz_draw_config* cfg);

/* graphics_device::update (src/Engine/Graphics.cpp:6016): the scene constants
 * of the next frame. The 408 bytes are staged in pinned memory and copied to the
 * device by rz_render, before the frame reads them (into the buffer of the
 * frame's target set, on an upload stream, overlapping the frame before), so a
 * frame always uses its own constants (the reference writes the next frame's
 * buffer, 5064-5065; that one-frame lag is not reproduced). */
int rz_update(struct rz_ctx* ctx, const rz_scene_data* scene);

/* graphics_device::render (src/Engine/Graphics.cpp:4934): enqueues the shadow
 * pass, the camera pass and the shading pass on the context's stream and
 * returns without waiting. Errors found on the device (an overflowing
 * raster work queue, for instance) are reported by the next rz_sync. */
int rz_render(struct rz_ctx* ctx);

/* Waits for the stream, at most timeout_ms milliseconds (0 = no limit).
 * Returns RZ_TIMEOUT if the frame is still running, RZ_OVERFLOW or
 * RZ_GRAPHICS_FRAME_FAILURE if the device flagged an error in a frame. */
int rz_sync(struct rz_ctx* ctx, uint32_t timeout_ms);

/* Device pointers of the buffers of the frame rendered last (valid until the
 * next rz_resize/rz_destroy). The colour and depth targets are double-buffered:
 * frames alternate between two target sets, so color_rgba8 and depth_f32
 * change from one frame to the next; take them after each frame. */
int rz_get_frame(struct rz_ctx* ctx, rz_frame_out* out);

/* Enqueues device-to-host copies of the colour (width*height*4 bytes) and/or
 * depth (width*height*4 bytes) images of the frame rendered last; NULL skips
 * one. They are copied straight from the frame's target set on a copy stream of
 * the context, after the frame, while the next frame renders into the other
 * set (the reference keeps several frames in flight, src/Engine/Graphics.cpp:177,
 * and presents asynchronously); the frame after that, which renders into the
 * same set again, waits for the copies. The host buffers are complete after
 * rz_sync, or after rz_read_sync. */
int rz_read_frame(struct rz_ctx* ctx, void* color_host, size_t color_bytes,
                  void* depth_host, size_t depth_bytes);

/* Waits until at most `pending` (0 or 1) of the read-backs queued by
 * rz_read_frame are still travelling: 1 waits for all but the newest, so a
 * caller with two host buffers may refill the older one. RZ_TIMEOUT after
 * timeout_ms (0: no limit). Library addition (the reference presents to a
 * swapchain instead). */
int rz_read_sync(struct rz_ctx* ctx, uint32_t pending, uint32_t timeout_ms);

/* Counters of the last completed frame (call after rz_sync). */
int rz_get_stats(struct rz_ctx* ctx, rz_stats* out);

/* Batched views. A context holds scenes and views: scene 0 is the one
 * rz_set_asset / rz_set_objects define, rz_add_scene appends more (each with its
 * own asset, objects and surfaces), and rz_set_views replaces the view list
 * (initially one view of scene 0 with rz_config's extent). rz_render renders
 * every view: each stage of the frame is one launch over all views, captured in
 * one CUDA graph. This has no counterpart in the reference, which renders one
 * camera per frame; it is the batching of many views of uneven size. */
typedef struct rz_view {
    uint32_t scene;            /* scene index */
    uint32_t width;            /* colour/depth extent */
    uint32_t height;
    uint32_t shadow_map_size;  /* the view's own square shadow map */
    rz_draw_config draw_config;
} rz_view;

/* Appends a scene (asset + objects + surfaces, as rz_set_asset + rz_set_objects
 * take them) and returns its index in *scene_index. */
int rz_add_scene(struct rz_ctx* ctx,
                 const rz_mesh* meshes, uint32_t mesh_count,
                 const rz_material* materials, uint32_t material_count,
                 const rz_texture* textures, uint32_t texture_count,
                 const rz_sampler* samplers, uint32_t sampler_count,
                 const rz_object* objects, uint32_t object_count,
                 const rz_surface* surfaces, uint32_t surface_count,
                 uint32_t* scene_index);

/* Replaces the list of views rendered by rz_render. Views keep the scene
 * constants already given to the same index. */
int rz_set_views(struct rz_ctx* ctx, const rz_view* views, uint32_t count);

/* Scene constants (gpu_scene_data) of one view for the next frame; rz_update is view 0. */
int rz_update_view(struct rz_ctx* ctx, uint32_t view, const rz_scene_data* scene);

/* Device pointers of one view's frame buffers (rz_get_frame is view 0). */
int rz_get_view_frame(struct rz_ctx* ctx, uint32_t view, rz_frame_out* out);

/* Raster work distribution and batching (see rz_autotune). */
typedef struct rz_tuning {
    uint32_t chunk_stamps;  /* stamps (8x4 pixels) per raster work chunk, the unit a warp takes: 8..256 */
    uint32_t small_extent;  /* triangles up to this extent (pixels, each way) are rasterised one per lane: 1..16 */
    uint32_t queue_chunks;  /* raster work-queue depth per pass in chunks (0 = sized from the scene) */
    uint32_t batched;       /* 1: each stage is one launch over all views; 0: per-view sequential launches */
} rz_tuning;

/* Sets / reads the tuning of the following frames. */
int rz_set_tuning(struct rz_ctx* ctx, const rz_tuning* tuning);
int rz_get_tuning(struct rz_ctx* ctx, rz_tuning* tuning);

/* Diagnostic: the bound of each look-back wait of the blended list's ordered
 * setup (iterations of about 32 ns) for the following frames; 0 restores the
 * default (2^22). A wait that runs out flags the frame (rz_sync returns
 * RZ_GRAPHICS_FRAME_FAILURE) and the blended list is left out of that frame.
 * This library addition has no counterpart in the reference, whose ordering
 * comes from the hardware; tests use it to make the waits run out. */
int rz_set_wait_limit(struct rz_ctx* ctx, uint32_t lookback_spins);

/* Autotuner: renders the current views `frames` times (after one warm-up
 * frame) with every candidate of chunk_stamps in {16, 32, 64} x small_extent in
 * {4, 8, 12}, measures device time with CUDA events, applies the fastest and
 * returns it; `ms` (optional) receives the mean frame time of each candidate in
 * that order. The views need their scene constants (rz_update_view) first. */
int rz_autotune(struct rz_ctx* ctx, uint32_t frames, rz_tuning* chosen, float* ms, uint32_t capacity);

/* Frame stages timed by rz_get_stage_times (CUDA events on the context's stream). */
#define RZ_STAGE_SHADOW_CLEAR 0u  /* shadow-map clear */
#define RZ_STAGE_SHADOW_SETUP 1u  /* shadow draw matrices + triangle setup */
#define RZ_STAGE_SHADOW_RASTER 2u /* shadow raster */
#define RZ_STAGE_CAMERA_CLEAR 3u  /* visibility clear + camera draw constants */
#define RZ_STAGE_CAMERA_SETUP 4u  /* camera triangle setup */
#define RZ_STAGE_CAMERA_RASTER 5u /* camera raster (visibility buffer) */
#define RZ_STAGE_SHADE 6u         /* deferred shading + sRGB encode */
#define RZ_STAGE_COUNT 7u

/* Enables (1) or disables (0) per-stage event timing of the following frames.
 * This is a diagnostic switch: it adds event records between the stages. */
int rz_set_stage_timing(struct rz_ctx* ctx, uint32_t enable);

/* Milliseconds spent in each stage of the last completed frame (call after
 * rz_sync). Writes min(capacity, RZ_STAGE_COUNT) values and the count. */
int rz_get_stage_times(struct rz_ctx* ctx, float* ms, uint32_t capacity, uint32_t* count);

/* Shadow depth pass for callers that cannot allocate device memory while they
 * run (engines that own every device allocation through their own allocator or
 * a fixed budget, frame loops that must not call cudaMalloc/cudaFree). This entry
 * point has no counterpart in the reference. It rasterises one draw into a D32
 * depth target exactly as rz_render's shadow pass does (clear to 0, MVP =
 * projection * world, clipping, culling, depth bias, GREATER_OR_EQUAL), using
 * only a fixed scratch array compiled into the library (about 3.3 MiB per
 * device, held until the process exits); it allocates nothing.
 *   positions: device array of vertex_count float4 (x, y, z, unused)
 *   indices:   device array of index_count u32 (a multiple of 3, at most
 *              3 * 16384: larger draws return RZ_INVALID_ARGUMENT)
 *   projection, world: host column-major 4x4 matrices
 *   depth_out: device array of width * height floats, overwritten
 * Runs on `stream` (a cudaStream_t, NULL = default stream) and waits for it.
 * Returns RZ_OVERFLOW (the depth target is then incomplete) if the coverage
 * needs more than the fixed work queue (65,536 chunks of 32 8x4-pixel stamps),
 * or if clipping fans the triangles out into more than 24,576 setup records.
 * Calls share the scratch array: calls that overlap on the GPU race and must be
 * serialised by the caller. The first call on a device looks up the array's
 * device address (and, with lazy module loading, may load the module that
 * holds it); make it before any stream capture starts on that device, as a
 * warm-up call at start-up where a frame loop must not allocate. */
int rz_shadow_depth_static(const void* positions, uint32_t vertex_count, const uint32_t* indices,
                           uint32_t index_count, const float projection[16], const float world[16],
                           const rz_draw_config* cfg, uint32_t width, uint32_t height, float* depth_out,
                           void* stream);

/* The context's cudaStream_t, for callers that time or chain work on it: work
 * enqueued on it after rz_render runs after that frame's kernels. (The context
 * also uses streams of its own for the frame's concurrent branches, the uploads
 * of the per-frame inputs and the read-backs; they are joined to this stream or
 * waited for by rz_sync.) */
void* rz_get_stream(struct rz_ctx* ctx);

/* Human-readable message of the last failing call on this context. */
const char* rz_last_error(struct rz_ctx* ctx);

/* RZ_ABI_VERSION of the loaded library. */
uint32_t rz_abi_version(void);

/* ---- .rsy asset files ------------------------------------------------------
 * Reader for the asset format of rosy_asset::asset (src/Asset/Asset.h:10-148,
 * read by src/Asset/Asset.cpp:409-848), so that Rosy's own assets feed
 * rz_set_asset / rz_set_objects. rz_rsy_read replaces asset::read (fopen_s and
 * all): RZ_OPEN_FAILED if the file cannot be opened, RZ_READ_FAILED if it is
 * truncated, has the wrong magic, version or endianness, or a count larger than
 * the file. Images are named, not embedded (the engine loads them as separate
 * files), so textures are supplied by the caller. */
struct rz_rsy;
typedef struct rz_rsy rz_rsy;

typedef struct rz_rsy_info {
    uint32_t mesh_count;
    uint32_t material_count;
    uint32_t sampler_count;
    uint32_t image_count;
    uint32_t node_count;
    uint32_t scene_count;
    uint32_t root_scene;
    uint32_t object_count;        /* graphics objects of the root scene (statics first, then mobs) */
    uint32_t surface_count;       /* surfaces of those objects, in scene order */
    uint32_t static_object_count; /* objects before the first mob */
    float coordinate_system[16];  /* the asset's coordinate system (column-major) */
} rz_rsy_info;

int rz_rsy_read(const char* path, struct rz_rsy** out);
void rz_rsy_free(struct rz_rsy* asset);
int rz_rsy_get_info(const struct rz_rsy* asset, rz_rsy_info* out);

/* Meshes as rz_mesh records whose pointers stay valid until rz_rsy_free;
 * materials and samplers copied out. RZ_OVERFLOW if capacity is too small. */
int rz_rsy_get_meshes(const struct rz_rsy* asset, rz_mesh* out, uint32_t capacity);
int rz_rsy_get_materials(const struct rz_rsy* asset, rz_material* out, uint32_t capacity);
int rz_rsy_get_samplers(const struct rz_rsy* asset, rz_sampler* out, uint32_t capacity);

/* Type and name of image `index` (name NUL-terminated, truncated to name_capacity - 1). */
int rz_rsy_get_image(const struct rz_rsy* asset, uint32_t index, uint32_t* image_type, char* name,
                     uint32_t name_capacity, uint32_t* name_length);

/* The root scene flattened as the level flattens a new asset
 * (src/Engine/Level.cpp:922-1160, node transforms src/Engine/Node.cpp:96-103):
 * one graphics object per node with a mesh, breadth first, static nodes first
 * and nodes under a node named "mobs" after them; one surface per mesh surface.
 * RZ_INVALID_ARGUMENT if the root scene or a node index is out of range. */
int rz_rsy_get_scene(const struct rz_rsy* asset, rz_object* objects, uint32_t object_capacity, rz_surface* surfaces,
                     uint32_t surface_capacity);

/* ---- .dds images and BC7 -----------------------------------------------------
 * Reader for the .dds files the engine loads for every asset image
 * (src/Engine/Graphics.cpp:3605-3647 through dds::readFile / dds::readImage,
 * src/libs/dds.hpp:409-596). rz_dds_read replaces dds::readFile and
 * rz_dds_parse dds::readImage, with the same checks and one more: the file
 * must hold every mip level its header announces (dds::readImage points its
 * mip spans past the end of a short file). Results: RZ_OPEN_FAILED (file cannot
 * be opened); RZ_READ_FAILED (shorter than the magic and header, wrong magic:
 * ReadResult::Failure; a DX10 file shorter than 148 bytes, a zero width or
 * height, or mips past the end of the file: ReadResult::InvalidSize);
 * RZ_INVALID_ARGUMENT (a format other than BC7, or an array of more than one
 * image: ReadResult::UnsupportedFormat — the engine uploads every image as BC7,
 * Graphics.cpp:3632-3647). */
struct rz_dds;
typedef struct rz_dds rz_dds;

typedef struct rz_dds_info {
    uint32_t width;
    uint32_t height;
    uint32_t levels;         /* max(1, mipmapCount), as dds::Image::numMips */
    uint32_t dxgi_format;    /* the DX10 header's format: 97 BC7_TYPELESS, 98 BC7_UNORM, 99 BC7_UNORM_SRGB */
    uint32_t supports_alpha; /* DDPF_ALPHAPIXELS of the pixel format (dds::Image::supportsAlpha) */
    uint32_t reserved;
    uint64_t data_bytes;     /* bytes of all levels */
    const void* data;        /* the levels' BC7 blocks, level 0 first; valid until rz_dds_free */
} rz_dds_info;

int rz_dds_read(const char* path, struct rz_dds** out);
int rz_dds_parse(const void* bytes, uint64_t size, struct rz_dds** out); /* copies the bytes */
void rz_dds_free(struct rz_dds* image);
int rz_dds_get_info(const struct rz_dds* image, rz_dds_info* out);

/* Decodes one image of BC7 blocks (device memory, max(1,(w+3)/4) x
 * max(1,(h+3)/4) blocks in rows) into width x height RGBA8 texels (device
 * memory, rows of width * 4 bytes), enqueued on `stream` (a cudaStream_t, NULL =
 * default stream). Decoding follows the
 * BC7 format exactly (every texel equals what the GPU's texture unit decodes
 * from the same block; the reserved mode decodes to 0,0,0,0). */
int rz_bc7_decode(const void* blocks, uint32_t width, uint32_t height, void* rgba8, void* stream);

/* The same image decoded by the GPU's texture unit (a BC7 CUDA array sampled
 * at texel centres), synchronously: the hardware decoder the reference's
 * VK_FORMAT_BC7_*_BLOCK images go through, for checking rz_bc7_decode. Width
 * and height must be multiples of 4. */
int rz_bc7_decode_texture_unit(const void* blocks, uint32_t width, uint32_t height, void* rgba8);

/* ---- G-buffer ------------------------------------------------------------
 * Inputs of the learned upsampler. The reference has no G-buffer (it shades
 * forward into its draw image); these are extra outputs of the same shading
 * pass. With rz_set_gbuffer(ctx, 1) every following frame also writes, per
 * pixel of every view: the albedo (the sampled base colour of fragmentMain,
 * rounded to f16 and sRGB-encoded; alpha = 255 where a triangle covers the
 * pixel, else 0) and the interpolated world-space normal, octahedral-encoded as
 * two f16 (x in the low half). With 4x multisampling both are averaged over the
 * pixel's samples (the normal renormalised) and the albedo's alpha is the
 * covered fraction of the samples.
 * Single-sampled frames also get the sub-pixel sources of the upsampler's x2
 * base, a u16 per pixel: for each point k = 2 * (y half) + (x half) at
 * (x + 0.25 / 0.75, y + 0.25 / 0.75) that a full-resolution pixel samples, the
 * front-most of the triangles visible at the 3x3 neighbourhood's pixel centres
 * (float edge functions, the depth plane through the vertices' z / w), and
 * bit 4k + s set when bilinear source s of that pixel (0 own, 1 horizontal,
 * 2 vertical, 3 diagonal neighbour, clamped at the borders) shows the same
 * triangle (or background); 0xFFFF where the neighbourhood shows one triangle.
 * The upsampler renormalises the bilinear weights over the marked sources.
 * NULL (4x multisampling, or a caller's own G-buffer) means plain bilinear. */
typedef struct rz_gbuffer {
    const void* color_rgba8;      /* width*height RGBA8 sRGB (the frame's colour) */
    const void* depth_f32;        /* width*height f32 (reverse-Z, 0 = background) */
    const void* albedo_rgba8;     /* width*height RGBA8 */
    const void* normal_oct_f16x2; /* width*height u32 */
    const void* sources_u16;      /* width*height u16 sub-pixel sources, or NULL */
    uint32_t width;
    uint32_t height;
} rz_gbuffer;

int rz_set_gbuffer(struct rz_ctx* ctx, uint32_t enable);

/* Device pointers of one view's G-buffer (valid after rz_sync of a frame
 * rendered with the G-buffer on). */
int rz_get_view_gbuffer(struct rz_ctx* ctx, uint32_t view, rz_gbuffer* out);

/* ---- Debug-line overlay --------------------------------------------------
 * The reference's DRAW DEBUG step (src/Engine/Graphics.cpp:5694-5738, shaders
 * src/shaders/debug.slang, objects src/Engine/Types.h:81-98): after the blended
 * list, each object draws LINE_LIST segments 5 pixels wide in one constant
 * colour (alpha 1), depth-tested GREATER_OR_EQUAL against the opaque depth
 * with depth writes off (the state the blended list left), into every view.
 * A line or cross object draws vertices 0-1 of the reference's vertex table
 * (Graphics.cpp:3222-3249: the segment (0,0,0)-(0,0,1)); a circle draws
 * vertices 8-107 (50 segments of the unit circle in the xy plane).
 * flags selects the vertex stage by equality, as debug.slang does: 1 screen
 * space (transform * (x, y * width/height, z, w), then z = w = 1), 2 view
 * space (proj * transform * v, then z = w = 1), 4 "transform is points" (the
 * segment joins the transform's first two columns, times view_projection;
 * lines and crosses only), anything else world space (view_projection *
 * transform * v). Lines are rasterised as rectangles (Vulkan's strict lines),
 * at every coverage sample with 4x multisampling. */
#define RZ_DEBUG_LINE 0u
#define RZ_DEBUG_CIRCLE 1u
#define RZ_DEBUG_CROSS 2u /* drawn as the line, as the reference's draw switch does */
#define RZ_DEBUG_SCREEN_SPACE 1u
#define RZ_DEBUG_VIEW_SPACE 2u
#define RZ_DEBUG_TRANSFORM_IS_POINTS 4u
#define RZ_MAX_DEBUG_OBJECTS 65536u

typedef struct rz_debug_object {
    uint32_t type;       /* RZ_DEBUG_LINE / RZ_DEBUG_CIRCLE / RZ_DEBUG_CROSS */
    uint32_t flags;      /* see above */
    float transform[16]; /* column-major, as glm stores it */
    float color[4];      /* rgb drawn, alpha ignored (the shader writes 1) */
} rz_debug_object;

/* Replaces the overlay's objects (count 0 turns the overlay off); used by
 * every following frame, in this order (later segments cover earlier ones). */
int rz_set_debug_objects(struct rz_ctx* ctx, const rz_debug_object* objects, uint32_t count);

/* ---- Learned upsampler ---------------------------------------------------
 * Reconstructs a 2W x 2H RGBA8 sRGB frame from a W x H G-buffer. The network is
 * four 3x3 convolutions with zero padding, 16 -> 32 -> 32 -> 32 -> 12 channels,
 * ReLU after the first three, BF16 weights and activations with FP32
 * accumulation on the tensor cores; its 12 output channels are pixel-shuffled
 * (x2) into RGB and added to the bilinear x2 upsampling of the input colour
 * (sRGB values / 255), then clamped and rounded to 8 bits. The input channels
 * are: colour rgb / 255, albedo rgb / 255, normal (octahedral u, v), coverage
 * (albedo alpha / 255), min(16 * depth, 4), and six zeros.
 *
 * Parameters are one f32 array of RZ_UPSAMPLER_PARAM_COUNT values: for each
 * layer l = 0..3 its weights [cout_l][9][cin_l] (tap = 3 * ky + kx, ky, kx in
 * 0..2 for offsets -1..1) followed by its biases [cout_l], with (cin, cout) =
 * (16, 32), (32, 32), (32, 32), (32, 16); the weights of input channels 10..15
 * of layer 0 and of output channels 12..15 of layer 3 should be zero (their
 * gradients are zero).
 *
 * Training: rz_upsampler_accumulate runs the network on one G-buffer, the loss
 * sum over the 2W x 2H x 3 output values of (prediction - target / 255)^2
 * (prediction before clamping), and the backward pass, adding the gradients of
 * that sum to the gradient buffer; rz_upsampler_adam_step applies Adam with
 * the gradient multiplied by grad_scale and clears the gradient buffer. Every
 * call runs on `stream` (a cudaStream_t; NULL = default stream) without
 * waiting, except the get functions, which synchronise it. One upsampler is
 * used by one host thread at a time. */
#define RZ_UPSAMPLER_PARAM_COUNT 27760u

struct rz_upsampler;
typedef struct rz_upsampler rz_upsampler;

/* Allocates the weights and activation buffers for inputs up to max_width x
 * max_height on `device`; parameters start at zero. */
int rz_upsampler_create(struct rz_upsampler** out, int device, uint32_t max_width, uint32_t max_height);
void rz_upsampler_destroy(struct rz_upsampler* u);

/* Copies `count` (= RZ_UPSAMPLER_PARAM_COUNT) host f32 parameters in / out and
 * resets the Adam moments (set only). */
int rz_upsampler_set_params(struct rz_upsampler* u, const float* params, uint32_t count, void* stream);
int rz_upsampler_get_params(struct rz_upsampler* u, float* params, uint32_t count, void* stream);

/* Inference: out_rgba8 is a device array of (2 * in->width) * (2 * in->height) u32. */
int rz_upsampler_infer(struct rz_upsampler* u, const rz_gbuffer* in, void* out_rgba8, void* stream);

/* Forward + loss + backward on one frame; target_rgba8 is the full-resolution
 * (2W x 2H) frame on the device. out_rgba8 (optional, may be NULL) receives the
 * prediction as in rz_upsampler_infer. */
int rz_upsampler_accumulate(struct rz_upsampler* u, const rz_gbuffer* in, const void* target_rgba8, void* out_rgba8,
                            void* stream);

/* Copies the accumulated gradients (count = RZ_UPSAMPLER_PARAM_COUNT, may be
 * NULL), the accumulated loss sum and the number of accumulated output values
 * to the host. */
int rz_upsampler_get_grads(struct rz_upsampler* u, float* grads, uint32_t count, double* loss_sum,
                           uint64_t* values, void* stream);

/* p -= lr * m_hat / (sqrt(v_hat) + eps) with g = grad_scale * gradient; then
 * clears the gradients and the loss sum. */
int rz_upsampler_adam_step(struct rz_upsampler* u, float lr, float beta1, float beta2, float eps, float grad_scale,
                           void* stream);

/* Device-side error bits of the upsampler's kernels so far (a copy or
 * tensor-core wait that ran out of its time limit sets bit 0; the bits stay set
 * for the life of the object); synchronises `stream`. */
int rz_upsampler_status(struct rz_upsampler* u, uint32_t* flags, void* stream);

/* Diagnostic: the time limit, in SM clock cycles, of each wait inside the
 * upsampler's kernels (TMA copies landed, MMAs done, accumulators drained) for
 * the following calls; 0 restores the default (about one second). A wait that
 * runs out sets bit 0 of the status and its kernel stops early, after its copies
 * and MMAs in flight have completed, with its output incomplete. This library
 * addition has no counterpart in the reference; tests use it to make the waits
 * run out. */
int rz_upsampler_set_wait_limit(struct rz_upsampler* u, uint64_t cycles);

/* Tensor-core self-test: D (128 x n, f32) = A (128 x k, bf16, row-major) *
 * B (n x k, bf16, row-major)^T with one CTA, the MMA layout the convolutions
 * use; n in {16, 32}, k in {16, 32, 48, 64}. All pointers are device arrays.
 * Synchronises `stream`. */
int rz_upsampler_selftest_gemm(const void* a_bf16, const void* b_bf16, float* d_f32, uint32_t n, uint32_t k,
                               void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ROSY_GB300_H */
