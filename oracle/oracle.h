/*
 * ORACLE — test infrastructure only. A scalar CPU restatement of Rosy's shadow
 * depth pass and mesh forward pass, used by the tests, by the smoke check and
 * as the timed CPU baseline of bench.py. The renderer library never calls it.
 *
 * Parity status: unpinned by the reference. Rosy has no tests, golden images or
 * known-answer vectors, and it cannot be built or run here (Windows/VS2022,
 * Vulkan SDK, empty submodules, no graphics stack on either machine), so this
 * restatement is pinned by hand-derived known-answer tests instead. The BC7
 * decoder (bc7_oracle.cpp) is pinned against the GPU texture unit's own BC7
 * decoding, the decoder behind the reference's images (tests/golden/bc7_hw.npz).
 */
#ifndef RZ_ORACLE_H
#define RZ_ORACLE_H

#include <stdint.h>

#include "../include/rosy_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_scene {
    const rz_vertex* vertices;      /* all meshes concatenated */
    uint32_t vertex_count;
    uint32_t index_count;
    const uint32_t* indices;        /* mesh-local, all meshes concatenated */
    const uint32_t* meshes;         /* 4 per mesh: vertex_offset, vertex_count, index_offset, index_count */
    uint32_t mesh_count;
    uint32_t object_count;
    const rz_object* objects;
    const rz_surface* surfaces;
    uint32_t surface_count;
    uint32_t material_count;
    const rz_material* materials;
    const rz_texture* textures;
    uint32_t texture_count;
    uint32_t sampler_count;
    const rz_sampler* samplers;
    const rz_scene_data* scene;
    const rz_draw_config* draw_config;
    uint32_t width;
    uint32_t height;
    uint32_t shadow_size;
    uint32_t samples;               /* camera-pass samples per pixel: 0 or 1, or 4 (standard 4x positions) */
    uint32_t debug_object_count;    /* debug-line overlay, drawn after the blended list (may be 0) */
    const rz_debug_object* debug_objects;
} oracle_scene;

typedef struct oracle_out {
    uint8_t* color;      /* width*height*4, RGBA8 sRGB (may be NULL) */
    float* depth;        /* samples * width*height, one plane per sample (may be NULL) */
    uint32_t* ids;       /* samples * width*height, triangle id + 1, 0 = background (may be NULL) */
    float* shadow;       /* cascades * shadow_size^2: one map per shadow cascade (may be NULL) */
    double* color_f64;   /* width*height*4, FP64 shading, sRGB-encoded in [0,1] before 8-bit rounding (may be NULL) */
    uint64_t* texel_bytes; /* if non-NULL: compulsory texture + shadow-map bytes the shading touched */
} oracle_out;

/* Renders one frame. threads <= 0 uses all hardware threads. Returns 0 on success. */
int oracle_render(const oracle_scene* scene, oracle_out* out, int threads);

/* Only the raster passes: the shadow map and the camera pass's depth/ids. */
int oracle_raster(const oracle_scene* scene, oracle_out* out, int threads);

/* Sub-pixel sources of the learned path's triangle-aware base (the renderer's
 * k_subpixel_sources; no counterpart in the reference): for each pixel of the
 * scene's width*height visibility `ids` (triangle id + 1, 0 = background), the
 * front-most triangle (largest depth plane value through the vertices' z / w)
 * of its 3x3 neighbourhood at each of the four sample points
 * (x + 0.25 / 0.75, y + 0.25 / 0.75) of the 2x image, and which of each point's
 * four bilinear sources (own, horizontal, vertical, diagonal neighbour, clamped
 * at the borders) show that triangle: bit 4k + s of out[pixel] for point
 * k = 2 * (y half) + (x half) and source s. */
int oracle_subpixel_sources(const oracle_scene* scene, const uint32_t* ids, uint16_t* out, int threads);

/* BC7 (bc7_oracle.cpp): one 16-byte block to 16 RGBA8 texels (row-major), and
 * one image of max(1,(w+3)/4) x max(1,(h+3)/4) blocks in rows to w x h RGBA8.
 * oracle_render decodes the scene's RZ_TEXELS_BC7 textures with it first. */
void oracle_bc7_block(const uint8_t block[16], uint8_t out[64]);
int oracle_bc7_decode(const uint8_t* blocks, uint32_t width, uint32_t height, uint8_t* rgba);

#ifdef __cplusplus
}
#endif

#endif
