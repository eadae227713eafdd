// Internal device-side layouts of the renderer (host + device). Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/rosy_gb300.h"

namespace rz {

// One draw of a pass: surface_graphics_data resolved against the mesh table
// (src/Engine/Graphics.cpp:5268-5288 shadow loop, 5631-5653 opaque loop).
struct DrawRec {
    uint32_t vertex_base;  // first vertex of the mesh in the concatenated vertex buffer
    uint32_t first_index;  // mesh.index_offset + start_index
    uint32_t tri_count;    // index_count / 3
    uint32_t object;       // graphic_objects_offset + graphics_object_index
    int32_t material;      // -1 = none
    uint32_t tri_base;     // first triangle id of this draw within the pass
    uint32_t varying_base; // camera pass: first varying record of this draw (one per mesh vertex)
    uint32_t vertex_count; // vertices of the draw's mesh
    uint32_t view;         // the view this draw renders into
    uint32_t cascade;      // shadow pass: the shadow cascade of the view this draw renders into
    uint32_t pad[2];
};
static_assert(sizeof(DrawRec) == 48, "DrawRec layout");

// One view of a frame (a batch renders many): its targets, viewport sizes,
// fixed-function state and scene constants. All views' targets live in pools.
struct ViewRec {
    int width, height;            // camera viewport
    int shadow_w, shadow_h;       // shadow-map viewport
    int cull_front, ccw_front;
    int bias_enabled;
    float bias_constant, bias_clamp, bias_slope;
    uint32_t pcf_mode;
    uint32_t shade_block_base;    // first 16x16 shading tile of this view (tiles are numbered view by view)
    uint64_t* vis;                // width*height
    uint32_t* color;              // width*height RGBA8
    float* depth;                 // width*height
    uint32_t* shadow;             // shadow_w*shadow_h depth bits
    uint2* color16;               // width*height RGBA16F (only with blended surfaces)
    const rz_scene_data* scene;
    int cascades;                 // shadow cascades (1..kMaxCascades), each shadow_w*shadow_h, consecutive
    int samples;                  // camera-pass samples per pixel (1 or 4): vis holds `samples` planes of width*height
    uint32_t* gb_albedo;          // width*height RGBA8 sRGB albedo, or null (G-buffer off)
    uint32_t* gb_normal;          // width*height world normal, octahedral 2 x f16, or null
    uint16_t* gb_sources;         // width*height sub-pixel source masks (single-sampled G-buffer), or null
};

// gpu_material, src/Engine/Graphics.cpp:345-360, packed as in 4071-4150.
struct GpuMaterial {
    float color[4];
    float metallic_factor, roughness_factor, alpha_cutoff;
    uint32_t alpha_mode;
    uint32_t tex[4];      // color, normal, metallic, mixmap image index; UINT32_MAX = absent
    uint32_t sampler[4];  // sampler index; == sampler_count selects the default sampler
};
static_assert(sizeof(GpuMaterial) == 64, "gpu_material is 64 bytes");

// Bindless texture table entry. Texels are RGBA8, level-major, each level
// row-major (the caller's layout), one device allocation per texture.
struct TexDesc {
    uint32_t width, height, levels, srgb;
    uint64_t base;             // device address of the texture's texels (level 0 first)
    uint32_t level_off[16];    // texel offset of each level from base
};

// Per-draw constants of the camera pass computed on the device each frame:
// MVP = viewproj * W, CSM = (ndc_to_tc * shadowProjNear) * W, and the camera and
// sun positions in object space (src/shaders/basic.slang:76-77, 114, 116).
struct DrawConsts {
    float mvp[16];
    float csm[16];
    float cam_obj[4];
    float sun_obj[4];
};

// Sampler state: bit 0 min linear, bit 1 mag linear, bit 2 mip linear,
// bits 4-5 wrap u, bits 6-7 wrap v (0 clamp, 1 mirrored repeat, 2 repeat).
typedef uint32_t SamplerBits;

// Raster setup record, one per (sub-)triangle with S > 0 ordering; 64 bytes.
struct TriRecord {
    int32_t X0, Y0, X1, Y1, X2, Y2;  // 8-bit sub-pixel fixed point
    float z0, dzdx, dzdy, bias;      // depth plane (per sub-pixel) and constant depth bias
    uint32_t p0;                     // px0 | py0 << 16 (bounding box, pixels)
    uint32_t p1;                     // px1 | py1 << 16 (inclusive)
    uint32_t id;                     // camera pass: triangle id + 1
    uint32_t view;                   // view (target) of the triangle
    uint64_t stamp_offset;           // exclusive prefix of stamps over all records
};
static_assert(sizeof(TriRecord) == 64, "TriRecord is 64 bytes");

// Records of the shadow pass carry the cascade in the top bits of their view field.
constexpr uint32_t kViewBits = 24;
constexpr uint32_t kCascadeMask = 3u;     // cascade = (view >> kViewBits) & kCascadeMask
// Large records also carry raster facts the setup computed once, so that the
// raster decodes them instead of recomputing them for every chunk a record
// meets: view bits 26-28 the top-left bias of edges 0-2 (1: not a top-left
// edge), 29 medium, 30 box cut by the viewport, 31 near origin; stamp_offset
// bits 40-63 the stamps per row of the record's box.
constexpr uint32_t kRecFlagShift = 26;
constexpr uint32_t kRecViewMask = (1u << kRecFlagShift) - 1u;  // view index and cascade
constexpr int kStampOffsetBits = 40;
constexpr uint32_t kViewMask = (1u << kViewBits) - 1u;
constexpr int kMaxCascades = 4;

// Standard sample positions of 4x multisampling (Vulkan standardSampleLocations),
// in 1/256 pixel: (0.375, 0.125), (0.875, 0.375), (0.125, 0.625), (0.625, 0.875).
constexpr int kMsaaSamples = 4;
constexpr int32_t kMsaaX[kMsaaSamples] = {96, 224, 32, 160};
constexpr int32_t kMsaaY[kMsaaSamples] = {32, 96, 160, 224};
__host__ __device__ constexpr int32_t msaa_x(int k) { return k == 0 ? 96 : k == 1 ? 224 : k == 2 ? 32 : 160; }
__host__ __device__ constexpr int32_t msaa_y(int k) { return k == 0 ? 32 : k == 1 ? 96 : k == 2 ? 160 : 224; }

constexpr int kStampW = 8;
constexpr int kStampH = 4;
constexpr int kChunkStamps = 32;      // default stamps per raster work chunk
constexpr int kSetupThreads = 256;    // triangles per setup CTA
constexpr float kGuardBand = 64.0f;

// Device error bits (rz_stats.error_flags).
constexpr uint32_t kErrRecordOverflow = 1u << 0;
constexpr uint32_t kErrStampOverflow = 1u << 1;
constexpr uint32_t kErrLookbackTimeout = 1u << 2;
constexpr uint32_t kErrBadIndex = 1u << 3;

// Iterations a look-back wait spins (about 32 ns each) before it gives up with
// kErrLookbackTimeout; rz_set_wait_limit can lower it.
constexpr uint32_t kLookbackSpins = 1u << 22;

// Per-pass scratch header, cleared before each pass.
struct PassHeader {
    uint32_t ticket;          // CTA tile ticket of the setup kernel
    uint32_t records;         // large records written
    uint64_t stamps;          // total stamps of the large records
    uint32_t chunks;          // ceil(stamps / kChunkStamps), clamped to the capacity
    uint32_t records_needed;  // large records the frame produced (may exceed the capacity)
    uint32_t small_records;   // small records appended (may exceed the capacity)
    uint32_t done;            // setup CTAs finished (unordered passes)
    uint64_t alloc;           // unordered passes: (records << 40) | stamps allocated so far
};
static_assert(sizeof(PassHeader) == 40, "PassHeader layout");

// A record is "small" when the triangle's own extent (not its clamped bounding
// box) is at most kSmallExtent pixels in x and y: one lane rasterises it.
constexpr int kSmallExtent = 8;       // default
constexpr int kMaxSmallExtent = 16;   // edge values of a lane-rasterised triangle stay below 2^26

// Pass description handed to the setup/raster launchers.
struct PassParams {
    const DrawRec* draws;
    uint32_t draw_count;
    uint32_t tri_total;       // triangles to set up: ids tri_offset .. tri_offset + tri_total - 1
    uint32_t tri_offset;
    uint32_t chunk_stamps;    // stamps per raster work chunk (tuning)
    uint32_t small_extent;    // largest extent (pixels) of a lane-rasterised triangle (tuning)
    const float* mvp;         // MVP of draw d at mvp + mvp_stride * d
    uint32_t mvp_stride;
    const float4* pos;        // positions (x, y, z, pad)
    const uint32_t* indices;
    uint32_t vertex_count;
    const ViewRec* views;
    int write_id;             // 1: camera pass (64-bit depth|id keys); 0: shadow (depth only)
    int ordered;              // 1: keep every record in submission order, cull none (blended list)
    TriRecord* records;       // large records (stamp-balanced raster)
    uint32_t record_capacity;
    TriRecord* small_records; // small records (one lane each)
    uint32_t small_capacity;
    uint64_t* tile_status;    // one word per setup CTA
    uint32_t* chunk_map;
    uint32_t chunk_capacity;
    PassHeader* header;
    uint32_t* error_flags;
    uint32_t lookback_spins;  // bound of each look-back wait (ordered passes)
    // coverage sample of this raster launch, in 1/256 pixel: the pixel centre
    // (128, 128) or one of the standard 4x positions; camera-pass target plane
    int32_t sample_x, sample_y;
    uint32_t sample_plane;
    int32_t bb_hi;  // smallest sample offset the setup boxed for (32 with 4x samples, else 128)
    // buffers the setup launch zeroes besides its own work (the depth target's
    // CLEAR load-op, folded into the launch that precedes the raster); none when
    // clear_count is 0
    void* clear_ptr[2];
    size_t clear_bytes[2];
    uint32_t clear_count;
    // opaque camera pass only (else null): per triangle that produced a record,
    // its draw and its three varying record indices, for the shading
    uint4* tri_refs;
};

struct ShadeParams {
    const ViewRec* views;
    uint32_t view_count;
    uint32_t shade_blocks;    // 16x16 tiles to shade: block_offset .. block_offset + shade_blocks - 1
    uint32_t block_offset;
    const DrawRec* draws;     // opaque list
    uint32_t draw_count;
    const DrawConsts* consts; // per opaque draw
    float4* varyings;         // 8 float4 per (draw, mesh vertex), written by k_vertex
    uint32_t varying_count;
    const rz_vertex* vertices;
    const uint32_t* indices;
    const rz_object* objects;
    const GpuMaterial* materials;
    const TexDesc* textures;
    uint32_t texture_count;
    const SamplerBits* samplers;  // sampler_count + 1 entries (last = default)
    uint32_t sampler_count;
    const float* srgb_table;      // 256 entries
    int blended;                  // 1: k_shade stores the RGBA16F draw image (color16) for k_blend
    uint32_t samples;             // camera-pass samples per pixel of the views (1 or 4)
    // the opaque camera setup's per-triangle (draw, varying record of each vertex),
    // indexed by pass-global triangle id; null for the blended list, whose
    // triangles are then looked up through the draw list and the index buffer
    const uint4* tri_refs;
};

// The blended list (src/Engine/Graphics.cpp:5654-5691) over the opaque result.
// Debug-line overlay (src/Engine/Graphics.cpp:5694-5738): one segment before
// the vertex stage: its two vertices (from the vertex table, or the points of a
// "transform is points" object) and its object; 48 bytes.
struct DebugPair {
    float a[4], b[4];
    uint32_t object;
    uint32_t pad[3];
};

// One segment of one view after the vertex stage, clipping and the viewport:
// window ends in 1/256 pixel, their depths, the inclusive pixel box
// (x | y << 16) that can hold covered samples, the object's colour; 64 bytes.
struct DebugSeg {
    int32_t X0, Y0, X1, Y1;
    float z0, z1;
    uint32_t p0, p1;
    float rgb[3];
    uint32_t live;                // 0: clipped away or outside the view
    uint32_t pad[4];
};

// (half the line width of 5 pixels, in 1/256 pixel)^2
constexpr int64_t kDebugHalfWidth2 = 640 * 640;
constexpr int32_t kDebugHalfWidth = 640;

struct BlendParams {
    ShadeParams sh;               // blended draws, their constants and varyings
    const TriRecord* records;     // setup records of the blended triangles, in submission order
    const PassHeader* header;
    const uint32_t* error_flags;  // the blended pass's flags: its records are not used after a look-back timeout
    uint32_t record_capacity;
    uint32_t debug_count;         // overlay segments per view (0: no overlay)
    const DebugSeg* debug;        // view v's segments at debug + v * debug_count, in draw order
};

// Up to four buffers to zero in one launch (16-byte stores, byte tail).
struct ClearList {
    void* ptr[6];
    size_t bytes[6];
    int count;
};

// Launchers (rz_raster.cu / rz_shade.cu). All enqueue on `stream`, and add the
// kernels they enqueue to a per-thread count: take_launches() returns the count
// since its last call and starts a new one (a frame's exact launch count).
void note_launch();
uint32_t take_launches();
void launch_clear(const ClearList& list, int sm_count, cudaStream_t stream);
// blocks of `threads` threads that zero a clear list (0 if it is empty)
unsigned clear_blocks(const ClearList& list, int sm_count, unsigned threads);
// The per-draw matrices; with `clear` the same launch also zeroes that list.
void launch_prep(const DrawRec* draws, uint32_t n, const rz_object* objects, const ViewRec* views,
                 float* out_mvp, cudaStream_t stream, const ClearList* clear = nullptr, int sm_count = 0);
void launch_prep_camera(const DrawRec* draws, uint32_t n, const rz_object* objects, const ViewRec* views,
                        DrawConsts* out, cudaStream_t stream, const ClearList* clear = nullptr, int sm_count = 0);
void launch_setup(const PassParams& p, cudaStream_t stream);
void launch_raster(const PassParams& p, int sm_count, cudaStream_t stream);
void launch_vertex(const ShadeParams& p, cudaStream_t stream);
// k_vertex over the varying records [first, varying_count) of the draws in p
// (whose varying_base values start at `first`).
void launch_vertex_range(const ShadeParams& p, uint32_t first, cudaStream_t stream);
void launch_blend(const BlendParams& p, cudaStream_t stream);
// k_debug_prep: the overlay's `count` segments for each of the `view_count` views.
void launch_debug_prep(const DebugPair* pairs, uint32_t count, const rz_debug_object* objects, const ViewRec* views,
                       uint32_t view_count, DebugSeg* out, cudaStream_t stream);
void launch_shade(const ShadeParams& p, cudaStream_t stream);
void launch_subpixel_sources(const ShadeParams& p, cudaStream_t stream);

// BC7 (rz_bc7.cu): bytes of a mip chain's blocks, and the decode of a chain
// (device blocks) into RGBA8 texels (device, level l starting at level_off[l]).
uint64_t bc7_chain_bytes(uint32_t width, uint32_t height, uint32_t levels);
cudaError_t bc7_decode_chain(const void* blocks, uint32_t width, uint32_t height, uint32_t levels,
                             const uint32_t* level_off, uint32_t* texels, cudaStream_t stream);
int setup_ctas(uint32_t tri_total);

}  // namespace rz
