// Host side of the C ABI (include/rosy_gb300.h): the headless replacement of
// Rosy's graphics_device for the shadow pass + scene pass. One CUDA stream per
// context stands in for the Vulkan queue and its command buffer; a frame is a
// fixed sequence of clears and kernels that is captured once into a CUDA graph
// and replayed until the layout changes.
//
// A context holds scenes (an asset plus its objects and surfaces; scene 0 is the
// one rz_set_asset / rz_set_objects define) and views (a camera with its own
// extent, shadow map, draw state and scene constants onto one scene). Every
// kernel of a frame runs once over all views: draws carry their view, and each
// view's targets are ranges of shared pools. The single-view API is a batch of
// one view.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "rz_internal.h"

using namespace rz;

namespace {

struct PassBuffers {
    TriRecord* records = nullptr;
    uint32_t record_capacity = 0;
    TriRecord* small_records = nullptr;
    uint32_t small_capacity = 0;
    uint64_t* tile_status = nullptr;
    uint32_t tile_capacity = 0;
    uint32_t* chunk_map = nullptr;
    uint32_t chunk_capacity = 0;
};

template <class T>
cudaError_t dalloc(T** p, size_t count) {
    *p = nullptr;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
}

template <class T>
void dfree(T*& p) {
    if (p) cudaFree(p);
    p = nullptr;
}

// The frame report: pass headers and device error words, one block on the
// device and its pinned host mirror, copied back in one copy at the end of each
// frame. Each branch of the frame graph zeroes (with one clear range) and writes
// its own error word next to its own headers, so that the clears of the two
// concurrent branches never touch the other's flags.
struct FrameReport {
    PassHeader shadow;
    uint32_t shadow_errors;  // shadow pass
    uint32_t pad0;
    PassHeader camera;
    PassHeader blended;
    uint32_t camera_errors;  // camera and blended passes
    uint32_t pad1;
    uint32_t errors() const { return shadow_errors | camera_errors; }
};
static_assert(sizeof(FrameReport) == 136 && offsetof(FrameReport, camera) == 48, "frame report layout");

// A scene: its slice of the concatenated asset and object arrays, and its surfaces.
struct SceneHost {
    uint32_t mesh_base = 0, mesh_count = 0;
    uint32_t material_base = 0, material_count = 0;
    uint32_t texture_base = 0, texture_count = 0;
    uint32_t sampler_base = 0, sampler_count = 0;
    uint32_t object_base = 0, object_count = 0;
    std::vector<rz_surface> surfaces;
    bool has_objects = false;
};

struct ViewHost {
    uint32_t scene = 0;
    uint32_t width = 0, height = 0, shadow = 0;
    rz_draw_config dc{};
    bool has_scene_data = false;
};

constexpr uint32_t kDefaultSampler = 0xFFFFFFFFu;  // any index >= the sampler count selects the default

}  // namespace

struct rz_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;  // shadow pass branch of the frame graph
    cudaStream_t vtx = nullptr;   // vertex stage, beside the camera pass's setup and raster
    cudaEvent_t vtx_fork = nullptr, vtx_join = nullptr;
    // read-back (rz_read_frame): device staging copies on the frame stream, then
    // device-to-host copies on their own stream so that the next frame renders meanwhile
    cudaStream_t copy_stream = nullptr;
    // read-back (rz_read_frame): the D2H copies of a frame's colour and depth,
    // which are read straight from its target set, one completion event per set
    cudaEvent_t read_done[2] = {nullptr, nullptr};
    bool read_issued[2] = {false, false};
    uint32_t read_newest = 0;     // target set of the newest read-back
    uint64_t reads_issued = 0;
    cudaEvent_t fork = nullptr, join = nullptr;
    cudaEvent_t camera_done = nullptr, sources_done = nullptr;  // the side branch of the G-buffer's sub-pixel sources
    uint32_t queue_chunks = 0;    // fixed work-queue depth (0 = sized from the scene)
    uint32_t chunk_stamps = kChunkStamps;
    uint32_t small_extent = kSmallExtent;
    uint32_t lookback_spins = kLookbackSpins;
    bool batched = true;          // false: per-view sequential launches
    std::string last_error;

    // asset of all scenes, concatenated (host copies of the small arrays, device arrays)
    std::vector<rz_vertex> verts;
    std::vector<float4> pos;
    std::vector<uint32_t> idx;
    std::vector<uint32_t> mesh_table;  // 4 per mesh: vertex_offset, vertex_count, index_offset, index_count
    std::vector<GpuMaterial> materials;
    std::vector<TexDesc> tex_descs;
    std::vector<uint32_t*> tex_allocs;  // one device allocation per texture
    std::vector<SamplerBits> samplers;  // without the default sampler
    std::vector<rz_object> objects;
    std::vector<SceneHost> scenes;
    rz_vertex* d_vertices = nullptr;
    float4* d_pos = nullptr;
    uint32_t* d_indices = nullptr;
    GpuMaterial* d_materials = nullptr;
    TexDesc* d_textures = nullptr;
    SamplerBits* d_samplers = nullptr;
    // The per-frame inputs (object records, scene constants) are double-buffered
    // with the target sets: the host stages them in pinned memory, and before a
    // frame renders into set k they are copied into set k's buffers on the upload
    // stream, once the frame that last used set k is done; the frame waits for
    // that copy, which so overlaps the frame before it.
    rz_object* d_objects = nullptr;       // the object records of the frame being enqueued
    rz_object* d_objects_base = nullptr;  // both sets: set k at k * objects.size()
    rz_object* h_objects = nullptr;       // pinned staging: every object, current
    size_t h_objects_capacity = 0;
    cudaStream_t upload = nullptr;
    cudaEvent_t upload_done[2] = {nullptr, nullptr};  // the last copy into set k
    cudaEvent_t set_done[2] = {nullptr, nullptr};     // the last frame that used set k
    uint64_t objects_version = 1, scene_version = 1;  // bumped by every update
    uint64_t set_objects_version[2] = {0, 0}, set_scene_version[2] = {0, 0};
    float* d_srgb = nullptr;
    bool asset_dirty = true;         // device asset arrays need an upload

    // views
    std::vector<ViewHost> views;
    rz_scene_data* d_scene_data = nullptr;  // one per view, per set: set k at k * scene_data_capacity
    rz_scene_data* h_scene_data = nullptr;  // pinned staging, one per view
    uint32_t scene_data_capacity = 0;
    // The colour and depth targets are double-buffered: frames alternate between
    // two target sets, so the read-back of one frame copies its images to the
    // host while the next frame renders into the other set. Each set has its
    // view table (whose ViewRec.color / .depth point into it) and its frame graph.
    ViewRec* d_views = nullptr;          // the view table of the frame being enqueued
    ViewRec* d_views_set[2] = {nullptr, nullptr};
    uint32_t parity = 0;                 // target set of the next frame
    uint32_t last_parity = 0;            // target set of the last frame enqueued
    std::vector<ViewRec> view_recs;      // target set 0
    std::vector<uint32_t> view_id_base;  // first opaque triangle id of each view
    // per-view ranges for sequential launches
    struct ViewRange {
        uint32_t shadow_tri_base, shadow_tris, opaque_tri_base, opaque_tris;
        uint32_t varying_begin, varying_end, block_base, blocks;
        size_t pix_off, pix, shadow_off, shadow;
    };
    std::vector<ViewRange> ranges;
    uint64_t* d_vis = nullptr;
    uint32_t* d_color = nullptr;
    float* d_depth = nullptr;
    uint32_t* d_shadow = nullptr;
    uint2* d_color16 = nullptr;
    bool gbuffer = false;             // shading also writes albedo + normal (rz_set_gbuffer)
    uint32_t samples = 1;             // camera-pass samples per pixel (1 or 4)
    uint32_t* d_gb_albedo = nullptr;
    uint32_t* d_gb_normal = nullptr;
    uint16_t* d_gb_sources = nullptr;
    size_t gb_capacity = 0;
    size_t pix_capacity = 0, shadow_capacity = 0, color16_capacity = 0;
    size_t pix_total = 0, shadow_total = 0;
    uint32_t shade_blocks = 0;

    // draw lists over all views
    DrawRec* d_shadow_draws = nullptr;
    DrawRec* d_opaque_draws = nullptr;
    DrawRec* d_blended_draws = nullptr;
    uint32_t shadow_draw_count = 0, opaque_draw_count = 0, blended_draw_count = 0;
    uint32_t shadow_tris = 0, opaque_tris = 0, blended_tris = 0;
    float* d_shadow_mvp = nullptr;
    DrawConsts* d_camera_consts = nullptr;
    DrawConsts* d_blended_consts = nullptr;
    float4* d_varyings = nullptr;
    uint4* d_tri_refs = nullptr;  // per opaque triangle: its draw and varying records (written by the camera setup)
    uint32_t varying_count = 0, blended_varying_base = 0;
    bool layout_dirty = true;        // draw lists, pools and view table need a rebuild

    // raster scratch
    PassBuffers shadow_pass, camera_pass, blended_pass;
    // The frame report (pass headers, error words), one per target set: a frame
    // fills its set's report, which is copied to the host on the copy stream
    // after the frame (off the frame stream); the readers wait for that copy.
    FrameReport* d_report = nullptr;       // the report of the frame being enqueued
    FrameReport* d_report_base = nullptr;  // both sets
    FrameReport* h_report = nullptr;       // pinned: the report of the last frame enqueued
    FrameReport* h_report_base = nullptr;  // both sets
    cudaEvent_t report_done[2] = {nullptr, nullptr};
    bool report_issued[2] = {false, false};
    bool grow_records = false, grow_chunks = false;

    // frame sequencing
    cudaGraphExec_t graph_set[2] = {nullptr, nullptr};  // one per target set
    bool graph_dirty = true;
    bool use_graph = true;
    cudaEvent_t frame_done = nullptr;
    bool frame_pending = false;
    bool timing = false;
    uint32_t frame_launches = 0;  // kernels the last enqueued frame launches (graph replays included)
    // debug-line overlay: objects and their segments (host), their device copies, and
    // the segments of every view after the vertex stage (k_debug_prep)
    std::vector<rz_debug_object> debug_objects;
    std::vector<DebugPair> debug_pairs;
    rz_debug_object* d_debug_objects = nullptr;
    DebugPair* d_debug_pairs = nullptr;
    DebugSeg* d_debug_segs = nullptr;
    size_t debug_seg_capacity = 0;
    uint32_t debug_count = 0;     // segments per view in the current layout (0: overlay off)
    cudaEvent_t stage_ev[RZ_STAGE_COUNT + 1] = {};
    uint32_t frames = 0;
};

namespace {

int fail(rz_ctx* ctx, int code, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return code;
}

int cuda_fail(rz_ctx* ctx, cudaError_t e, const char* what) {
    return fail(ctx, e == cudaErrorMemoryAllocation ? RZ_ALLOCATION_FAILURE : RZ_ERROR,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define RZ_CUDA(ctx, expr, what)                                \
    do {                                                        \
        cudaError_t _e = (expr);                                \
        if (_e != cudaSuccess) return cuda_fail(ctx, _e, what); \
    } while (0)

void drop_graph(rz_ctx* c) {
    for (int k = 0; k < 2; ++k) {
        if (c->graph_set[k]) cudaGraphExecDestroy(c->graph_set[k]);
        c->graph_set[k] = nullptr;
    }
    c->graph_dirty = true;
}

void free_pass(PassBuffers& p) {
    dfree(p.records);
    dfree(p.small_records);
    dfree(p.tile_status);
    dfree(p.chunk_map);
    p.record_capacity = p.small_capacity = p.tile_capacity = p.chunk_capacity = 0;
}

// Sizes the raster scratch of a pass: one record per triangle plus room for
// clipped fans, and a chunk map for `stamps_hint` stamps.
int size_pass(rz_ctx* c, PassBuffers& p, uint32_t tris, uint64_t stamps_hint) {
    const uint32_t rec_cap = tris + tris / 4 + 4096;
    const uint32_t tiles = (uint32_t)setup_ctas(tris) + 1;
    uint64_t chunks = (stamps_hint + c->chunk_stamps - 1) / c->chunk_stamps + 1024;
    if (c->queue_chunks) chunks = c->queue_chunks;
    if (chunks > 0xFFFFFFFFull) chunks = 0xFFFFFFFFull;
    if (rec_cap > p.record_capacity) {
        dfree(p.records);
        RZ_CUDA(c, dalloc(&p.records, rec_cap), "raster records");
        p.record_capacity = rec_cap;
    }
    if (rec_cap > p.small_capacity) {
        dfree(p.small_records);
        RZ_CUDA(c, dalloc(&p.small_records, rec_cap), "small raster records");
        p.small_capacity = rec_cap;
    }
    if (tiles > p.tile_capacity) {
        dfree(p.tile_status);
        RZ_CUDA(c, dalloc(&p.tile_status, tiles), "tile status");
        p.tile_capacity = tiles;
    }
    if (chunks > p.chunk_capacity || c->queue_chunks) {
        dfree(p.chunk_map);
        RZ_CUDA(c, dalloc(&p.chunk_map, (size_t)chunks), "chunk map");
        p.chunk_capacity = (uint32_t)chunks;
    }
    return RZ_OK;
}

// Stamps a pass may need: never more than every triangle covering its whole
// target; otherwise room for 256 full-screen layers of overdraw plus 16 stamps
// per triangle. A frame that needs more reports RZ_OVERFLOW and the capacity
// grows for the next frame.
uint64_t stamp_hint(uint32_t tris, uint64_t target_pixels) {
    const uint64_t screen = target_pixels / (kStampW * kStampH) + 1;
    const uint64_t bound = (uint64_t)tris * screen;
    const uint64_t hint = screen * 256 + (uint64_t)tris * 16;
    return bound < hint ? bound : hint;
}

SamplerBits sampler_bits(const rz_sampler& s) {
    // src/Engine/Graphics.cpp:250-278 (filters/wraps), 3996-4014 (mip linear)
    SamplerBits b = 0;
    if (!(s.min_filter <= 2)) b |= 1u;
    if (!(s.mag_filter <= 2)) b |= 2u;
    b |= 4u;
    const uint32_t wu = s.wrap_s == 0 ? 0u : (s.wrap_s == 1 ? 1u : 2u);
    const uint32_t wv = s.wrap_t == 0 ? 0u : (s.wrap_t == 1 ? 1u : 2u);
    return b | (wu << 4) | (wv << 6);
}

void free_asset(rz_ctx* c) {
    for (uint32_t* p : c->tex_allocs) cudaFree(p);
    c->tex_allocs.clear();
    c->verts.clear();
    c->pos.clear();
    c->idx.clear();
    c->mesh_table.clear();
    c->materials.clear();
    c->tex_descs.clear();
    c->samplers.clear();
    c->objects.clear();
    c->scenes.clear();
    c->asset_dirty = true;
    c->layout_dirty = true;
}

// Appends an asset to the concatenated arrays as a new scene (no objects yet).
// Meshes are concatenated as set_asset does (src/Engine/Graphics.cpp:4310-4334)
// and materials packed with its index mapping (4071-4150).
int append_asset(rz_ctx* c, const rz_mesh* meshes, uint32_t mesh_count, const rz_material* mats, uint32_t mat_count,
                 const rz_texture* textures, uint32_t tex_count, const rz_sampler* samplers, uint32_t sampler_count,
                 SceneHost& out) {
    if (mesh_count == 0 || !meshes) return fail(c, RZ_INVALID_ARGUMENT, "asset has no meshes");
    if ((mat_count && !mats) || (tex_count && !textures) || (sampler_count && !samplers))
        return fail(c, RZ_INVALID_ARGUMENT, "null array with non-zero count");
    uint64_t nv = c->verts.size(), ni = c->idx.size();
    for (uint32_t m = 0; m < mesh_count; ++m) {
        if ((meshes[m].position_count && !meshes[m].positions) || (meshes[m].index_count && !meshes[m].indices))
            return fail(c, RZ_INVALID_ARGUMENT, "mesh with null data");
        for (uint32_t i = 0; i < meshes[m].index_count; ++i)
            if (meshes[m].indices[i] >= meshes[m].position_count)
                return fail(c, RZ_INVALID_ARGUMENT, "mesh " + std::to_string(m) + " index out of range");
        nv += meshes[m].position_count;
        ni += meshes[m].index_count;
    }
    if (nv >= 0xFFFFFFFFull || ni >= 0xFFFFFFFFull) return fail(c, RZ_OVERFLOW, "asset too large");
    for (uint32_t i = 0; i < tex_count; ++i) {
        const rz_texture& t = textures[i];
        // extents up to 2^30 keep the sampler's int texel arithmetic exact
        if (t.width == 0 || t.height == 0 || t.width > (1u << 30) || t.height > (1u << 30) || t.levels == 0 ||
            t.levels > 16 || !t.texels ||
            (t.format != RZ_TEXELS_RGBA8 && t.format != RZ_TEXELS_BC7))
            return fail(c, RZ_INVALID_ARGUMENT, "texture " + std::to_string(i) + " is malformed");
        // levels <= 16 is checked above, so counting stops there (a shift by 32 is undefined)
        uint32_t max_levels = 1;
        while (max_levels < 16 && ((t.width >> max_levels) || (t.height >> max_levels))) ++max_levels;
        if (t.levels > max_levels) return fail(c, RZ_INVALID_ARGUMENT, "texture has too many levels");
    }
    SceneHost sh;
    sh.mesh_base = (uint32_t)(c->mesh_table.size() / 4);
    sh.mesh_count = mesh_count;
    sh.material_base = (uint32_t)c->materials.size();
    sh.material_count = mat_count;
    sh.texture_base = (uint32_t)c->tex_descs.size();
    sh.texture_count = tex_count;
    sh.sampler_base = (uint32_t)c->samplers.size();
    sh.sampler_count = sampler_count;
    sh.object_base = (uint32_t)c->objects.size();
    for (uint32_t m = 0; m < mesh_count; ++m) {
        const rz_mesh& mesh = meshes[m];
        c->mesh_table.push_back((uint32_t)c->verts.size());
        c->mesh_table.push_back(mesh.position_count);
        c->mesh_table.push_back((uint32_t)c->idx.size());
        c->mesh_table.push_back(mesh.index_count);
        for (uint32_t i = 0; i < mesh.position_count; ++i) {
            c->verts.push_back(mesh.positions[i]);
            c->pos.push_back(make_float4(mesh.positions[i].position[0], mesh.positions[i].position[1],
                                         mesh.positions[i].position[2], 1.0f));
        }
        c->idx.insert(c->idx.end(), mesh.indices, mesh.indices + mesh.index_count);
    }
    for (uint32_t i = 0; i < mat_count; ++i) {
        const rz_material& m = mats[i];
        GpuMaterial g{};
        for (int k = 0; k < 4; ++k) g.color[k] = m.base_color_factor[k];
        g.metallic_factor = m.metallic_factor;
        g.roughness_factor = m.roughness_factor;
        g.alpha_cutoff = m.alpha_cutoff;
        g.alpha_mode = m.alpha_mode;
        const uint32_t img[4] = {m.color_image_index, m.normal_image_index, m.metallic_image_index, m.mixmap_image_index};
        const uint32_t smp[4] = {m.color_sampler_index, m.normal_sampler_index, m.metallic_sampler_index, m.mixmap_sampler_index};
        for (int k = 0; k < 4; ++k) {
            g.tex[k] = RZ_INVALID_INDEX;
            g.sampler[k] = kDefaultSampler;
            if (img[k] < tex_count) {
                g.tex[k] = sh.texture_base + img[k];
                if (smp[k] < sampler_count) g.sampler[k] = sh.sampler_base + smp[k];
            }
        }
        c->materials.push_back(g);
    }
    for (uint32_t i = 0; i < tex_count; ++i) {
        const rz_texture& t = textures[i];
        TexDesc d{};
        d.width = t.width;
        d.height = t.height;
        d.levels = t.levels;
        d.srgb = t.image_type == RZ_IMAGE_NORMAL_MAP ? 0u : 1u;
        uint64_t off = 0;
        for (uint32_t l = 0; l < t.levels; ++l) {
            d.level_off[l] = (uint32_t)off;
            off += (uint64_t)std::max(1u, t.width >> l) * std::max(1u, t.height >> l);
        }
        if (off >= 0xFFFFFFFFull) return fail(c, RZ_OVERFLOW, "texture too large");
        uint32_t* dp = nullptr;
        RZ_CUDA(c, dalloc(&dp, (size_t)off), "texture");
        c->tex_allocs.push_back(dp);
        if (t.format == RZ_TEXELS_BC7) {
            // the blocks go through a staging buffer and are decoded into the RGBA8 texels
            const uint64_t nb = bc7_chain_bytes(t.width, t.height, t.levels);
            void* staging = nullptr;
            RZ_CUDA(c, cudaMalloc(&staging, nb), "BC7 staging");
            cudaError_t e = cudaMemcpy(staging, t.texels, nb, cudaMemcpyHostToDevice);
            if (e == cudaSuccess) e = bc7_decode_chain(staging, t.width, t.height, t.levels, d.level_off, dp, 0);
            if (e == cudaSuccess) e = cudaStreamSynchronize(0);
            cudaFree(staging);
            RZ_CUDA(c, e, "BC7 decode");
        } else {
            RZ_CUDA(c, cudaMemcpy(dp, t.texels, (size_t)off * 4, cudaMemcpyHostToDevice), "upload texels");
        }
        d.base = reinterpret_cast<uint64_t>(dp);
        c->tex_descs.push_back(d);
    }
    for (uint32_t i = 0; i < sampler_count; ++i) c->samplers.push_back(sampler_bits(samplers[i]));
    out = sh;
    c->asset_dirty = true;
    c->layout_dirty = true;
    return RZ_OK;
}

// Validates a scene's surfaces against its asset and objects.
int check_surfaces(rz_ctx* c, const SceneHost& sh, uint32_t object_count, const rz_surface* surfaces, uint32_t n) {
    for (uint32_t i = 0; i < n; ++i) {
        const rz_surface& s = surfaces[i];
        if (s.mesh_index >= sh.mesh_count) return fail(c, RZ_INVALID_ARGUMENT, "surface mesh index out of range");
        const uint64_t obj = (uint64_t)s.graphic_objects_offset + s.graphics_object_index;
        if (obj >= object_count) return fail(c, RZ_INVALID_ARGUMENT, "surface object index out of range");
        const uint32_t* mt = &c->mesh_table[4 * (sh.mesh_base + s.mesh_index)];
        if ((uint64_t)s.start_index + s.index_count > mt[3])
            return fail(c, RZ_INVALID_ARGUMENT, "surface index range outside its mesh");
        const bool has_mat = s.material_index < sh.material_count;
        if (!s.blended && has_mat && c->materials[sh.material_base + s.material_index].alpha_mode != 0)
            return fail(c, RZ_INVALID_ARGUMENT, "opaque surface with a non-opaque material");
    }
    return RZ_OK;
}

int upload_asset(rz_ctx* c) {
    cudaStreamSynchronize(c->stream);
    dfree(c->d_vertices);
    dfree(c->d_pos);
    dfree(c->d_indices);
    dfree(c->d_materials);
    dfree(c->d_textures);
    dfree(c->d_samplers);
    const size_t nv = c->verts.size(), ni = c->idx.size();
    RZ_CUDA(c, dalloc(&c->d_vertices, std::max<size_t>(nv, 1)), "vertex buffer");
    RZ_CUDA(c, dalloc(&c->d_pos, std::max<size_t>(nv, 1)), "position stream");
    RZ_CUDA(c, dalloc(&c->d_indices, std::max<size_t>(ni, 1)), "index buffer");
    RZ_CUDA(c, dalloc(&c->d_materials, std::max<size_t>(c->materials.size(), 1)), "material buffer");
    RZ_CUDA(c, dalloc(&c->d_textures, std::max<size_t>(c->tex_descs.size(), 1)), "texture table");
    RZ_CUDA(c, dalloc(&c->d_samplers, c->samplers.size() + 1), "sampler table");
    if (nv) {
        RZ_CUDA(c, cudaMemcpy(c->d_vertices, c->verts.data(), nv * sizeof(rz_vertex), cudaMemcpyHostToDevice), "upload vertices");
        RZ_CUDA(c, cudaMemcpy(c->d_pos, c->pos.data(), nv * sizeof(float4), cudaMemcpyHostToDevice), "upload positions");
    }
    if (ni) RZ_CUDA(c, cudaMemcpy(c->d_indices, c->idx.data(), ni * 4, cudaMemcpyHostToDevice), "upload indices");
    if (!c->materials.empty())
        RZ_CUDA(c, cudaMemcpy(c->d_materials, c->materials.data(), c->materials.size() * sizeof(GpuMaterial),
                              cudaMemcpyHostToDevice), "upload materials");
    if (!c->tex_descs.empty())
        RZ_CUDA(c, cudaMemcpy(c->d_textures, c->tex_descs.data(), c->tex_descs.size() * sizeof(TexDesc),
                              cudaMemcpyHostToDevice), "upload texture table");
    std::vector<SamplerBits> sb = c->samplers;
    // default sampler: linear/linear, nearest mip, repeat (src/Engine/Graphics.cpp:3421-3438)
    sb.push_back(1u | 2u | (2u << 4) | (2u << 6));
    RZ_CUDA(c, cudaMemcpy(c->d_samplers, sb.data(), sb.size() * sizeof(SamplerBits), cudaMemcpyHostToDevice), "upload samplers");
    c->asset_dirty = false;
    c->layout_dirty = true;
    return RZ_OK;
}

// Waits until the copies queued from the host staging have read it.
cudaError_t wait_uploads(rz_ctx* c) {
    for (int k = 0; k < 2; ++k) {
        const cudaError_t e = cudaEventSynchronize(c->upload_done[k]);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

int upload_objects(rz_ctx* c) {
    cudaStreamSynchronize(c->stream);
    cudaStreamSynchronize(c->upload);
    dfree(c->d_objects_base);
    c->d_objects = nullptr;
    const size_t n = c->objects.size();
    RZ_CUDA(c, dalloc(&c->d_objects_base, 2 * std::max<size_t>(n, 1)), "object buffer");
    c->d_objects = c->d_objects_base;
    if (n > c->h_objects_capacity) {
        if (c->h_objects) cudaFreeHost(c->h_objects);
        c->h_objects = nullptr;
        c->h_objects_capacity = 0;
        RZ_CUDA(c, cudaMallocHost(&c->h_objects, n * sizeof(rz_object)), "object staging");
        c->h_objects_capacity = n;
    }
    if (n) std::memcpy(c->h_objects, c->objects.data(), n * sizeof(rz_object));
    ++c->objects_version;  // both sets take the objects before their next frame
    c->layout_dirty = true;  // the graph holds the object buffer's address
    return RZ_OK;
}

int ensure_scene_data(rz_ctx* c, uint32_t n) {
    if (n <= c->scene_data_capacity) return RZ_OK;
    cudaStreamSynchronize(c->stream);
    cudaStreamSynchronize(c->upload);
    rz_scene_data* d = nullptr;
    rz_scene_data* h = nullptr;
    RZ_CUDA(c, dalloc(&d, 2 * (size_t)n), "scene constants");
    RZ_CUDA(c, cudaMallocHost(&h, n * sizeof(rz_scene_data)), "scene staging");
    std::memset(h, 0, n * sizeof(rz_scene_data));
    if (c->scene_data_capacity) std::memcpy(h, c->h_scene_data, c->scene_data_capacity * sizeof(rz_scene_data));
    ++c->scene_version;  // both sets take the staged constants before their next frame
    dfree(c->d_scene_data);
    if (c->h_scene_data) cudaFreeHost(c->h_scene_data);
    c->d_scene_data = d;
    c->h_scene_data = h;
    c->scene_data_capacity = n;
    c->layout_dirty = true;
    return RZ_OK;
}

// Shadow cascades of a view: draw_config.shadow_cascades clamped to 1..kMaxCascades (0 = 1).
uint32_t cascades_of(const ViewHost& v) {
    const uint32_t n = v.dc.shadow_cascades;
    return n < 1 ? 1u : (n > (uint32_t)kMaxCascades ? (uint32_t)kMaxCascades : n);
}

// Rebuilds the draw lists over all views, the target pools and the view table.
int build_layout(rz_ctx* c) {
    if (c->views.empty()) return fail(c, RZ_INVALID_STATE, "no views");
    cudaStreamSynchronize(c->stream);
    cudaStreamSynchronize(c->copy_stream);  // read-backs copy straight from the targets
    drop_graph(c);
    // pools
    size_t pix = 0, shadow = 0;
    uint32_t blocks = 0;
    std::vector<size_t> pix_off, shadow_off;
    std::vector<uint32_t> block_base;
    for (const ViewHost& v : c->views) {
        pix_off.push_back(pix);
        shadow_off.push_back(shadow);
        block_base.push_back(blocks);
        pix += (size_t)v.width * v.height;
        shadow += (size_t)cascades_of(v) * v.shadow * v.shadow;
        blocks += ((v.width + 15) / 16) * ((v.height + 15) / 16);
    }
    // draw lists, view-major, each view's surfaces in scene order (src/Engine/Graphics.cpp:4715-4735)
    std::vector<DrawRec> shadow_list, opaque, blended;
    uint64_t shadow_tris = 0, opaque_tris = 0, blended_tris = 0, varyings = 0;
    c->view_id_base.assign(c->views.size(), 0);
    c->ranges.assign(c->views.size(), rz_ctx::ViewRange{});
    for (uint32_t vi = 0; vi < c->views.size(); ++vi) {
        const ViewHost& v = c->views[vi];
        c->view_id_base[vi] = (uint32_t)opaque_tris;
        rz_ctx::ViewRange& rg = c->ranges[vi];
        rg.shadow_tri_base = (uint32_t)shadow_tris;
        rg.opaque_tri_base = (uint32_t)opaque_tris;
        rg.varying_begin = (uint32_t)varyings;
        rg.block_base = block_base[vi];
        rg.blocks = ((v.width + 15) / 16) * ((v.height + 15) / 16);
        rg.pix_off = pix_off[vi];
        rg.pix = (size_t)v.width * v.height;
        rg.shadow_off = shadow_off[vi];
        rg.shadow = (size_t)cascades_of(v) * v.shadow * v.shadow;
        if (v.scene >= c->scenes.size()) return fail(c, RZ_INVALID_STATE, "view refers to a missing scene");
        const SceneHost& sh = c->scenes[v.scene];
        if (!sh.has_objects) return fail(c, RZ_INVALID_STATE, "scene has no objects (rz_set_objects)");
        if (!v.has_scene_data) return fail(c, RZ_INVALID_STATE, "view has no scene constants (rz_update)");
        for (const rz_surface& s : sh.surfaces) {
            const uint32_t* mt = &c->mesh_table[4 * (sh.mesh_base + s.mesh_index)];
            DrawRec d{};
            d.vertex_base = mt[0];
            d.first_index = mt[2] + s.start_index;
            d.tri_count = s.index_count / 3;
            d.object = sh.object_base + s.graphic_objects_offset + s.graphics_object_index;
            d.material = s.material_index < sh.material_count ? (int32_t)(sh.material_base + s.material_index) : -1;
            d.vertex_count = mt[1];
            d.view = vi;
            for (uint32_t k = 0; k < cascades_of(v); ++k) {
                d.cascade = k;
                d.tri_base = (uint32_t)shadow_tris;
                shadow_list.push_back(d);
                shadow_tris += d.tri_count;
            }
            d.cascade = 0;
            if (s.blended) {
                d.tri_base = (uint32_t)blended_tris;
                blended.push_back(d);
                blended_tris += d.tri_count;
            } else {
                d.tri_base = (uint32_t)opaque_tris;
                d.varying_base = (uint32_t)varyings;
                varyings += d.vertex_count;
                opaque.push_back(d);
                opaque_tris += d.tri_count;
            }
        }
        rg.shadow_tris = (uint32_t)(shadow_tris - rg.shadow_tri_base);
        rg.opaque_tris = (uint32_t)(opaque_tris - rg.opaque_tri_base);
        rg.varying_end = (uint32_t)varyings;
    }
    const uint64_t blended_varying_base = varyings;
    for (DrawRec& d : blended) {
        d.varying_base = (uint32_t)varyings;
        varyings += d.vertex_count;
    }
    if (shadow_tris >= 0xFFFFFFF0ull || varyings >= 0xFFFFFFF0ull) return fail(c, RZ_OVERFLOW, "too many triangles");
    // buffers
    if (pix > c->pix_capacity) {
        dfree(c->d_vis);
        dfree(c->d_color);
        dfree(c->d_depth);
        c->pix_capacity = 0;
        RZ_CUDA(c, dalloc(&c->d_vis, pix * c->samples), "visibility buffers");
        RZ_CUDA(c, dalloc(&c->d_color, 2 * pix), "colour buffers");
        RZ_CUDA(c, dalloc(&c->d_depth, 2 * pix), "depth buffers");
        RZ_CUDA(c, cudaMemset(c->d_color, 0, 2 * pix * 4), "clear colour");
        RZ_CUDA(c, cudaMemset(c->d_depth, 0, 2 * pix * 4), "clear depth");
        c->pix_capacity = pix;
    }
    if (shadow > c->shadow_capacity) {
        dfree(c->d_shadow);
        c->shadow_capacity = 0;
        RZ_CUDA(c, dalloc(&c->d_shadow, shadow), "shadow maps");
        c->shadow_capacity = shadow;
    }
    // the overlay draws into the per-sample RGBA16F draw images, as the blended list does
    const bool overlay = !c->debug_pairs.empty();
    if ((!blended.empty() || overlay) && pix > c->color16_capacity) {
        dfree(c->d_color16);
        c->color16_capacity = 0;
        RZ_CUDA(c, dalloc(&c->d_color16, pix * c->samples), "RGBA16F draw images");
        c->color16_capacity = pix;
    }
    if (c->gbuffer && pix > c->gb_capacity) {
        dfree(c->d_gb_albedo);
        dfree(c->d_gb_normal);
        dfree(c->d_gb_sources);
        c->gb_capacity = 0;
        RZ_CUDA(c, dalloc(&c->d_gb_albedo, pix), "G-buffer albedo");
        RZ_CUDA(c, dalloc(&c->d_gb_normal, pix), "G-buffer normals");
        RZ_CUDA(c, dalloc(&c->d_gb_sources, pix), "G-buffer sub-pixel sources");
        c->gb_capacity = pix;
    }
    dfree(c->d_debug_objects);
    dfree(c->d_debug_pairs);
    c->debug_count = 0;
    if (overlay) {
        const size_t segs = c->debug_pairs.size() * c->views.size();
        if (segs > c->debug_seg_capacity) {
            dfree(c->d_debug_segs);
            c->debug_seg_capacity = 0;
            RZ_CUDA(c, dalloc(&c->d_debug_segs, segs), "overlay segments");
            c->debug_seg_capacity = segs;
        }
        RZ_CUDA(c, dalloc(&c->d_debug_objects, c->debug_objects.size()), "overlay objects");
        RZ_CUDA(c, dalloc(&c->d_debug_pairs, c->debug_pairs.size()), "overlay vertices");
        RZ_CUDA(c, cudaMemcpy(c->d_debug_objects, c->debug_objects.data(), c->debug_objects.size() * sizeof(rz_debug_object),
                              cudaMemcpyHostToDevice), "upload overlay objects");
        RZ_CUDA(c, cudaMemcpy(c->d_debug_pairs, c->debug_pairs.data(), c->debug_pairs.size() * sizeof(DebugPair),
                              cudaMemcpyHostToDevice), "upload overlay vertices");
        c->debug_count = (uint32_t)c->debug_pairs.size();
    }
    c->view_recs.resize(c->views.size());
    for (uint32_t vi = 0; vi < c->views.size(); ++vi) {
        const ViewHost& v = c->views[vi];
        ViewRec r{};
        r.width = (int)v.width;
        r.height = (int)v.height;
        r.shadow_w = r.shadow_h = (int)v.shadow;
        r.cull_front = v.dc.cull_enabled ? 1 : 0;
        r.ccw_front = v.dc.reverse_winding_order_enabled ? 1 : 0;
        r.bias_enabled = v.dc.depth_bias_enabled ? 1 : 0;
        r.bias_constant = v.dc.depth_bias_constant;
        r.bias_clamp = v.dc.depth_bias_clamp;
        r.bias_slope = v.dc.depth_bias_slope_factor;
        r.pcf_mode = v.dc.pcf_mode;
        r.cascades = (int)cascades_of(v);
        r.shade_block_base = block_base[vi];
        r.vis = c->d_vis + pix_off[vi] * c->samples;  // `samples` planes of width*height
        r.color = c->d_color + pix_off[vi];
        r.depth = c->d_depth + pix_off[vi];
        r.shadow = c->d_shadow + shadow_off[vi];
        r.color16 = c->d_color16 ? c->d_color16 + pix_off[vi] * c->samples : nullptr;
        r.samples = (int)c->samples;
        r.scene = c->d_scene_data + vi;
        r.gb_albedo = c->gbuffer ? c->d_gb_albedo + pix_off[vi] : nullptr;
        r.gb_normal = c->gbuffer ? c->d_gb_normal + pix_off[vi] : nullptr;
        r.gb_sources = (c->gbuffer && c->samples == 1) ? c->d_gb_sources + pix_off[vi] : nullptr;
        c->view_recs[vi] = r;
    }
    for (int k = 0; k < 2; ++k) dfree(c->d_views_set[k]);
    c->d_views = nullptr;
    dfree(c->d_shadow_draws);
    dfree(c->d_opaque_draws);
    dfree(c->d_blended_draws);
    dfree(c->d_shadow_mvp);
    dfree(c->d_camera_consts);
    dfree(c->d_blended_consts);
    dfree(c->d_varyings);
    dfree(c->d_tri_refs);
    for (int k = 0; k < 2; ++k) RZ_CUDA(c, dalloc(&c->d_views_set[k], c->view_recs.size()), "view table");
    RZ_CUDA(c, dalloc(&c->d_shadow_draws, std::max<size_t>(shadow_list.size(), 1)), "shadow draw list");
    RZ_CUDA(c, dalloc(&c->d_opaque_draws, std::max<size_t>(opaque.size(), 1)), "opaque draw list");
    RZ_CUDA(c, dalloc(&c->d_blended_draws, std::max<size_t>(blended.size(), 1)), "blended draw list");
    RZ_CUDA(c, dalloc(&c->d_shadow_mvp, std::max<size_t>(shadow_list.size(), 1) * 16), "shadow matrices");
    RZ_CUDA(c, dalloc(&c->d_camera_consts, std::max<size_t>(opaque.size(), 1)), "camera constants");
    RZ_CUDA(c, dalloc(&c->d_blended_consts, std::max<size_t>(blended.size(), 1)), "blended constants");
    RZ_CUDA(c, dalloc(&c->d_varyings, std::max<size_t>((size_t)varyings, 1) * 8), "varying records");
    RZ_CUDA(c, dalloc(&c->d_tri_refs, std::max<size_t>((size_t)opaque_tris, 1)), "triangle references");
    for (int k = 0; k < 2; ++k) {
        std::vector<ViewRec> set = c->view_recs;
        for (ViewRec& r : set) {
            r.color += (size_t)k * pix;
            r.depth += (size_t)k * pix;
            r.scene += (size_t)k * c->scene_data_capacity;
        }
        RZ_CUDA(c, cudaMemcpy(c->d_views_set[k], set.data(), set.size() * sizeof(ViewRec), cudaMemcpyHostToDevice),
                "upload views");
    }
    c->d_views = c->d_views_set[0];
    c->parity = 0;
    c->last_parity = 0;
    if (!shadow_list.empty())
        RZ_CUDA(c, cudaMemcpy(c->d_shadow_draws, shadow_list.data(), shadow_list.size() * sizeof(DrawRec), cudaMemcpyHostToDevice), "upload draws");
    if (!opaque.empty())
        RZ_CUDA(c, cudaMemcpy(c->d_opaque_draws, opaque.data(), opaque.size() * sizeof(DrawRec), cudaMemcpyHostToDevice), "upload draws");
    if (!blended.empty())
        RZ_CUDA(c, cudaMemcpy(c->d_blended_draws, blended.data(), blended.size() * sizeof(DrawRec), cudaMemcpyHostToDevice), "upload draws");
    c->shadow_draw_count = (uint32_t)shadow_list.size();
    c->opaque_draw_count = (uint32_t)opaque.size();
    c->blended_draw_count = (uint32_t)blended.size();
    c->shadow_tris = (uint32_t)shadow_tris;
    c->opaque_tris = (uint32_t)opaque_tris;
    c->blended_tris = (uint32_t)blended_tris;
    c->varying_count = (uint32_t)varyings;
    c->blended_varying_base = (uint32_t)blended_varying_base;
    c->pix_total = pix;
    c->shadow_total = shadow;
    c->shade_blocks = blocks;
    int rc = size_pass(c, c->shadow_pass, c->shadow_tris, stamp_hint(c->shadow_tris, shadow));
    if (rc == RZ_OK) rc = size_pass(c, c->camera_pass, c->opaque_tris, stamp_hint(c->opaque_tris, pix));
    if (rc == RZ_OK && c->blended_tris) rc = size_pass(c, c->blended_pass, c->blended_tris, stamp_hint(c->blended_tris, pix));
    if (rc != RZ_OK) return rc;
    c->layout_dirty = false;
    return RZ_OK;
}

PassParams pass_params(rz_ctx* c, int kind) {
    PassParams p{};
    p.pos = c->d_pos;
    p.indices = c->d_indices;
    p.vertex_count = (uint32_t)c->verts.size();
    p.views = c->d_views;
    p.error_flags = kind == 0 ? &c->d_report->shadow_errors : &c->d_report->camera_errors;
    p.chunk_stamps = c->chunk_stamps;
    p.small_extent = c->small_extent;
    p.lookback_spins = c->lookback_spins;
    p.sample_x = 128;  // pixel centre
    p.sample_y = 128;
    p.sample_plane = 0;
    p.bb_hi = (kind != 0 && c->samples > 1) ? 32 : 128;
    PassBuffers* pb;
    if (kind == 2) {  // blended list: cull none, records kept in submission order
        p.draws = c->d_blended_draws;
        p.draw_count = c->blended_draw_count;
        p.tri_total = c->blended_tris;
        p.mvp = reinterpret_cast<const float*>(c->d_blended_consts);
        p.mvp_stride = sizeof(DrawConsts) / sizeof(float);
        p.write_id = 1;
        p.ordered = 1;
        p.header = &c->d_report->blended;
        pb = &c->blended_pass;
    } else if (kind == 1) {
        p.draws = c->d_opaque_draws;
        p.draw_count = c->opaque_draw_count;
        p.tri_total = c->opaque_tris;
        p.mvp = reinterpret_cast<const float*>(c->d_camera_consts);
        p.mvp_stride = sizeof(DrawConsts) / sizeof(float);
        p.write_id = 1;
        p.header = &c->d_report->camera;
        pb = &c->camera_pass;
    } else {
        p.draws = c->d_shadow_draws;
        p.draw_count = c->shadow_draw_count;
        p.tri_total = c->shadow_tris;
        p.mvp = c->d_shadow_mvp;
        p.mvp_stride = 16;
        p.write_id = 0;
        p.header = &c->d_report->shadow;
        pb = &c->shadow_pass;
    }
    p.records = pb->records;
    p.record_capacity = pb->record_capacity;
    p.small_records = pb->small_records;
    p.small_capacity = pb->small_capacity;
    p.tile_status = pb->tile_status;
    p.chunk_map = pb->chunk_map;
    p.chunk_capacity = pb->chunk_capacity;
    p.tri_refs = kind == 1 ? c->d_tri_refs : nullptr;
    return p;
}

ShadeParams shade_params(rz_ctx* c) {
    ShadeParams sh{};
    sh.views = c->d_views;
    sh.view_count = (uint32_t)c->views.size();
    sh.samples = c->samples;
    sh.shade_blocks = c->shade_blocks;
    sh.draws = c->d_opaque_draws;
    sh.draw_count = c->opaque_draw_count;
    sh.consts = c->d_camera_consts;
    sh.varyings = c->d_varyings;
    sh.varying_count = c->blended_varying_base;  // the opaque draws' records
    sh.vertices = c->d_vertices;
    sh.indices = c->d_indices;
    sh.objects = c->d_objects;
    sh.materials = c->d_materials;
    sh.textures = c->d_textures;
    sh.texture_count = (uint32_t)c->tex_descs.size();
    sh.samplers = c->d_samplers;
    sh.sampler_count = (uint32_t)c->samplers.size();
    sh.srgb_table = c->d_srgb;
    sh.tri_refs = c->d_tri_refs;
    sh.blended = (c->blended_tris || c->debug_count) ? 1 : 0;  // k_blend finishes the frame
    return sh;
}

void stamp(rz_ctx* c, int i) {
    if (c->timing) cudaEventRecord(c->stage_ev[i], c->stream);
}

// Shadow passes of all views (src/Engine/Graphics.cpp:5195-5292): clear to 0,
// per-draw matrices, setup, raster.
// The shadow maps are zeroed by the setup launch when there is one (the raster
// follows it), else by the clear launch.
void enqueue_shadow(rz_ctx* c, cudaStream_t s, bool stamps) {
    ClearList cl{};
    cl.ptr[0] = &c->d_report->shadow;  // the shadow header and error word
    cl.bytes[0] = offsetof(FrameReport, camera);
    cl.count = 1;
    if (c->shadow_tris) {
        cl.ptr[1] = c->shadow_pass.tile_status;
        cl.bytes[1] = (size_t)setup_ctas(c->shadow_tris) * 8;
        cl.count = 2;
    } else {
        cl.ptr[1] = c->d_shadow;
        cl.bytes[1] = c->shadow_total * 4;
        cl.count = 2;
    }
    // the per-draw matrices and the clear in one launch
    if (c->shadow_tris) launch_prep(c->d_shadow_draws, c->shadow_draw_count, c->d_objects, c->d_views, c->d_shadow_mvp, s, &cl, c->sm_count);
    else launch_clear(cl, c->sm_count, s);
    if (stamps) stamp(c, 1);
    if (c->shadow_tris) {
        PassParams sp = pass_params(c, 0);
        sp.clear_ptr[0] = c->d_shadow;
        sp.clear_bytes[0] = c->shadow_total * 4;
        sp.clear_count = 1;
        launch_setup(sp, s);
        if (stamps) stamp(c, 2);
        launch_raster(sp, c->sm_count, s);
    } else if (stamps) {
        stamp(c, 2);
    }
}

// Camera passes of all views (5566-5653): visibility cleared to 0, opaque list,
// then the vertex stage of the shading; the blended list's setup.
// The camera raster: one launch per coverage sample, each into its plane of the
// visibility buffer (the setup records are shared).
void launch_camera_raster(rz_ctx* c, PassParams cp, cudaStream_t s) {
    if (c->samples <= 1) {
        launch_raster(cp, c->sm_count, s);
        return;
    }
    for (int k = 0; k < kMsaaSamples; ++k) {
        cp.sample_x = kMsaaX[k];
        cp.sample_y = kMsaaY[k];
        cp.sample_plane = (uint32_t)k;
        launch_raster(cp, c->sm_count, s);
    }
}

// The visibility buffer is zeroed by the opaque setup launch when there is one,
// else by the clear launch.
void enqueue_camera(rz_ctx* c, cudaStream_t s, bool stamps, const ShadeParams& sh) {
    ClearList cl{};
    cl.ptr[0] = &c->d_report->camera;  // the camera and blended headers and their error word
    cl.bytes[0] = sizeof(FrameReport) - offsetof(FrameReport, camera);
    cl.count = 1;
    if (!c->opaque_tris) {
        cl.ptr[cl.count] = c->d_vis;
        cl.bytes[cl.count] = c->pix_total * 8 * c->samples;
        ++cl.count;
    }
    if (c->opaque_tris) {
        cl.ptr[cl.count] = c->camera_pass.tile_status;
        cl.bytes[cl.count] = (size_t)setup_ctas(c->opaque_tris) * 8;
        ++cl.count;
    }
    if (c->blended_tris) {
        cl.ptr[cl.count] = c->blended_pass.tile_status;
        cl.bytes[cl.count] = (size_t)setup_ctas(c->blended_tris) * 8;
        ++cl.count;
    }
    // the per-draw constants and the clear in one launch
    launch_prep_camera(c->d_opaque_draws, c->opaque_draw_count, c->d_objects, c->d_views, c->d_camera_consts, s, &cl, c->sm_count);
    // the vertex stage needs only the per-draw constants: outside stage timing it
    // runs on a branch of its own beside the camera pass's setup and raster
    const bool vtx_branch = !stamps;
    if (vtx_branch) {
        cudaEventRecord(c->vtx_fork, s);
        cudaStreamWaitEvent(c->vtx, c->vtx_fork, 0);
        launch_vertex(sh, c->vtx);
        cudaEventRecord(c->vtx_join, c->vtx);
    }
    if (stamps) stamp(c, 4);
    if (c->opaque_tris) {
        PassParams cp = pass_params(c, 1);
        cp.clear_ptr[0] = c->d_vis;
        cp.clear_bytes[0] = c->pix_total * 8 * c->samples;
        cp.clear_count = 1;
        launch_setup(cp, s);
        cp.clear_count = 0;
        if (stamps) stamp(c, 5);
        launch_camera_raster(c, cp, s);
    } else if (stamps) {
        stamp(c, 5);
    }
    if (vtx_branch) cudaStreamWaitEvent(s, c->vtx_join, 0);
    else launch_vertex(sh, s);
    if (c->blended_tris) {
        launch_prep_camera(c->d_blended_draws, c->blended_draw_count, c->d_objects, c->d_views, c->d_blended_consts, s);
        launch_setup(pass_params(c, 2), s);
        ShadeParams bs = sh;
        bs.draws = c->d_blended_draws;
        bs.draw_count = c->blended_draw_count;
        bs.consts = c->d_blended_consts;
        bs.varying_count = c->varying_count;
        bs.tri_refs = nullptr;
        launch_vertex_range(bs, c->blended_varying_base, s);
    }
}

// Per-view sequential launches: the same kernels, restricted to one view at a
// time (its draws, its pixels, its targets), view after view. This is what the
// batched frame is measured against.
void enqueue_sequential(rz_ctx* c, cudaStream_t s, const ShadeParams& sh) {
    for (uint32_t vi = 0; vi < c->views.size(); ++vi) {
        const rz_ctx::ViewRange& rg = c->ranges[vi];
        ClearList cl{};
        cl.ptr[0] = c->d_shadow + rg.shadow_off;
        cl.bytes[0] = rg.shadow * 4;
        cl.ptr[1] = c->d_vis + rg.pix_off * c->samples;
        cl.bytes[1] = rg.pix * 8 * c->samples;
        cl.ptr[2] = &c->d_report->shadow;  // headers only: the error words hold the whole frame's flags
        cl.bytes[2] = sizeof(PassHeader);
        cl.ptr[3] = &c->d_report->camera;
        cl.bytes[3] = sizeof(PassHeader);
        cl.count = 4;
        if (c->shadow_tris) {
            cl.ptr[4] = c->shadow_pass.tile_status;
            cl.bytes[4] = (size_t)setup_ctas(rg.shadow_tris) * 8;
            cl.count = 5;
        }
        launch_clear(cl, c->sm_count, s);
        if (c->opaque_tris) {
            ClearList c2{};
            c2.ptr[0] = c->camera_pass.tile_status;
            c2.bytes[0] = (size_t)setup_ctas(rg.opaque_tris) * 8;
            c2.count = 1;
            launch_clear(c2, c->sm_count, s);
        }
        if (rg.shadow_tris) {
            PassParams sp = pass_params(c, 0);
            sp.tri_offset = rg.shadow_tri_base;
            sp.tri_total = rg.shadow_tris;
            launch_setup(sp, s);
            launch_raster(sp, c->sm_count, s);
        }
        if (rg.opaque_tris) {
            PassParams cp = pass_params(c, 1);
            cp.tri_offset = rg.opaque_tri_base;
            cp.tri_total = rg.opaque_tris;
            launch_setup(cp, s);
            launch_camera_raster(c, cp, s);
        }
        ShadeParams v = sh;
        v.varying_count = rg.varying_end;
        launch_vertex_range(v, rg.varying_begin, s);
        v.block_offset = rg.block_base;
        v.shade_blocks = rg.blocks;
        launch_shade(v, s);
    }
}

// Enqueues one frame (everything after the scene/object uploads). With stage
// timing the stages run one after the other on the main stream between
// events; otherwise the shadow passes run on a side stream concurrently with
// the camera passes, joining before the shading (which reads the shadow maps),
// and the G-buffer's sub-pixel sources (which read only the visibility) follow
// the shadow passes on the side stream, concurrently with the shading.
int enqueue_frame(rz_ctx* c) {
    cudaStream_t s = c->stream;
    take_launches();  // start this frame's count
    const ShadeParams sh = shade_params(c);
    const bool sources = c->gbuffer && c->samples == 1;  // the learned path's x2 base
    bool sources_side = false;
    if (!c->batched && !c->blended_tris && !c->timing && !c->debug_count) {
        // per-view launches clear the pass headers view by view; the error words once per frame
        RZ_CUDA(c, cudaMemsetAsync(c->d_report, 0, sizeof(FrameReport), s), "clear frame report");
        launch_prep(c->d_shadow_draws, c->shadow_draw_count, c->d_objects, c->d_views, c->d_shadow_mvp, s);
        launch_prep_camera(c->d_opaque_draws, c->opaque_draw_count, c->d_objects, c->d_views, c->d_camera_consts, s);
        enqueue_sequential(c, s, sh);
    } else if (c->timing) {
        stamp(c, 0);
        enqueue_shadow(c, s, true);
        stamp(c, 3);
        enqueue_camera(c, s, true, sh);
        stamp(c, 6);
    } else {
        RZ_CUDA(c, cudaEventRecord(c->fork, s), "fork");
        RZ_CUDA(c, cudaStreamWaitEvent(c->side, c->fork, 0), "fork");
        enqueue_shadow(c, c->side, false);
        enqueue_camera(c, s, false, sh);
        RZ_CUDA(c, cudaEventRecord(c->join, c->side), "join");
        if (sources) {
            RZ_CUDA(c, cudaEventRecord(c->camera_done, s), "camera done");
            RZ_CUDA(c, cudaStreamWaitEvent(c->side, c->camera_done, 0), "camera done");
            launch_subpixel_sources(sh, c->side);
            RZ_CUDA(c, cudaEventRecord(c->sources_done, c->side), "sources done");
            sources_side = true;
        }
        RZ_CUDA(c, cudaStreamWaitEvent(s, c->join, 0), "join");
    }
    if (c->batched || c->blended_tris || c->timing || c->debug_count) launch_shade(sh, s);
    if (sources && !sources_side) launch_subpixel_sources(sh, s);
    if (c->blended_tris || c->debug_count) {
        if (c->debug_count)
            launch_debug_prep(c->d_debug_pairs, c->debug_count, c->d_debug_objects, c->d_views, (uint32_t)c->views.size(),
                              c->d_debug_segs, s);
        BlendParams bp{};
        bp.sh = sh;
        bp.sh.draws = c->d_blended_draws;
        bp.sh.draw_count = c->blended_draw_count;
        bp.sh.consts = c->d_blended_consts;
        bp.sh.tri_refs = nullptr;  // the blended triangles are looked up through their draws
        bp.records = c->blended_pass.records;
        bp.header = &c->d_report->blended;
        bp.error_flags = &c->d_report->camera_errors;
        bp.record_capacity = c->blended_pass.record_capacity;
        bp.debug = c->d_debug_segs;
        bp.debug_count = c->debug_count;
        launch_blend(bp, s);
    }
    if (c->timing) stamp(c, 7);
    if (sources_side) RZ_CUDA(c, cudaStreamWaitEvent(s, c->sources_done, 0), "sources done");
    RZ_CUDA(c, cudaGetLastError(), "kernel launch");
    c->frame_launches = take_launches();
    return RZ_OK;
}

int check_ready(rz_ctx* c) {
    if (!c) return RZ_INVALID_ARGUMENT;
    if (c->scenes.empty()) return fail(c, RZ_INVALID_STATE, "rz_set_asset has not been called");
    for (const ViewHost& v : c->views) {
        if (v.scene >= c->scenes.size()) return fail(c, RZ_INVALID_STATE, "view refers to a missing scene");
        if (!c->scenes[v.scene].has_objects) return fail(c, RZ_INVALID_STATE, "rz_set_objects has not been called");
        if (!v.has_scene_data) return fail(c, RZ_INVALID_STATE, "rz_update has not been called");
    }
    return RZ_OK;
}

// Resizes the raster queues from what an overflowing frame needed (exact counts
// reported by the device), with 25% headroom.
int grow_queues(rz_ctx* c) {
    cudaStreamSynchronize(c->stream);
    cudaEventSynchronize(c->report_done[c->last_parity]);
    drop_graph(c);
    c->queue_chunks = 0;
    auto grow = [&](PassBuffers& p, const PassHeader& h) -> int {
        const uint64_t want_chunks = (h.stamps + c->chunk_stamps - 1) / c->chunk_stamps;
        const uint64_t want_recs = h.records_needed;
        if (want_chunks > p.chunk_capacity) {
            const uint64_t n = std::min<uint64_t>(want_chunks + want_chunks / 4 + 1024, 0xFFFFFFFFull);
            dfree(p.chunk_map);
            p.chunk_capacity = 0;
            RZ_CUDA(c, dalloc(&p.chunk_map, (size_t)n), "chunk map");
            p.chunk_capacity = (uint32_t)n;
        }
        if (want_recs > p.record_capacity) {
            const uint64_t n = std::min<uint64_t>(want_recs + want_recs / 4 + 1024, 0xFFFFFFull);
            dfree(p.records);
            p.record_capacity = 0;
            RZ_CUDA(c, dalloc(&p.records, (size_t)n), "raster records");
            p.record_capacity = (uint32_t)n;
        }
        if (h.small_records > p.small_capacity) {
            const uint64_t n = std::min<uint64_t>((uint64_t)h.small_records + h.small_records / 4 + 1024, 0xFFFFFFFFull);
            dfree(p.small_records);
            p.small_capacity = 0;
            RZ_CUDA(c, dalloc(&p.small_records, (size_t)n), "small raster records");
            p.small_capacity = (uint32_t)n;
        }
        return RZ_OK;
    };
    int rc = grow(c->shadow_pass, c->h_report->shadow);
    if (rc == RZ_OK) rc = grow(c->camera_pass, c->h_report->camera);
    if (rc == RZ_OK && c->blended_tris) rc = grow(c->blended_pass, c->h_report->blended);
    c->grow_records = c->grow_chunks = false;
    return rc;
}

rz_frame_out frame_of(rz_ctx* c, uint32_t v) {
    rz_frame_out o{};
    const ViewRec& r = c->view_recs[v];
    o.color_rgba8 = r.color + (size_t)c->last_parity * c->pix_total;
    o.depth_f32 = r.depth + (size_t)c->last_parity * c->pix_total;
    o.visibility_u64 = r.vis;
    o.shadow_map_f32 = r.shadow;
    o.width = (uint32_t)r.width;
    o.height = (uint32_t)r.height;
    o.shadow_map_size = (uint32_t)r.shadow_w;
    o.triangle_id_base = c->view_id_base[v];
    return o;
}

// The overlay's segments before the vertex stage, in draw order. Vertex table of
// src/Engine/Graphics.cpp:3222-3249: a line (0,0,0)-(0,0,1) at vertices 0-1 and,
// from vertex 8, pairs of unit-circle points at angles step*(i+1) and that plus
// step, step = (float)pi * 4 / 100 in float arithmetic; a circle draws 100
// vertices from 8 (50 segments), a line or cross 2 from 0 (Graphics.cpp:5727-5737).
std::vector<DebugPair> debug_pairs_of(const rz_debug_object* objects, uint32_t count) {
    const float step = (float)3.141592653589793 * 4.0f / 100.0f;
    std::vector<DebugPair> out;
    for (uint32_t o = 0; o < count; ++o) {
        const rz_debug_object& d = objects[o];
        DebugPair p{};
        p.object = o;
        if (d.flags == RZ_DEBUG_TRANSFORM_IS_POINTS) {  // the transform's columns 0 and 1
            for (int k = 0; k < 4; ++k) {
                p.a[k] = d.transform[k];
                p.b[k] = d.transform[4 + k];
            }
            out.push_back(p);
        } else if (d.type == RZ_DEBUG_CIRCLE) {
            for (int i = 0; i < 50; ++i) {
                const float cur = step * (float)(i + 1), next = cur + step;
                p.a[0] = std::sin(cur);
                p.a[1] = std::cos(cur);
                p.a[2] = 0.0f;
                p.a[3] = 1.0f;
                p.b[0] = std::sin(next);
                p.b[1] = std::cos(next);
                p.b[2] = 0.0f;
                p.b[3] = 1.0f;
                out.push_back(p);
            }
        } else {
            p.a[3] = 1.0f;
            p.b[2] = 1.0f;
            p.b[3] = 1.0f;
            out.push_back(p);
        }
    }
    return out;
}

// Polls `done` (a stream or an event query) until it reports completion, an
// error, or timeout_ms runs out (0: no limit).
template <class Query>
int wait_until(rz_ctx* c, Query done, uint32_t timeout_ms, const char* what) {
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const cudaError_t q = done();
        if (q == cudaSuccess) return RZ_OK;
        if (q != cudaErrorNotReady) return cuda_fail(c, q, what);
        if (timeout_ms) {
            const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
            if (ms >= (long long)timeout_ms) return fail(c, RZ_TIMEOUT, std::string(what) + " still running");
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

}  // namespace

extern "C" {

uint32_t rz_abi_version(void) { return RZ_ABI_VERSION; }

int rz_create(rz_ctx** out, const rz_config* cfg) {
    if (!out || !cfg) return RZ_INVALID_ARGUMENT;
    *out = nullptr;
    if (cfg->width == 0 || cfg->height == 0 || cfg->width > 16384 || cfg->height > 16384) return RZ_INVALID_ARGUMENT;
    if (cfg->shadow_map_size == 0 || cfg->shadow_map_size > 16384) return RZ_INVALID_ARGUMENT;
    if (cfg->samples != 1 && cfg->samples != (uint32_t)kMsaaSamples) return RZ_INVALID_ARGUMENT;
    rz_ctx* c = new rz_ctx();
    c->device = cfg->device;
    c->samples = cfg->samples;
    c->queue_chunks = cfg->queue_chunks;
    auto bail = [&](int code) {
        rz_destroy(c);
        return code;
    };
    if (cudaSetDevice(c->device) != cudaSuccess) return bail(RZ_GRAPHICS_INIT_FAILURE);
    if (cudaDeviceGetAttribute(&c->sm_count, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess)
        return bail(RZ_GRAPHICS_INIT_FAILURE);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->vtx, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->vtx_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->vtx_join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->camera_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->sources_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking) != cudaSuccess)
        return bail(RZ_GRAPHICS_INIT_FAILURE);
    for (int k = 0; k < 2; ++k)
        if (cudaEventCreateWithFlags(&c->read_done[k], cudaEventDisableTiming) != cudaSuccess)
            return bail(RZ_GRAPHICS_INIT_FAILURE);
    if (cudaEventCreateWithFlags(&c->frame_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaStreamCreateWithFlags(&c->upload, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->upload_done[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->upload_done[1], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->set_done[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->set_done[1], cudaEventDisableTiming) != cudaSuccess)
        return bail(RZ_GRAPHICS_INIT_FAILURE);
    if (dalloc(&c->d_report_base, 2) != cudaSuccess || cudaMemset(c->d_report_base, 0, 2 * sizeof(FrameReport)) != cudaSuccess ||
        dalloc(&c->d_srgb, 256) != cudaSuccess)
        return bail(RZ_ALLOCATION_FAILURE);
    if (cudaMallocHost(&c->h_report_base, 2 * sizeof(FrameReport)) != cudaSuccess) return bail(RZ_ALLOCATION_FAILURE);
    std::memset(c->h_report_base, 0, 2 * sizeof(FrameReport));
    c->d_report = c->d_report_base;
    c->h_report = c->h_report_base;
    for (int k = 0; k < 2; ++k)
        if (cudaEventCreateWithFlags(&c->report_done[k], cudaEventDisableTiming) != cudaSuccess)
            return bail(RZ_GRAPHICS_INIT_FAILURE);
    // sRGB decode table (colour, metallic-roughness and mixmap images are sRGB
    // formats, src/Engine/Graphics.cpp:3632-3647): IEC 61966-2-1 in double, rounded to float.
    float table[256];
    for (int i = 0; i < 256; ++i) {
        const double v = i / 255.0;
        table[i] = (float)(v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4));
    }
    if (cudaMemcpy(c->d_srgb, table, sizeof(table), cudaMemcpyHostToDevice) != cudaSuccess) return bail(RZ_ERROR);
    // view 0 with the reference defaults (src/Engine/Level.cpp:1246-1255)
    ViewHost v;
    v.scene = 0;
    v.width = cfg->width;
    v.height = cfg->height;
    v.shadow = cfg->shadow_map_size;
    v.dc.cull_enabled = 1;
    v.dc.reverse_winding_order_enabled = 0;
    v.dc.depth_bias_enabled = 1;
    v.dc.depth_bias_constant = -21.882f;
    v.dc.depth_bias_clamp = -20.937f;
    v.dc.depth_bias_slope_factor = -3.0f;
    v.dc.pcf_mode = RZ_PCF_5TAP;
    c->views.push_back(v);
    if (ensure_scene_data(c, 1) != RZ_OK) return bail(RZ_ALLOCATION_FAILURE);
    const char* g = std::getenv("RZ_NO_GRAPH");
    c->use_graph = !(g && g[0] == '1');
    *out = c;
    return RZ_OK;
}

void rz_destroy(rz_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->side) cudaStreamSynchronize(c->side);
    if (c->vtx) cudaStreamSynchronize(c->vtx);
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
    if (c->upload) cudaStreamSynchronize(c->upload);
    drop_graph(c);
    free_asset(c);
    free_pass(c->shadow_pass);
    free_pass(c->camera_pass);
    free_pass(c->blended_pass);
    dfree(c->d_vertices);
    dfree(c->d_pos);
    dfree(c->d_indices);
    dfree(c->d_materials);
    dfree(c->d_textures);
    dfree(c->d_samplers);
    dfree(c->d_objects_base);
    c->d_objects = nullptr;
    dfree(c->d_srgb);
    dfree(c->d_scene_data);
    for (int k = 0; k < 2; ++k) dfree(c->d_views_set[k]);
    dfree(c->d_vis);
    dfree(c->d_color);
    dfree(c->d_depth);
    dfree(c->d_shadow);
    dfree(c->d_color16);
    dfree(c->d_debug_objects);
    dfree(c->d_debug_pairs);
    dfree(c->d_debug_segs);
    dfree(c->d_gb_albedo);
    dfree(c->d_gb_normal);
    dfree(c->d_gb_sources);
    dfree(c->d_shadow_draws);
    dfree(c->d_opaque_draws);
    dfree(c->d_blended_draws);
    dfree(c->d_shadow_mvp);
    dfree(c->d_camera_consts);
    dfree(c->d_blended_consts);
    dfree(c->d_varyings);
    dfree(c->d_tri_refs);
    dfree(c->d_report_base);
    c->d_report = nullptr;
    if (c->h_scene_data) cudaFreeHost(c->h_scene_data);
    if (c->h_report_base) cudaFreeHost(c->h_report_base);
    c->h_report = nullptr;
    for (int k = 0; k < 2; ++k)
        if (c->report_done[k]) cudaEventDestroy(c->report_done[k]);
    if (c->h_objects) cudaFreeHost(c->h_objects);
    if (c->frame_done) cudaEventDestroy(c->frame_done);
    for (auto& e : c->stage_ev)
        if (e) cudaEventDestroy(e);
    for (int k = 0; k < 2; ++k) {
        if (c->upload_done[k]) cudaEventDestroy(c->upload_done[k]);
        if (c->set_done[k]) cudaEventDestroy(c->set_done[k]);
    }
    if (c->upload) cudaStreamDestroy(c->upload);
    if (c->fork) cudaEventDestroy(c->fork);
    if (c->vtx_fork) cudaEventDestroy(c->vtx_fork);
    if (c->vtx_join) cudaEventDestroy(c->vtx_join);
    if (c->join) cudaEventDestroy(c->join);
    if (c->camera_done) cudaEventDestroy(c->camera_done);
    if (c->sources_done) cudaEventDestroy(c->sources_done);
    if (c->copy_stream) cudaStreamSynchronize(c->copy_stream);
    for (int k = 0; k < 2; ++k) {
        if (c->read_done[k]) cudaEventDestroy(c->read_done[k]);
    }
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->vtx) cudaStreamDestroy(c->vtx);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int rz_resize(rz_ctx* c, uint32_t width, uint32_t height) {
    if (!c) return RZ_INVALID_ARGUMENT;
    if (width == 0 || height == 0 || width > 16384 || height > 16384) return fail(c, RZ_INVALID_ARGUMENT, "bad extent");
    c->views[0].width = width;
    c->views[0].height = height;
    c->layout_dirty = true;
    return RZ_OK;
}

int rz_set_asset(rz_ctx* c, const rz_mesh* meshes, uint32_t mesh_count, const rz_material* mats, uint32_t mat_count,
                 const rz_texture* textures, uint32_t tex_count, const rz_sampler* samplers, uint32_t sampler_count) {
    if (!c) return RZ_INVALID_ARGUMENT;
    if (mesh_count == 0 || !meshes) return fail(c, RZ_INVALID_ARGUMENT, "asset has no meshes");
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    drop_graph(c);
    free_asset(c);
    SceneHost sh;
    const int rc = append_asset(c, meshes, mesh_count, mats, mat_count, textures, tex_count, samplers, sampler_count, sh);
    if (rc != RZ_OK) {
        free_asset(c);
        return rc;
    }
    c->scenes.push_back(sh);
    return upload_asset(c);
}

int rz_set_objects(rz_ctx* c, const rz_object* objects, uint32_t object_count, const rz_surface* surfaces,
                   uint32_t surface_count) {
    if (!c) return RZ_INVALID_ARGUMENT;
    if (c->scenes.empty()) return fail(c, RZ_INVALID_STATE, "rz_set_asset has not been called");
    // src/Engine/Graphics.cpp:4693-4697: an empty scene is an invalid argument
    if (object_count == 0 || !objects || surface_count == 0 || !surfaces) return fail(c, RZ_INVALID_ARGUMENT, "empty scene");
    if (c->scenes.size() != 1) return fail(c, RZ_INVALID_STATE, "rz_set_objects applies to a single-scene context");
    SceneHost& sh = c->scenes[0];
    const int rc = check_surfaces(c, sh, object_count, surfaces, surface_count);
    if (rc != RZ_OK) return rc;
    cudaSetDevice(c->device);
    c->objects.assign(objects, objects + object_count);
    sh.object_base = 0;
    sh.object_count = object_count;
    sh.surfaces.assign(surfaces, surfaces + surface_count);
    sh.has_objects = true;
    return upload_objects(c);
}

int rz_add_scene(rz_ctx* c, const rz_mesh* meshes, uint32_t mesh_count, const rz_material* mats, uint32_t mat_count,
                 const rz_texture* textures, uint32_t tex_count, const rz_sampler* samplers, uint32_t sampler_count,
                 const rz_object* objects, uint32_t object_count, const rz_surface* surfaces, uint32_t surface_count,
                 uint32_t* scene_index) {
    if (!c) return RZ_INVALID_ARGUMENT;
    if (object_count == 0 || !objects || surface_count == 0 || !surfaces) return fail(c, RZ_INVALID_ARGUMENT, "empty scene");
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    drop_graph(c);
    // roll back the host arrays if the asset or its surfaces are rejected
    const size_t nv = c->verts.size(), ni = c->idx.size(), nm = c->mesh_table.size(), nmat = c->materials.size();
    const size_t ntex = c->tex_descs.size(), nsmp = c->samplers.size();
    auto rollback = [&]() {
        for (size_t i = ntex; i < c->tex_allocs.size(); ++i) cudaFree(c->tex_allocs[i]);
        c->tex_allocs.resize(ntex);
        c->verts.resize(nv);
        c->pos.resize(nv);
        c->idx.resize(ni);
        c->mesh_table.resize(nm);
        c->materials.resize(nmat);
        c->tex_descs.resize(ntex);
        c->samplers.resize(nsmp);
    };
    SceneHost sh;
    int rc = append_asset(c, meshes, mesh_count, mats, mat_count, textures, tex_count, samplers, sampler_count, sh);
    if (rc == RZ_OK) rc = check_surfaces(c, sh, object_count, surfaces, surface_count);
    if (rc != RZ_OK) {
        rollback();
        return rc;
    }
    sh.object_base = (uint32_t)c->objects.size();
    sh.object_count = object_count;
    c->objects.insert(c->objects.end(), objects, objects + object_count);
    sh.surfaces.assign(surfaces, surfaces + surface_count);
    sh.has_objects = true;
    c->scenes.push_back(sh);
    if (scene_index) *scene_index = (uint32_t)(c->scenes.size() - 1);
    rc = upload_asset(c);
    if (rc == RZ_OK) rc = upload_objects(c);
    return rc;
}

int rz_set_views(rz_ctx* c, const rz_view* views, uint32_t count) {
    if (!c || !views || count == 0) return RZ_INVALID_ARGUMENT;
    for (uint32_t i = 0; i < count; ++i) {
        const rz_view& v = views[i];
        if (v.width == 0 || v.height == 0 || v.width > 16384 || v.height > 16384 || v.shadow_map_size == 0 ||
            v.shadow_map_size > 16384)
            return fail(c, RZ_INVALID_ARGUMENT, "bad view extent");
        if (v.draw_config.pcf_mode > RZ_PCF_3X3) return fail(c, RZ_INVALID_ARGUMENT, "unknown pcf mode");
        if (v.scene >= c->scenes.size()) return fail(c, RZ_INVALID_ARGUMENT, "view refers to a missing scene");
    }
    cudaSetDevice(c->device);
    const int rc = ensure_scene_data(c, count);
    if (rc != RZ_OK) return rc;
    std::vector<ViewHost> vs(count);
    for (uint32_t i = 0; i < count; ++i) {
        vs[i].scene = views[i].scene;
        vs[i].width = views[i].width;
        vs[i].height = views[i].height;
        vs[i].shadow = views[i].shadow_map_size;
        vs[i].dc = views[i].draw_config;
        vs[i].has_scene_data = i < c->views.size() ? c->views[i].has_scene_data : false;
    }
    c->views = vs;
    c->layout_dirty = true;
    return RZ_OK;
}

int rz_update_objects(rz_ctx* c, uint32_t offset, const rz_object* objects, uint32_t count) {
    if (!c) return RZ_INVALID_ARGUMENT;
    if (c->scenes.empty() || !c->scenes[0].has_objects) return fail(c, RZ_INVALID_STATE, "rz_set_objects has not been called");
    if (count == 0) return RZ_OK;
    const SceneHost& sh = c->scenes[0];
    if (!objects || (uint64_t)offset + count > sh.object_count) return fail(c, RZ_INVALID_ARGUMENT, "object range");
    cudaSetDevice(c->device);
    // the staging is copied to the device before each frame (rz_render); the
    // copies queued so far have read it before it changes
    RZ_CUDA(c, wait_uploads(c), "wait staging");
    const uint32_t at = sh.object_base + offset;
    std::memcpy(c->h_objects + at, objects, (size_t)count * sizeof(rz_object));
    std::memcpy(c->objects.data() + at, objects, (size_t)count * sizeof(rz_object));
    ++c->objects_version;
    return RZ_OK;
}

int rz_set_draw_config(rz_ctx* c, const rz_draw_config* cfg) {
    if (!c || !cfg) return RZ_INVALID_ARGUMENT;
    if (cfg->pcf_mode > RZ_PCF_3X3) return fail(c, RZ_INVALID_ARGUMENT, "unknown pcf mode");
    c->views[0].dc = *cfg;
    c->layout_dirty = true;
    return RZ_OK;
}

int rz_update_view(rz_ctx* c, uint32_t view, const rz_scene_data* scene) {
    if (!c || !scene) return RZ_INVALID_ARGUMENT;
    if (view >= c->views.size()) return fail(c, RZ_INVALID_ARGUMENT, "no such view");
    cudaSetDevice(c->device);
    RZ_CUDA(c, wait_uploads(c), "wait staging");
    std::memcpy(c->h_scene_data + view, scene, sizeof(rz_scene_data));
    ++c->scene_version;
    c->views[view].has_scene_data = true;
    return RZ_OK;
}

int rz_update(rz_ctx* c, const rz_scene_data* scene) { return rz_update_view(c, 0, scene); }

// Copies the staged object records and scene constants into target set k when
// they changed since set k's last frame, on the upload stream once that frame is
// done, and makes the frame stream wait for the copy.
int upload_set(rz_ctx* c, uint32_t k) {
    const bool objs = c->set_objects_version[k] != c->objects_version;
    const bool scene = c->set_scene_version[k] != c->scene_version;
    if (!objs && !scene) return RZ_OK;
    RZ_CUDA(c, cudaStreamWaitEvent(c->upload, c->set_done[k], 0), "set free");
    const size_t n = c->objects.size();
    if (objs && n)
        RZ_CUDA(c, cudaMemcpyAsync(c->d_objects_base + (size_t)k * n, c->h_objects, n * sizeof(rz_object),
                                   cudaMemcpyHostToDevice, c->upload), "upload objects");
    if (scene)
        RZ_CUDA(c, cudaMemcpyAsync(c->d_scene_data + (size_t)k * c->scene_data_capacity, c->h_scene_data,
                                   c->views.size() * sizeof(rz_scene_data), cudaMemcpyHostToDevice, c->upload),
                "upload scene");
    RZ_CUDA(c, cudaEventRecord(c->upload_done[k], c->upload), "uploaded");
    RZ_CUDA(c, cudaStreamWaitEvent(c->stream, c->upload_done[k], 0), "wait upload");
    c->set_objects_version[k] = c->objects_version;
    c->set_scene_version[k] = c->scene_version;
    return RZ_OK;
}

// After a frame is enqueued: its completion event, and the next frame's target set.
int frame_enqueued(rz_ctx* c) {
    const uint32_t k = c->parity;
    RZ_CUDA(c, cudaEventRecord(c->set_done[k], c->stream), "record set");
    // the frame report to the host, off the frame stream (on the copy stream: the
    // upload stream's next copy must not wait for this frame's end)
    RZ_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->set_done[k], 0), "frame before its report");
    RZ_CUDA(c, cudaMemcpyAsync(c->h_report_base + k, c->d_report_base + k, sizeof(FrameReport), cudaMemcpyDeviceToHost,
                               c->copy_stream), "read frame report");
    RZ_CUDA(c, cudaEventRecord(c->report_done[k], c->copy_stream), "report read");
    c->report_issued[k] = true;
    c->h_report = c->h_report_base + k;
    RZ_CUDA(c, cudaEventRecord(c->frame_done, c->stream), "record frame");
    c->frame_pending = true;
    ++c->frames;
    c->last_parity = c->parity;
    c->parity ^= 1u;
    return RZ_OK;
}

int rz_render(rz_ctx* c) {
    const int ready = check_ready(c);
    if (ready != RZ_OK) return ready;
    cudaSetDevice(c->device);
    if (c->asset_dirty) {
        const int rc = upload_asset(c);
        if (rc != RZ_OK) return rc;
    }
    if (c->layout_dirty) {
        const int rc = build_layout(c);
        if (rc != RZ_OK) return rc;
    }
    if (c->grow_records || c->grow_chunks) {
        const int rc = grow_queues(c);
        if (rc != RZ_OK) return rc;
    }
    // The frame renders into target set `parity`: the read-back of the frame that
    // last rendered there has to have landed first.
    if (c->read_issued[c->parity])
        RZ_CUDA(c, cudaStreamWaitEvent(c->stream, c->read_done[c->parity], 0), "read-back of the target set");
    c->d_views = c->d_views_set[c->parity];
    c->d_objects = c->d_objects_base + (size_t)c->parity * c->objects.size();
    c->d_report = c->d_report_base + c->parity;
    // the frame zeroes its set's report: the copy of its previous contents has landed
    if (c->report_issued[c->parity])
        RZ_CUDA(c, cudaStreamWaitEvent(c->stream, c->report_done[c->parity], 0), "report of the target set");
    {
        const int rc = upload_set(c, c->parity);
        if (rc != RZ_OK) return rc;
    }
    cudaGraphExec_t& graph = c->graph_set[c->parity];
    // Stage timing records events between the stages and enqueues directly.
    if (c->use_graph && !c->timing) {
        if (!graph) {
            cudaGraph_t g = nullptr;
            RZ_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
            const int rc = enqueue_frame(c);
            const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
            if (rc != RZ_OK) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            cudaError_t ie = e;
            if (e == cudaSuccess) ie = cudaGraphInstantiate(&graph, g, 0);
            if (g) cudaGraphDestroy(g);
            if (ie != cudaSuccess) {
                // capture of this frame shape is not supported here: enqueue directly from now on
                cudaGetLastError();
                graph = nullptr;
                c->use_graph = false;
                const int rc2 = enqueue_frame(c);
                if (rc2 != RZ_OK) return rc2;
                return frame_enqueued(c);
            }
            c->graph_dirty = false;
        }
        RZ_CUDA(c, cudaGraphLaunch(graph, c->stream), "launch frame graph");
    } else {
        const int rc = enqueue_frame(c);
        if (rc != RZ_OK) return rc;
    }
    return frame_enqueued(c);
}

int rz_sync(rz_ctx* c, uint32_t timeout_ms) {
    if (!c) return RZ_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    const auto t0 = std::chrono::steady_clock::now();
    int rc = wait_until(c, [&] { return cudaStreamQuery(c->stream); }, timeout_ms, "frame");
    if (rc != RZ_OK) return rc;
    if (c->reads_issued) {  // and the read-backs queued so far
        uint32_t left = 0;
        if (timeout_ms) {
            const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
            left = ms >= (long long)timeout_ms ? 1u : timeout_ms - (uint32_t)ms;
        }
        rc = wait_until(c, [&] { return cudaStreamQuery(c->copy_stream); }, left, "frame read-back");
        if (rc != RZ_OK) return rc;
    }
    if (!c->frame_pending) return RZ_OK;
    {  // and the last frame's report
        uint32_t left = 0;
        if (timeout_ms) {
            const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
            left = ms >= (long long)timeout_ms ? 1u : timeout_ms - (uint32_t)ms;
        }
        rc = wait_until(c, [&] { return cudaEventQuery(c->report_done[c->last_parity]); }, left, "frame report");
        if (rc != RZ_OK) return rc;
    }
    c->frame_pending = false;
    const uint32_t e = c->h_report->errors();
    if (e & (kErrRecordOverflow)) c->grow_records = true;
    if (e & (kErrStampOverflow)) c->grow_chunks = true;
    if (e & (kErrRecordOverflow | kErrStampOverflow))
        return fail(c, RZ_OVERFLOW, "raster work queue overflowed; capacity grows for the next frame");
    if (e) return fail(c, RZ_GRAPHICS_FRAME_FAILURE, "device error flags " + std::to_string(e));
    return RZ_OK;
}

int rz_get_view_frame(rz_ctx* c, uint32_t view, rz_frame_out* out) {
    if (!c || !out) return RZ_INVALID_ARGUMENT;
    if (c->layout_dirty || view >= c->view_recs.size()) return fail(c, RZ_INVALID_STATE, "no rendered frame for this view");
    *out = frame_of(c, view);
    return RZ_OK;
}

int rz_get_frame(rz_ctx* c, rz_frame_out* out) { return rz_get_view_frame(c, 0, out); }

int rz_set_debug_objects(rz_ctx* c, const rz_debug_object* objects, uint32_t count) {
    if (!c) return RZ_INVALID_ARGUMENT;
    if (count && !objects) return fail(c, RZ_INVALID_ARGUMENT, "null debug objects with a non-zero count");
    if (count > RZ_MAX_DEBUG_OBJECTS) return fail(c, RZ_INVALID_ARGUMENT, "too many debug objects");
    for (uint32_t i = 0; i < count; ++i) {
        if (objects[i].type > RZ_DEBUG_CROSS) return fail(c, RZ_INVALID_ARGUMENT, "unknown debug object type");
        // a circle's vertex ids (8-107) index past the transform's four points
        if (objects[i].flags == RZ_DEBUG_TRANSFORM_IS_POINTS && objects[i].type == RZ_DEBUG_CIRCLE)
            return fail(c, RZ_INVALID_ARGUMENT, "a circle cannot take its points from the transform");
    }
    std::vector<DebugPair> pairs = debug_pairs_of(objects, count);
    cudaSetDevice(c->device);
    const bool same_shape = !c->layout_dirty && c->debug_count != 0 && count == c->debug_objects.size() &&
                            pairs.size() == c->debug_pairs.size();
    const bool was_on = !c->debug_pairs.empty();
    c->debug_objects.assign(objects, objects + count);
    c->debug_pairs = std::move(pairs);
    if (same_shape) {
        // same buffers: the new contents follow the frames already enqueued on the stream
        RZ_CUDA(c, cudaMemcpyAsync(c->d_debug_objects, c->debug_objects.data(), count * sizeof(rz_debug_object),
                                   cudaMemcpyHostToDevice, c->stream), "upload overlay objects");
        RZ_CUDA(c, cudaMemcpyAsync(c->d_debug_pairs, c->debug_pairs.data(), c->debug_pairs.size() * sizeof(DebugPair),
                                   cudaMemcpyHostToDevice, c->stream), "upload overlay vertices");
        return RZ_OK;
    }
    if (was_on || count) c->layout_dirty = true;  // new buffers and frame graph at the next rz_render
    return RZ_OK;
}

int rz_set_gbuffer(rz_ctx* c, uint32_t enable) {
    if (!c) return RZ_INVALID_ARGUMENT;
    if (c->frame_pending) return fail(c, RZ_INVALID_STATE, "a frame is in flight; call rz_sync first");
    if ((enable != 0) != c->gbuffer) {
        c->gbuffer = enable != 0;
        c->layout_dirty = true;
        drop_graph(c);
    }
    return RZ_OK;
}

int rz_get_view_gbuffer(rz_ctx* c, uint32_t view, rz_gbuffer* out) {
    if (!c || !out) return RZ_INVALID_ARGUMENT;
    if (!c->gbuffer) return fail(c, RZ_INVALID_STATE, "G-buffer output is off (rz_set_gbuffer)");
    if (c->layout_dirty || view >= c->view_recs.size()) return fail(c, RZ_INVALID_STATE, "no rendered frame for this view");
    const ViewRec& r = c->view_recs[view];
    rz_gbuffer g{};
    g.color_rgba8 = r.color + (size_t)c->last_parity * c->pix_total;
    g.depth_f32 = r.depth + (size_t)c->last_parity * c->pix_total;
    g.albedo_rgba8 = r.gb_albedo;
    g.normal_oct_f16x2 = r.gb_normal;
    g.sources_u16 = r.gb_sources;
    g.width = (uint32_t)r.width;
    g.height = (uint32_t)r.height;
    *out = g;
    return RZ_OK;
}

int rz_read_frame(rz_ctx* c, void* color_host, size_t color_bytes, void* depth_host, size_t depth_bytes) {
    if (!c) return RZ_INVALID_ARGUMENT;
    if (c->layout_dirty || c->view_recs.empty()) return fail(c, RZ_INVALID_STATE, "no rendered frame");
    const ViewRec& r = c->view_recs[0];
    const size_t need = (size_t)r.width * r.height * 4;
    if ((color_host && color_bytes < need) || (depth_host && depth_bytes < need))
        return fail(c, RZ_INVALID_ARGUMENT, "host buffer too small");
    cudaSetDevice(c->device);
    if (!color_host && !depth_host) return RZ_OK;
    // the last frame's images, straight from its target set, on the copy stream
    // after the frame; the frame after next, which renders into the same set,
    // waits for this read-back (rz_render)
    const uint32_t set = c->last_parity;
    const size_t off = (size_t)set * c->pix_total;
    RZ_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->frame_done, 0), "frame before its read-back");
    if (color_host)
        RZ_CUDA(c, cudaMemcpyAsync(color_host, r.color + off, need, cudaMemcpyDeviceToHost, c->copy_stream), "read colour");
    if (depth_host)
        RZ_CUDA(c, cudaMemcpyAsync(depth_host, r.depth + off, need, cudaMemcpyDeviceToHost, c->copy_stream), "read depth");
    RZ_CUDA(c, cudaEventRecord(c->read_done[set], c->copy_stream), "read done");
    c->read_issued[set] = true;
    c->read_newest = set;
    ++c->reads_issued;
    return RZ_OK;
}

int rz_read_sync(rz_ctx* c, uint32_t pending, uint32_t timeout_ms) {
    if (!c || pending > 1) return RZ_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    if (pending == 0 || c->reads_issued == 0)
        return wait_until(c, [&] { return cudaStreamQuery(c->copy_stream); }, timeout_ms, "frame read-back");
    if (c->reads_issued < 2) return RZ_OK;  // at most one read-back was ever queued
    // all but the newest: the copy stream runs the read-backs in order, so they
    // have all landed once the last read-back of the other target set has
    const uint32_t older = c->read_newest ^ 1u;
    if (!c->read_issued[older]) return RZ_OK;
    return wait_until(c, [&] { return cudaEventQuery(c->read_done[older]); }, timeout_ms, "frame read-back");
}

int rz_get_stats(rz_ctx* c, rz_stats* out) {
    if (!c || !out) return RZ_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    cudaSetDevice(c->device);
    cudaEventSynchronize(c->report_done[c->last_parity]);  // the last frame's report has landed
    out->draw_call_count = c->shadow_draw_count + c->opaque_draw_count + c->blended_draw_count;
    out->triangle_count = c->shadow_tris + c->opaque_tris + c->blended_tris;
    out->shadow_setup_records = c->h_report->shadow.records + c->h_report->shadow.small_records;
    out->camera_setup_records = c->h_report->camera.records + c->h_report->camera.small_records;
    out->shadow_stamps = c->h_report->shadow.stamps;
    out->camera_stamps = c->h_report->camera.stamps;
    out->error_flags = c->h_report->errors();
    out->kernel_launches = c->frame_launches;  // counted by the launchers as the frame was enqueued
    return RZ_OK;
}

int rz_set_stage_timing(rz_ctx* c, uint32_t enable) {
    if (!c) return RZ_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    if (enable && !c->stage_ev[0]) {
        for (auto& e : c->stage_ev) RZ_CUDA(c, cudaEventCreate(&e), "create stage event");
    }
    c->timing = enable != 0;
    drop_graph(c);
    return RZ_OK;
}

int rz_get_stage_times(rz_ctx* c, float* ms, uint32_t capacity, uint32_t* count) {
    if (!c || (!ms && capacity)) return RZ_INVALID_ARGUMENT;
    if (!c->timing || !c->frames) return fail(c, RZ_INVALID_STATE, "stage timing is off or no frame was rendered");
    const uint32_t n = capacity < RZ_STAGE_COUNT ? capacity : RZ_STAGE_COUNT;
    for (uint32_t i = 0; i < n; ++i) {
        float t = 0.0f;
        RZ_CUDA(c, cudaEventElapsedTime(&t, c->stage_ev[i], c->stage_ev[i + 1]), "stage time");
        ms[i] = t;
    }
    if (count) *count = n;
    return RZ_OK;
}

int rz_set_tuning(rz_ctx* c, const rz_tuning* t) {
    if (!c || !t) return RZ_INVALID_ARGUMENT;
    if (t->chunk_stamps < 8 || t->chunk_stamps > 256 || t->small_extent < 1 || t->small_extent > (uint32_t)kMaxSmallExtent)
        return fail(c, RZ_INVALID_ARGUMENT, "tuning out of range");
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    const bool resize = t->chunk_stamps != c->chunk_stamps || t->queue_chunks != c->queue_chunks;
    c->chunk_stamps = t->chunk_stamps;
    c->small_extent = t->small_extent;
    c->queue_chunks = t->queue_chunks;
    c->batched = t->batched != 0;
    if (resize) {
        // re-size the chunk maps for the new chunk size / depth
        free_pass(c->shadow_pass);
        free_pass(c->camera_pass);
        free_pass(c->blended_pass);
        c->layout_dirty = true;
    }
    drop_graph(c);
    return RZ_OK;
}

int rz_set_wait_limit(rz_ctx* c, uint32_t lookback_spins) {
    if (!c) return RZ_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    c->lookback_spins = lookback_spins ? lookback_spins : kLookbackSpins;
    drop_graph(c);  // the limit is a kernel argument captured in the frame graph
    return RZ_OK;
}

int rz_get_tuning(rz_ctx* c, rz_tuning* t) {
    if (!c || !t) return RZ_INVALID_ARGUMENT;
    t->chunk_stamps = c->chunk_stamps;
    t->small_extent = c->small_extent;
    t->queue_chunks = c->queue_chunks;
    t->batched = c->batched ? 1u : 0u;
    return RZ_OK;
}

int rz_autotune(rz_ctx* c, uint32_t frames, rz_tuning* chosen, float* ms, uint32_t capacity) {
    if (!c || frames == 0) return RZ_INVALID_ARGUMENT;
    const uint32_t chunk_opts[3] = {16, 32, 64};
    const uint32_t small_opts[3] = {4, 8, 12};
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    RZ_CUDA(c, cudaEventCreate(&e0), "event");
    RZ_CUDA(c, cudaEventCreate(&e1), "event");
    rz_tuning base{};
    rz_get_tuning(c, &base);
    float best = 1e30f;
    rz_tuning best_t = base;
    int rc = RZ_OK;
    uint32_t n = 0;
    for (uint32_t a = 0; a < 3 && rc == RZ_OK; ++a) {
        for (uint32_t b = 0; b < 3 && rc == RZ_OK; ++b) {
            rz_tuning t = base;
            t.chunk_stamps = chunk_opts[a];
            t.small_extent = small_opts[b];
            t.queue_chunks = 0;
            rc = rz_set_tuning(c, &t);
            if (rc != RZ_OK) break;
            // warm-up (also grows the queues if they overflow)
            for (int w = 0; w < 2 && rc == RZ_OK; ++w) {
                rc = rz_render(c);
                if (rc == RZ_OK) {
                    const int s = rz_sync(c, 0);
                    if (s != RZ_OK && s != RZ_OVERFLOW) rc = s;
                }
            }
            if (rc != RZ_OK) break;
            cudaEventRecord(e0, c->stream);
            for (uint32_t f = 0; f < frames && rc == RZ_OK; ++f) rc = rz_render(c);
            cudaEventRecord(e1, c->stream);
            if (rc == RZ_OK) rc = rz_sync(c, 0);
            float t_ms = 0.0f;
            cudaEventElapsedTime(&t_ms, e0, e1);
            t_ms /= (float)frames;
            if (ms && n < capacity) ms[n] = t_ms;
            ++n;
            if (rc == RZ_OK && t_ms < best) {
                best = t_ms;
                best_t = t;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const int r2 = rz_set_tuning(c, &best_t);
    if (chosen) *chosen = best_t;
    return rc != RZ_OK ? rc : r2;
}

void* rz_get_stream(rz_ctx* c) { return c ? (void*)c->stream : nullptr; }

const char* rz_last_error(rz_ctx* c) { return c ? c->last_error.c_str() : "null context"; }

}  // extern "C"
