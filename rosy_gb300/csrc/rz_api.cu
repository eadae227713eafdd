// Host side of the C ABI (include/rosy_gb300.h): the headless replacement of
// Rosy's graphics_device for the shadow pass + scene pass. One CUDA stream per
// context stands in for the Vulkan queue and its command buffer; a frame is a
// fixed sequence of clears and kernels that is captured once into a CUDA graph
// and replayed until the scene layout changes.
#include <chrono>
#include <cmath>
#include <cstdio>
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

// Host mirror of the device-side frame report (copied back at the end of each frame).
struct FrameReport {
    uint32_t error_flags;
    uint32_t pad;
    PassHeader shadow;
    PassHeader camera;
    PassHeader blended;
};

}  // namespace

struct rz_ctx {
    int device = 0;
    int sm_count = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t side = nullptr;          // shadow pass branch of the frame graph
    cudaEvent_t fork = nullptr, join = nullptr;
    uint32_t width = 0, height = 0, shadow_size = 0;
    uint32_t queue_chunks = 0;  // fixed work-queue depth (0 = sized from the scene)
    std::string last_error;

    // frame buffers
    uint64_t* d_vis = nullptr;
    uint32_t* d_color = nullptr;
    float* d_depth = nullptr;
    uint32_t* d_shadow = nullptr;

    // scene constants
    rz_scene_data* d_scene = nullptr;
    rz_scene_data* h_scene = nullptr;  // pinned staging
    cudaEvent_t scene_copied = nullptr;
    bool have_scene = false;
    rz_draw_config draw_config{};

    // asset
    rz_vertex* d_vertices = nullptr;
    float4* d_pos = nullptr;
    uint32_t vertex_count = 0;
    uint32_t* d_indices = nullptr;
    uint32_t index_count = 0;
    std::vector<uint32_t> mesh_table;  // 4 per mesh
    std::vector<uint32_t> mesh_vertex_max;  // largest index used by each mesh's index buffer
    GpuMaterial* d_materials = nullptr;
    std::vector<GpuMaterial> materials;
    TexDesc* d_textures = nullptr;
    uint32_t texture_count = 0;
    uint32_t* d_texels = nullptr;
    SamplerBits* d_samplers = nullptr;
    uint32_t sampler_count = 0;
    float* d_srgb = nullptr;
    bool have_asset = false;

    // objects and draw lists
    rz_object* d_objects = nullptr;
    rz_object* h_objects = nullptr;  // pinned staging for rz_update_objects
    uint32_t object_count = 0;
    cudaEvent_t objects_copied = nullptr;
    DrawRec* d_shadow_draws = nullptr;
    DrawRec* d_opaque_draws = nullptr;
    DrawRec* d_blended_draws = nullptr;
    DrawConsts* d_blended_consts = nullptr;
    uint32_t blended_varying_base = 0;  // first varying record of the blended draws
    uint2* d_color16 = nullptr;         // RGBA16F draw image (only with blended surfaces)
    uint32_t shadow_draw_count = 0, opaque_draw_count = 0, blended_draw_count = 0;
    uint32_t shadow_tris = 0, opaque_tris = 0, blended_tris = 0;
    float* d_shadow_mvp = nullptr;
    DrawConsts* d_camera_consts = nullptr;
    float4* d_varyings = nullptr;
    uint32_t varying_count = 0;
    bool have_objects = false;

    // raster scratch
    PassBuffers shadow_pass, camera_pass, blended_pass;
    PassHeader* d_headers = nullptr;  // [0] shadow, [1] camera, [2] blended
    uint32_t* d_error = nullptr;
    FrameReport* h_report = nullptr;  // pinned
    bool grow_records = false, grow_chunks = false;

    // frame sequencing
    cudaGraphExec_t graph = nullptr;
    bool graph_dirty = true;
    bool use_graph = true;
    cudaEvent_t frame_done = nullptr;
    bool frame_pending = false;
    bool timing = false;
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

#define RZ_CUDA(ctx, expr, what)                         \
    do {                                                 \
        cudaError_t _e = (expr);                         \
        if (_e != cudaSuccess) return cuda_fail(ctx, _e, what); \
    } while (0)

void free_frame_buffers(rz_ctx* c) {
    dfree(c->d_vis);
    dfree(c->d_color);
    dfree(c->d_depth);
    dfree(c->d_shadow);
}

int alloc_frame_buffers(rz_ctx* c) {
    const size_t np = (size_t)c->width * c->height;
    RZ_CUDA(c, dalloc(&c->d_vis, np), "visibility buffer");
    RZ_CUDA(c, dalloc(&c->d_color, np), "colour buffer");
    RZ_CUDA(c, dalloc(&c->d_depth, np), "depth buffer");
    RZ_CUDA(c, dalloc(&c->d_shadow, (size_t)c->shadow_size * c->shadow_size), "shadow map");
    RZ_CUDA(c, cudaMemset(c->d_vis, 0, np * 8), "clear visibility");
    RZ_CUDA(c, cudaMemset(c->d_color, 0, np * 4), "clear colour");
    RZ_CUDA(c, cudaMemset(c->d_depth, 0, np * 4), "clear depth");
    RZ_CUDA(c, cudaMemset(c->d_shadow, 0, (size_t)c->shadow_size * c->shadow_size * 4), "clear shadow");
    return RZ_OK;
}

void free_pass(PassBuffers& p) {
    dfree(p.records);
    dfree(p.small_records);
    p.small_capacity = 0;
    dfree(p.tile_status);
    dfree(p.chunk_map);
    p.record_capacity = p.tile_capacity = p.chunk_capacity = 0;
}

// Sizes the raster scratch of a pass: one record per triangle plus room for
// clipped fans, and a chunk map for `stamps_hint` stamps.
int size_pass(rz_ctx* c, PassBuffers& p, uint32_t tris, uint64_t stamps_hint) {
    const uint32_t rec_cap = tris + tris / 4 + 4096;
    const uint32_t tiles = (uint32_t)setup_ctas(tris) + 1;
    uint64_t chunks = (stamps_hint + kChunkStamps - 1) / kChunkStamps + 1024;
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
    if (chunks > p.chunk_capacity) {
        dfree(p.chunk_map);
        RZ_CUDA(c, dalloc(&p.chunk_map, (size_t)chunks), "chunk map");
        p.chunk_capacity = (uint32_t)chunks;
    }
    return RZ_OK;
}

// Stamps a pass may need: never more than every triangle covering the whole
// target; otherwise room for 256 full-screen layers of overdraw plus 16 stamps
// per triangle. A frame that needs more reports RZ_OVERFLOW and the capacity
// grows for the next frame.
uint64_t default_stamp_hint(uint32_t tris, uint32_t w, uint32_t h) {
    const uint64_t screen = ((uint64_t)w / kStampW + 1) * ((uint64_t)h / kStampH + 1);
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

PassParams pass_params(rz_ctx* c, bool camera, bool blended = false) {
    PassParams p{};
    p.pos = c->d_pos;
    p.indices = c->d_indices;
    p.vertex_count = c->vertex_count;
    p.cull_front = c->draw_config.cull_enabled ? 1 : 0;
    p.ccw_front = c->draw_config.reverse_winding_order_enabled ? 1 : 0;
    p.error_flags = c->d_error;
    if (blended) {
        // blended list: cull none, no depth write, records kept in submission order
        p.draws = c->d_blended_draws;
        p.draw_count = c->blended_draw_count;
        p.tri_total = c->blended_tris;
        p.mvp = reinterpret_cast<const float*>(c->d_blended_consts);
        p.mvp_stride = sizeof(DrawConsts) / sizeof(float);
        p.width = (int)c->width;
        p.height = (int)c->height;
        p.cull_front = 0;
        p.write_id = 1;
        p.ordered = 1;
        p.records = c->blended_pass.records;
        p.record_capacity = c->blended_pass.record_capacity;
        p.small_records = c->blended_pass.small_records;
        p.small_capacity = c->blended_pass.small_capacity;
        p.tile_status = c->blended_pass.tile_status;
        p.chunk_map = c->blended_pass.chunk_map;
        p.chunk_capacity = c->blended_pass.chunk_capacity;
        p.header = c->d_headers + 2;
        p.target = nullptr;
    } else if (camera) {
        p.draws = c->d_opaque_draws;
        p.draw_count = c->opaque_draw_count;
        p.tri_total = c->opaque_tris;
        p.mvp = reinterpret_cast<const float*>(c->d_camera_consts);
        p.mvp_stride = sizeof(DrawConsts) / sizeof(float);
        p.width = (int)c->width;
        p.height = (int)c->height;
        p.bias_enabled = 0;
        p.write_id = 1;
        p.records = c->camera_pass.records;
        p.record_capacity = c->camera_pass.record_capacity;
        p.small_records = c->camera_pass.small_records;
        p.small_capacity = c->camera_pass.small_capacity;
        p.tile_status = c->camera_pass.tile_status;
        p.chunk_map = c->camera_pass.chunk_map;
        p.chunk_capacity = c->camera_pass.chunk_capacity;
        p.header = c->d_headers + 1;
        p.target = c->d_vis;
    } else {
        p.draws = c->d_shadow_draws;
        p.draw_count = c->shadow_draw_count;
        p.tri_total = c->shadow_tris;
        p.mvp = c->d_shadow_mvp;
        p.mvp_stride = 16;
        p.width = (int)c->shadow_size;
        p.height = (int)c->shadow_size;
        p.bias_enabled = c->draw_config.depth_bias_enabled ? 1 : 0;
        p.bias_constant = c->draw_config.depth_bias_constant;
        p.bias_clamp = c->draw_config.depth_bias_clamp;
        p.bias_slope = c->draw_config.depth_bias_slope_factor;
        p.write_id = 0;
        p.records = c->shadow_pass.records;
        p.record_capacity = c->shadow_pass.record_capacity;
        p.small_records = c->shadow_pass.small_records;
        p.small_capacity = c->shadow_pass.small_capacity;
        p.tile_status = c->shadow_pass.tile_status;
        p.chunk_map = c->shadow_pass.chunk_map;
        p.chunk_capacity = c->shadow_pass.chunk_capacity;
        p.header = c->d_headers + 0;
        p.target = c->d_shadow;
    }
    return p;
}

void stamp(rz_ctx* c, int i) {
    if (c->timing) cudaEventRecord(c->stage_ev[i], c->stream);
}

// Enqueues one frame (everything after the scene/object uploads).
ShadeParams shade_params(rz_ctx* c) {
    ShadeParams sh{};
    sh.vis = c->d_vis;
    sh.shadow = reinterpret_cast<const float*>(c->d_shadow);
    sh.shadow_size = (int)c->shadow_size;
    sh.color = c->d_color;
    sh.depth = c->d_depth;
    sh.width = (int)c->width;
    sh.height = (int)c->height;
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
    sh.texture_count = c->texture_count;
    sh.samplers = c->d_samplers;
    sh.sampler_count = c->sampler_count;
    sh.texels = c->d_texels;
    sh.scene = c->d_scene;
    sh.pcf_mode = c->draw_config.pcf_mode;
    sh.srgb_table = c->d_srgb;
    sh.color16 = c->blended_tris ? c->d_color16 : nullptr;
    return sh;
}

// Shadow pass (src/Engine/Graphics.cpp:5195-5292): clear to 0, per-draw
// matrices, setup, raster.
void enqueue_shadow(rz_ctx* c, cudaStream_t s, bool stamps) {
    ClearList cl{};
    cl.ptr[0] = c->d_shadow;
    cl.bytes[0] = (size_t)c->shadow_size * c->shadow_size * 4;
    cl.ptr[1] = c->d_headers + 0;
    cl.bytes[1] = sizeof(PassHeader);
    cl.count = 2;
    if (c->shadow_tris) {
        cl.ptr[2] = c->shadow_pass.tile_status;
        cl.bytes[2] = (size_t)setup_ctas(c->shadow_tris) * 8;
        cl.count = 3;
    }
    launch_clear(cl, c->sm_count, s);
    if (stamps) stamp(c, 1);
    if (c->shadow_tris) {
        launch_prep(c->d_shadow_draws, c->shadow_draw_count, c->d_objects, c->d_scene->shadow_projection_near,
                    c->d_shadow_mvp, s);
        const PassParams sp = pass_params(c, false);
        launch_setup(sp, s);
        if (stamps) stamp(c, 2);
        launch_raster(sp, c->sm_count, s);
    } else if (stamps) {
        stamp(c, 2);
    }
}

// Camera pass (5566-5653): visibility cleared to 0, opaque list, then the
// vertex stage of the shading.
void enqueue_camera(rz_ctx* c, cudaStream_t s, bool stamps, const ShadeParams& sh) {
    ClearList cl{};
    cl.ptr[0] = c->d_vis;
    cl.bytes[0] = (size_t)c->width * c->height * 8;
    cl.ptr[1] = c->d_headers + 1;
    cl.bytes[1] = sizeof(PassHeader);
    cl.count = 2;
    if (c->opaque_tris) {
        cl.ptr[2] = c->camera_pass.tile_status;
        cl.bytes[2] = (size_t)setup_ctas(c->opaque_tris) * 8;
        cl.count = 3;
    }
    launch_clear(cl, c->sm_count, s);
    launch_prep_camera(c->d_opaque_draws, c->opaque_draw_count, c->d_objects, c->d_scene, c->d_camera_consts, s);
    if (stamps) stamp(c, 4);
    if (c->opaque_tris) {
        const PassParams cp = pass_params(c, true);
        launch_setup(cp, s);
        if (stamps) stamp(c, 5);
        launch_raster(cp, c->sm_count, s);
    } else if (stamps) {
        stamp(c, 5);
    }
    launch_vertex(sh, s);
    if (c->blended_tris) {
        ClearList bl{};
        bl.ptr[0] = c->d_headers + 2;
        bl.bytes[0] = sizeof(PassHeader);
        bl.ptr[1] = c->blended_pass.tile_status;
        bl.bytes[1] = (size_t)setup_ctas(c->blended_tris) * 8;
        bl.count = 2;
        launch_clear(bl, c->sm_count, s);
        launch_prep_camera(c->d_blended_draws, c->blended_draw_count, c->d_objects, c->d_scene, c->d_blended_consts, s);
        launch_setup(pass_params(c, true, true), s);
        ShadeParams bs = sh;
        bs.draws = c->d_blended_draws;
        bs.draw_count = c->blended_draw_count;
        bs.consts = c->d_blended_consts;
        bs.varying_count = c->varying_count;
        launch_vertex_range(bs, c->blended_varying_base, s);
    }
}

// Enqueues one frame (everything after the scene/object uploads). With stage
// timing the stages run one after the other on the main stream between
// events; otherwise the shadow pass runs on a side stream concurrently with the
// camera pass, joining before the shading (which reads the shadow map).
int enqueue_frame(rz_ctx* c) {
    cudaStream_t s = c->stream;
    const ShadeParams sh = shade_params(c);
    RZ_CUDA(c, cudaMemsetAsync(c->d_error, 0, sizeof(uint32_t), s), "clear error flags");
    if (c->timing) {
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
        RZ_CUDA(c, cudaStreamWaitEvent(s, c->join, 0), "join");
    }
    launch_shade(sh, s);
    if (c->blended_tris) {
        BlendParams bp{};
        bp.sh = sh;
        bp.sh.draws = c->d_blended_draws;
        bp.sh.draw_count = c->blended_draw_count;
        bp.sh.consts = c->d_blended_consts;
        bp.records = c->blended_pass.records;
        bp.header = c->d_headers + 2;
        bp.record_capacity = c->blended_pass.record_capacity;
        bp.depth = c->d_depth;
        launch_blend(bp, s);
    }
    if (c->timing) stamp(c, 7);
    RZ_CUDA(c, cudaGetLastError(), "kernel launch");
    RZ_CUDA(c, cudaMemcpyAsync(&c->h_report->error_flags, c->d_error, sizeof(uint32_t), cudaMemcpyDeviceToHost, s),
            "read error flags");
    RZ_CUDA(c, cudaMemcpyAsync(&c->h_report->shadow, c->d_headers, 3 * sizeof(PassHeader), cudaMemcpyDeviceToHost, s),
            "read pass headers");
    return RZ_OK;
}

int check_ready(rz_ctx* c) {
    if (!c) return RZ_INVALID_ARGUMENT;
    if (!c->have_asset) return fail(c, RZ_INVALID_STATE, "rz_set_asset has not been called");
    if (!c->have_objects) return fail(c, RZ_INVALID_STATE, "rz_set_objects has not been called");
    if (!c->have_scene) return fail(c, RZ_INVALID_STATE, "rz_update has not been called");
    return RZ_OK;
}

void drop_graph(rz_ctx* c) {
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    c->graph_dirty = true;
}

}  // namespace

extern "C" {

uint32_t rz_abi_version(void) { return RZ_ABI_VERSION; }

int rz_create(rz_ctx** out, const rz_config* cfg) {
    if (!out || !cfg) return RZ_INVALID_ARGUMENT;
    *out = nullptr;
    if (cfg->width == 0 || cfg->height == 0 || cfg->width > 16384 || cfg->height > 16384) return RZ_INVALID_ARGUMENT;
    if (cfg->shadow_map_size == 0 || cfg->shadow_map_size > 16384) return RZ_INVALID_ARGUMENT;
    if (cfg->samples != 1) return RZ_INVALID_ARGUMENT;
    rz_ctx* c = new rz_ctx();
    c->device = cfg->device;
    c->width = cfg->width;
    c->height = cfg->height;
    c->shadow_size = cfg->shadow_map_size;
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
        cudaEventCreateWithFlags(&c->fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->join, cudaEventDisableTiming) != cudaSuccess)
        return bail(RZ_GRAPHICS_INIT_FAILURE);
    if (cudaEventCreateWithFlags(&c->frame_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->scene_copied, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->objects_copied, cudaEventDisableTiming) != cudaSuccess)
        return bail(RZ_GRAPHICS_INIT_FAILURE);
    if (alloc_frame_buffers(c) != RZ_OK) return bail(RZ_ALLOCATION_FAILURE);
    if (dalloc(&c->d_scene, 1) != cudaSuccess || dalloc(&c->d_headers, 3) != cudaSuccess ||
        dalloc(&c->d_error, 1) != cudaSuccess || dalloc(&c->d_srgb, 256) != cudaSuccess)
        return bail(RZ_ALLOCATION_FAILURE);
    if (cudaMallocHost(&c->h_scene, sizeof(rz_scene_data)) != cudaSuccess ||
        cudaMallocHost(&c->h_report, sizeof(FrameReport)) != cudaSuccess)
        return bail(RZ_ALLOCATION_FAILURE);
    std::memset(c->h_report, 0, sizeof(FrameReport));
    // sRGB decode table (colour, metallic-roughness and mixmap images are sRGB
    // formats, src/Engine/Graphics.cpp:3632-3647): IEC 61966-2-1 in double, rounded to float.
    float table[256];
    for (int i = 0; i < 256; ++i) {
        const double v = i / 255.0;
        table[i] = (float)(v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4));
    }
    if (cudaMemcpy(c->d_srgb, table, sizeof(table), cudaMemcpyHostToDevice) != cudaSuccess) return bail(RZ_ERROR);
    // reference defaults, src/Engine/Level.cpp:1246-1255
    c->draw_config.cull_enabled = 1;
    c->draw_config.reverse_winding_order_enabled = 0;
    c->draw_config.depth_bias_enabled = 1;
    c->draw_config.depth_bias_constant = -21.882f;
    c->draw_config.depth_bias_clamp = -20.937f;
    c->draw_config.depth_bias_slope_factor = -3.0f;
    c->draw_config.pcf_mode = RZ_PCF_5TAP;
    const char* g = std::getenv("RZ_NO_GRAPH");
    c->use_graph = !(g && g[0] == '1');
    *out = c;
    return RZ_OK;
}

void rz_destroy(rz_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    drop_graph(c);
    free_frame_buffers(c);
    free_pass(c->shadow_pass);
    free_pass(c->camera_pass);
    dfree(c->d_scene);
    dfree(c->d_headers);
    dfree(c->d_error);
    dfree(c->d_srgb);
    dfree(c->d_vertices);
    dfree(c->d_pos);
    dfree(c->d_indices);
    dfree(c->d_materials);
    dfree(c->d_textures);
    dfree(c->d_texels);
    dfree(c->d_samplers);
    dfree(c->d_objects);
    dfree(c->d_shadow_draws);
    dfree(c->d_opaque_draws);
    dfree(c->d_shadow_mvp);
    dfree(c->d_camera_consts);
    dfree(c->d_varyings);
    dfree(c->d_blended_draws);
    dfree(c->d_blended_consts);
    dfree(c->d_color16);
    free_pass(c->blended_pass);
    if (c->h_scene) cudaFreeHost(c->h_scene);
    if (c->h_report) cudaFreeHost(c->h_report);
    if (c->h_objects) cudaFreeHost(c->h_objects);
    if (c->frame_done) cudaEventDestroy(c->frame_done);
    for (auto& e : c->stage_ev)
        if (e) cudaEventDestroy(e);
    if (c->scene_copied) cudaEventDestroy(c->scene_copied);
    if (c->objects_copied) cudaEventDestroy(c->objects_copied);
    if (c->side) cudaStreamSynchronize(c->side);
    if (c->fork) cudaEventDestroy(c->fork);
    if (c->join) cudaEventDestroy(c->join);
    if (c->side) cudaStreamDestroy(c->side);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int rz_resize(rz_ctx* c, uint32_t width, uint32_t height) {
    if (!c) return RZ_INVALID_ARGUMENT;
    if (width == 0 || height == 0 || width > 16384 || height > 16384) return fail(c, RZ_INVALID_ARGUMENT, "bad extent");
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    drop_graph(c);
    free_frame_buffers(c);
    c->width = width;
    c->height = height;
    const int rc = alloc_frame_buffers(c);
    if (rc != RZ_OK) return rc;
    if (c->d_color16) {
        dfree(c->d_color16);
        RZ_CUDA(c, dalloc(&c->d_color16, (size_t)width * height), "RGBA16F draw image");
    }
    if (c->have_objects) {
        const int r2 = size_pass(c, c->camera_pass, c->opaque_tris, default_stamp_hint(c->opaque_tris, width, height));
        if (r2 != RZ_OK) return r2;
    }
    return RZ_OK;
}

int rz_set_asset(rz_ctx* c, const rz_mesh* meshes, uint32_t mesh_count, const rz_material* mats, uint32_t mat_count,
                 const rz_texture* textures, uint32_t tex_count, const rz_sampler* samplers, uint32_t sampler_count) {
    if (!c) return RZ_INVALID_ARGUMENT;
    if (mesh_count == 0 || !meshes) return fail(c, RZ_INVALID_ARGUMENT, "asset has no meshes");
    if ((mat_count && !mats) || (tex_count && !textures) || (sampler_count && !samplers))
        return fail(c, RZ_INVALID_ARGUMENT, "null array with non-zero count");
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    drop_graph(c);
    // meshes: concatenated vertex and index buffers (src/Engine/Graphics.cpp:4310-4334)
    uint64_t nv = 0, ni = 0;
    for (uint32_t m = 0; m < mesh_count; ++m) {
        if ((meshes[m].position_count && !meshes[m].positions) || (meshes[m].index_count && !meshes[m].indices))
            return fail(c, RZ_INVALID_ARGUMENT, "mesh with null data");
        nv += meshes[m].position_count;
        ni += meshes[m].index_count;
    }
    if (nv >= 0xFFFFFFFFull || ni >= 0xFFFFFFFFull) return fail(c, RZ_OVERFLOW, "asset too large");
    std::vector<rz_vertex> verts;
    std::vector<float4> pos;
    std::vector<uint32_t> idx;
    verts.reserve(nv);
    pos.reserve(nv);
    idx.reserve(ni);
    c->mesh_table.assign(4 * mesh_count, 0);
    c->mesh_vertex_max.assign(mesh_count, 0);
    for (uint32_t m = 0; m < mesh_count; ++m) {
        const rz_mesh& mesh = meshes[m];
        c->mesh_table[4 * m + 0] = (uint32_t)verts.size();
        c->mesh_table[4 * m + 1] = mesh.position_count;
        c->mesh_table[4 * m + 2] = (uint32_t)idx.size();
        c->mesh_table[4 * m + 3] = mesh.index_count;
        for (uint32_t i = 0; i < mesh.position_count; ++i) {
            verts.push_back(mesh.positions[i]);
            pos.push_back(make_float4(mesh.positions[i].position[0], mesh.positions[i].position[1],
                                      mesh.positions[i].position[2], 1.0f));
        }
        for (uint32_t i = 0; i < mesh.index_count; ++i) {
            if (mesh.indices[i] >= mesh.position_count)
                return fail(c, RZ_INVALID_ARGUMENT, "mesh " + std::to_string(m) + " index out of range");
            idx.push_back(mesh.indices[i]);
        }
    }
    // materials (src/Engine/Graphics.cpp:4071-4150)
    std::vector<GpuMaterial> gm(mat_count);
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
            g.sampler[k] = sampler_count;
            if (img[k] < tex_count) {
                g.tex[k] = img[k];
                if (smp[k] < sampler_count) g.sampler[k] = smp[k];
            }
        }
        gm[i] = g;
    }
    // textures: one RGBA8 pool, per-level offsets
    std::vector<TexDesc> td(tex_count);
    uint64_t total_texels = 0;
    for (uint32_t i = 0; i < tex_count; ++i) {
        const rz_texture& t = textures[i];
        if (t.width == 0 || t.height == 0 || t.levels == 0 || t.levels > 16 || !t.texels)
            return fail(c, RZ_INVALID_ARGUMENT, "texture " + std::to_string(i) + " is malformed");
        uint32_t max_levels = 1;
        while ((t.width >> max_levels) || (t.height >> max_levels)) ++max_levels;
        if (t.levels > max_levels) return fail(c, RZ_INVALID_ARGUMENT, "texture has too many levels");
        TexDesc d{};
        d.width = t.width;
        d.height = t.height;
        d.levels = t.levels;
        d.srgb = t.image_type == RZ_IMAGE_NORMAL_MAP ? 0u : 1u;
        d.base = total_texels;
        uint64_t off = 0;
        for (uint32_t l = 0; l < t.levels; ++l) {
            d.level_off[l] = (uint32_t)off;
            off += (uint64_t)std::max(1u, t.width >> l) * std::max(1u, t.height >> l);
        }
        if (off >= 0xFFFFFFFFull) return fail(c, RZ_OVERFLOW, "texture too large");
        td[i] = d;
        total_texels += off;
    }
    std::vector<SamplerBits> sb(sampler_count + 1);
    for (uint32_t i = 0; i < sampler_count; ++i) sb[i] = sampler_bits(samplers[i]);
    // default sampler: linear/linear, nearest mip, repeat (src/Engine/Graphics.cpp:3421-3438)
    sb[sampler_count] = 1u | 2u | (2u << 4) | (2u << 6);

    dfree(c->d_vertices);
    dfree(c->d_pos);
    dfree(c->d_indices);
    dfree(c->d_materials);
    dfree(c->d_textures);
    dfree(c->d_texels);
    dfree(c->d_samplers);
    RZ_CUDA(c, dalloc(&c->d_vertices, nv), "vertex buffer");
    RZ_CUDA(c, dalloc(&c->d_pos, nv), "position stream");
    RZ_CUDA(c, dalloc(&c->d_indices, std::max<uint64_t>(ni, 1)), "index buffer");
    RZ_CUDA(c, dalloc(&c->d_materials, std::max<uint32_t>(mat_count, 1)), "material buffer");
    RZ_CUDA(c, dalloc(&c->d_textures, std::max<uint32_t>(tex_count, 1)), "texture table");
    RZ_CUDA(c, dalloc(&c->d_texels, std::max<uint64_t>(total_texels, 1)), "texel pool");
    RZ_CUDA(c, dalloc(&c->d_samplers, sb.size()), "sampler table");
    RZ_CUDA(c, cudaMemcpy(c->d_vertices, verts.data(), nv * sizeof(rz_vertex), cudaMemcpyHostToDevice), "upload vertices");
    RZ_CUDA(c, cudaMemcpy(c->d_pos, pos.data(), nv * sizeof(float4), cudaMemcpyHostToDevice), "upload positions");
    if (ni) RZ_CUDA(c, cudaMemcpy(c->d_indices, idx.data(), ni * 4, cudaMemcpyHostToDevice), "upload indices");
    if (mat_count)
        RZ_CUDA(c, cudaMemcpy(c->d_materials, gm.data(), mat_count * sizeof(GpuMaterial), cudaMemcpyHostToDevice), "upload materials");
    if (tex_count)
        RZ_CUDA(c, cudaMemcpy(c->d_textures, td.data(), tex_count * sizeof(TexDesc), cudaMemcpyHostToDevice), "upload texture table");
    for (uint32_t i = 0; i < tex_count; ++i) {
        const uint64_t n = (i + 1 < tex_count ? td[i + 1].base : total_texels) - td[i].base;
        RZ_CUDA(c, cudaMemcpy(c->d_texels + td[i].base, textures[i].texels, n * 4, cudaMemcpyHostToDevice), "upload texels");
    }
    RZ_CUDA(c, cudaMemcpy(c->d_samplers, sb.data(), sb.size() * sizeof(SamplerBits), cudaMemcpyHostToDevice), "upload samplers");
    c->vertex_count = (uint32_t)nv;
    c->index_count = (uint32_t)ni;
    c->materials = gm;
    c->texture_count = tex_count;
    c->sampler_count = sampler_count;
    c->have_asset = true;
    c->have_objects = false;  // draw lists refer to the old meshes
    return RZ_OK;
}

int rz_set_objects(rz_ctx* c, const rz_object* objects, uint32_t object_count, const rz_surface* surfaces,
                   uint32_t surface_count) {
    if (!c) return RZ_INVALID_ARGUMENT;
    if (!c->have_asset) return fail(c, RZ_INVALID_STATE, "rz_set_asset has not been called");
    // src/Engine/Graphics.cpp:4693-4697: an empty scene is an invalid argument
    if (object_count == 0 || !objects || surface_count == 0 || !surfaces)
        return fail(c, RZ_INVALID_ARGUMENT, "empty scene");
    std::vector<DrawRec> shadow, opaque, blended;
    uint32_t shadow_tris = 0, opaque_tris = 0, blended_tris = 0, blended_draws = 0, varyings = 0;
    const uint32_t mesh_count = (uint32_t)(c->mesh_table.size() / 4);
    for (uint32_t i = 0; i < surface_count; ++i) {
        const rz_surface& s = surfaces[i];
        if (s.mesh_index >= mesh_count) return fail(c, RZ_INVALID_ARGUMENT, "surface mesh index out of range");
        const uint64_t obj = (uint64_t)s.graphic_objects_offset + s.graphics_object_index;
        if (obj >= object_count) return fail(c, RZ_INVALID_ARGUMENT, "surface object index out of range");
        const uint32_t* mt = &c->mesh_table[4 * s.mesh_index];
        if ((uint64_t)s.start_index + s.index_count > mt[3])
            return fail(c, RZ_INVALID_ARGUMENT, "surface index range outside its mesh");
        const bool has_mat = s.material_index < c->materials.size();
        if (!s.blended && has_mat && c->materials[s.material_index].alpha_mode != 0)
            return fail(c, RZ_INVALID_ARGUMENT, "opaque surface with a non-opaque material");
        DrawRec d{};
        d.vertex_base = mt[0];
        d.first_index = mt[2] + s.start_index;
        d.tri_count = s.index_count / 3;
        d.object = (uint32_t)obj;
        d.material = has_mat ? (int32_t)s.material_index : -1;
        d.tri_base = shadow_tris;
        shadow.push_back(d);
        if ((uint64_t)shadow_tris + d.tri_count >= 0xFFFFFFF0ull) return fail(c, RZ_OVERFLOW, "too many triangles");
        shadow_tris += d.tri_count;
        if (s.blended) {
            d.tri_base = blended_tris;
            d.vertex_count = mt[1];
            blended_tris += d.tri_count;
            ++blended_draws;
            blended.push_back(d);
        } else {
            d.tri_base = opaque_tris;
            d.varying_base = varyings;
            d.vertex_count = mt[1];
            if ((uint64_t)varyings + mt[1] >= 0xFFFFFFF0ull) return fail(c, RZ_OVERFLOW, "too many vertices");
            varyings += mt[1];
            opaque.push_back(d);
            opaque_tris += d.tri_count;
        }
    }
    // varying records of the blended draws follow the opaque ones
    const uint32_t blended_varying_base = varyings;
    for (DrawRec& d : blended) {
        if ((uint64_t)varyings + d.vertex_count >= 0xFFFFFFF0ull) return fail(c, RZ_OVERFLOW, "too many vertices");
        d.varying_base = varyings;
        varyings += d.vertex_count;
    }
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    drop_graph(c);
    dfree(c->d_objects);
    dfree(c->d_shadow_draws);
    dfree(c->d_opaque_draws);
    dfree(c->d_shadow_mvp);
    dfree(c->d_camera_consts);
    dfree(c->d_varyings);
    dfree(c->d_blended_draws);
    dfree(c->d_blended_consts);
    dfree(c->d_color16);
    if (c->h_objects) cudaFreeHost(c->h_objects);
    c->h_objects = nullptr;
    RZ_CUDA(c, dalloc(&c->d_objects, object_count), "object buffer");
    RZ_CUDA(c, cudaMallocHost(&c->h_objects, (size_t)object_count * sizeof(rz_object)), "object staging");
    RZ_CUDA(c, dalloc(&c->d_shadow_draws, std::max<size_t>(shadow.size(), 1)), "shadow draw list");
    RZ_CUDA(c, dalloc(&c->d_opaque_draws, std::max<size_t>(opaque.size(), 1)), "opaque draw list");
    RZ_CUDA(c, dalloc(&c->d_shadow_mvp, std::max<size_t>(shadow.size(), 1) * 16), "shadow matrices");
    RZ_CUDA(c, dalloc(&c->d_camera_consts, std::max<size_t>(opaque.size(), 1)), "camera constants");
    RZ_CUDA(c, dalloc(&c->d_blended_draws, std::max<size_t>(blended.size(), 1)), "blended draw list");
    RZ_CUDA(c, dalloc(&c->d_blended_consts, std::max<size_t>(blended.size(), 1)), "blended constants");
    if (!blended.empty())
        RZ_CUDA(c, dalloc(&c->d_color16, (size_t)c->width * c->height), "RGBA16F draw image");
    RZ_CUDA(c, dalloc(&c->d_varyings, std::max<size_t>(varyings, 1) * 8), "varying records");
    RZ_CUDA(c, cudaMemcpy(c->d_objects, objects, (size_t)object_count * sizeof(rz_object), cudaMemcpyHostToDevice), "upload objects");
    if (!shadow.empty())
        RZ_CUDA(c, cudaMemcpy(c->d_shadow_draws, shadow.data(), shadow.size() * sizeof(DrawRec), cudaMemcpyHostToDevice), "upload draws");
    if (!opaque.empty())
        RZ_CUDA(c, cudaMemcpy(c->d_opaque_draws, opaque.data(), opaque.size() * sizeof(DrawRec), cudaMemcpyHostToDevice), "upload draws");
    if (!blended.empty())
        RZ_CUDA(c, cudaMemcpy(c->d_blended_draws, blended.data(), blended.size() * sizeof(DrawRec), cudaMemcpyHostToDevice), "upload draws");
    c->object_count = object_count;
    c->shadow_draw_count = (uint32_t)shadow.size();
    c->opaque_draw_count = (uint32_t)opaque.size();
    c->blended_draw_count = blended_draws;
    c->shadow_tris = shadow_tris;
    c->opaque_tris = opaque_tris;
    c->blended_tris = blended_tris;
    c->varying_count = varyings;
    c->blended_varying_base = blended_varying_base;
    if (blended_tris) {
        const int rb = size_pass(c, c->blended_pass, blended_tris, default_stamp_hint(blended_tris, c->width, c->height));
        if (rb != RZ_OK) return rb;
    }
    int rc = size_pass(c, c->shadow_pass, shadow_tris, default_stamp_hint(shadow_tris, c->shadow_size, c->shadow_size));
    if (rc != RZ_OK) return rc;
    rc = size_pass(c, c->camera_pass, opaque_tris, default_stamp_hint(opaque_tris, c->width, c->height));
    if (rc != RZ_OK) return rc;
    c->have_objects = true;
    return RZ_OK;
}

int rz_update_objects(rz_ctx* c, uint32_t offset, const rz_object* objects, uint32_t count) {
    if (!c) return RZ_INVALID_ARGUMENT;
    if (!c->have_objects) return fail(c, RZ_INVALID_STATE, "rz_set_objects has not been called");
    if (count == 0) return RZ_OK;
    if (!objects || (uint64_t)offset + count > c->object_count) return fail(c, RZ_INVALID_ARGUMENT, "object range");
    cudaSetDevice(c->device);
    RZ_CUDA(c, cudaEventSynchronize(c->objects_copied), "wait staging");
    std::memcpy(c->h_objects + offset, objects, (size_t)count * sizeof(rz_object));
    RZ_CUDA(c, cudaMemcpyAsync(c->d_objects + offset, c->h_objects + offset, (size_t)count * sizeof(rz_object),
                               cudaMemcpyHostToDevice, c->stream), "upload objects");
    RZ_CUDA(c, cudaEventRecord(c->objects_copied, c->stream), "record");
    return RZ_OK;
}

int rz_set_draw_config(rz_ctx* c, const rz_draw_config* cfg) {
    if (!c || !cfg) return RZ_INVALID_ARGUMENT;
    if (cfg->pcf_mode > RZ_PCF_3X3) return fail(c, RZ_INVALID_ARGUMENT, "unknown pcf mode");
    c->draw_config = *cfg;
    drop_graph(c);
    return RZ_OK;
}

int rz_update(rz_ctx* c, const rz_scene_data* scene) {
    if (!c || !scene) return RZ_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    RZ_CUDA(c, cudaEventSynchronize(c->scene_copied), "wait staging");
    std::memcpy(c->h_scene, scene, sizeof(rz_scene_data));
    RZ_CUDA(c, cudaMemcpyAsync(c->d_scene, c->h_scene, sizeof(rz_scene_data), cudaMemcpyHostToDevice, c->stream),
            "upload scene");
    RZ_CUDA(c, cudaEventRecord(c->scene_copied, c->stream), "record");
    c->have_scene = true;
    return RZ_OK;
}

int rz_render(rz_ctx* c) {
    const int ready = check_ready(c);
    if (ready != RZ_OK) return ready;
    cudaSetDevice(c->device);
    if (c->grow_records || c->grow_chunks) {
        // Size the queues from what the overflowing frame needed (exact counts
        // from the device), with 25% headroom.
        cudaStreamSynchronize(c->stream);
        drop_graph(c);
        c->queue_chunks = 0;
        auto grow = [&](PassBuffers& p, const PassHeader& h) -> int {
            const uint64_t want_chunks = (h.stamps + kChunkStamps - 1) / kChunkStamps;
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
        if (rc != RZ_OK) return rc;
    }
    // Stage timing records events between the stages and enqueues directly.
    if (c->use_graph && !c->timing) {
        if (c->graph_dirty || !c->graph) {
            cudaGraph_t g = nullptr;
            RZ_CUDA(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
            const int rc = enqueue_frame(c);
            const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
            if (rc != RZ_OK) {
                if (g) cudaGraphDestroy(g);
                return rc;
            }
            cudaError_t ie = e;
            if (e == cudaSuccess) ie = cudaGraphInstantiate(&c->graph, g, 0);
            if (g) cudaGraphDestroy(g);
            if (ie != cudaSuccess) {
                // capture of this frame shape is not supported here: enqueue directly from now on
                cudaGetLastError();
                c->graph = nullptr;
                c->use_graph = false;
                const int rc2 = enqueue_frame(c);
                if (rc2 != RZ_OK) return rc2;
                RZ_CUDA(c, cudaEventRecord(c->frame_done, c->stream), "record frame");
                c->frame_pending = true;
                ++c->frames;
                return RZ_OK;
            }
            c->graph_dirty = false;
        }
        RZ_CUDA(c, cudaGraphLaunch(c->graph, c->stream), "launch frame graph");
    } else {
        const int rc = enqueue_frame(c);
        if (rc != RZ_OK) return rc;
    }
    RZ_CUDA(c, cudaEventRecord(c->frame_done, c->stream), "record frame");
    c->frame_pending = true;
    ++c->frames;
    return RZ_OK;
}

int rz_sync(rz_ctx* c, uint32_t timeout_ms) {
    if (!c) return RZ_INVALID_ARGUMENT;
    cudaSetDevice(c->device);
    const auto t0 = std::chrono::steady_clock::now();
    for (;;) {
        const cudaError_t q = cudaStreamQuery(c->stream);
        if (q == cudaSuccess) break;
        if (q != cudaErrorNotReady) return cuda_fail(c, q, "frame");
        if (timeout_ms) {
            const auto ms = std::chrono::duration_cast<std::chrono::milliseconds>(std::chrono::steady_clock::now() - t0).count();
            if (ms >= (long long)timeout_ms) return fail(c, RZ_TIMEOUT, "frame still running");
        }
        std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
    if (!c->frame_pending) return RZ_OK;
    c->frame_pending = false;
    const uint32_t e = c->h_report->error_flags;
    if (e & (kErrRecordOverflow)) c->grow_records = true;
    if (e & (kErrStampOverflow)) c->grow_chunks = true;
    if (e & (kErrRecordOverflow | kErrStampOverflow))
        return fail(c, RZ_OVERFLOW, "raster work queue overflowed; capacity grows for the next frame");
    if (e) return fail(c, RZ_GRAPHICS_FRAME_FAILURE, "device error flags " + std::to_string(e));
    return RZ_OK;
}

int rz_get_frame(rz_ctx* c, rz_frame_out* out) {
    if (!c || !out) return RZ_INVALID_ARGUMENT;
    out->color_rgba8 = c->d_color;
    out->depth_f32 = c->d_depth;
    out->visibility_u64 = c->d_vis;
    out->shadow_map_f32 = c->d_shadow;
    out->width = c->width;
    out->height = c->height;
    out->shadow_map_size = c->shadow_size;
    out->reserved = 0;
    return RZ_OK;
}

int rz_read_frame(rz_ctx* c, void* color_host, size_t color_bytes, void* depth_host, size_t depth_bytes) {
    if (!c) return RZ_INVALID_ARGUMENT;
    const size_t need = (size_t)c->width * c->height * 4;
    if ((color_host && color_bytes < need) || (depth_host && depth_bytes < need))
        return fail(c, RZ_INVALID_ARGUMENT, "host buffer too small");
    cudaSetDevice(c->device);
    if (color_host)
        RZ_CUDA(c, cudaMemcpyAsync(color_host, c->d_color, need, cudaMemcpyDeviceToHost, c->stream), "read colour");
    if (depth_host)
        RZ_CUDA(c, cudaMemcpyAsync(depth_host, c->d_depth, need, cudaMemcpyDeviceToHost, c->stream), "read depth");
    return RZ_OK;
}

int rz_get_stats(rz_ctx* c, rz_stats* out) {
    if (!c || !out) return RZ_INVALID_ARGUMENT;
    std::memset(out, 0, sizeof(*out));
    out->draw_call_count = c->shadow_draw_count + c->opaque_draw_count + c->blended_draw_count;
    out->triangle_count = c->shadow_tris + c->opaque_tris + c->blended_tris;
    out->shadow_setup_records = c->h_report->shadow.records + c->h_report->shadow.small_records;
    out->camera_setup_records = c->h_report->camera.records + c->h_report->camera.small_records;
    out->shadow_stamps = c->h_report->shadow.stamps;
    out->camera_stamps = c->h_report->camera.stamps;
    out->error_flags = c->h_report->error_flags;
    // clears (2) + prep (1) + prep_camera (1) + setup/raster per pass with triangles + vertex + shade
    out->kernel_launches = 2u + (c->shadow_tris ? 3u : 0u) + (c->opaque_tris ? 2u : 0u) + 2u + (c->varying_count ? 1u : 0u) +
                           (c->blended_tris ? 5u : 0u);
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

void* rz_get_stream(rz_ctx* c) { return c ? (void*)c->stream : nullptr; }

const char* rz_last_error(rz_ctx* c) { return c ? c->last_error.c_str() : "null context"; }

}  // extern "C"
