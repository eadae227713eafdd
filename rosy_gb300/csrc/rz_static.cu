// Shadow depth pass that allocates nothing: rz_shadow_depth_static.
//
// Some callers cannot allocate device memory once they are running: engines
// that own all device memory through their own allocator or a fixed budget, and
// frame loops that must not pay for cudaMalloc/cudaFree (which can synchronise
// the device) in the middle of a frame. For them this entry point runs the same
// setup and raster kernels as the shadow pass of rz_render, with all their
// scratch memory (setup records, look-back words, chunk map, pass header, error
// flags) in one file-scope __device__ array of fixed size. The caller passes the
// inputs and the output; nothing is allocated here.
//
// Limits: at most kStaticMaxTriangles triangles per call (larger draws are
// rejected with RZ_INVALID_ARGUMENT), kStaticRecords setup records and
// kStaticChunks work chunks (kStaticChunks * 32 stamps of 8x4 pixels). A call
// whose coverage needs more chunks, or whose clipped triangles fan out into more
// records than that (the same slack as rz_render's first frame: a quarter of the
// triangles plus 4,096), returns RZ_OVERFLOW and leaves the depth target
// incomplete. The array (about 3.3 MiB) stays resident on every device that
// loads the library until the process exits. All calls share it: calls that
// overlap on the GPU (on different streams, or from different host threads)
// race on it and must be serialised by the caller.
//
// The first call on a device resolves the array's device address with
// cudaGetSymbolAddress (with that device current) and caches it; make that
// first call before any stream capture begins on the device. With lazy module
// loading (the CUDA default) that first call may also be what loads the module
// and places the array, so a caller with a strict frame loop makes one warm-up
// call per device at start-up.
//
// Leftovers of earlier calls in the array do no harm: k_static_prep zeroes the
// pass header, the look-back words and the error flags; every chunk-map entry
// below the pass's chunk count is rewritten by the record holding that chunk's
// first stamp, unless that record overflowed, in which case the raster meets
// either a record index past the capacity or a record of this call whose stamp
// range does not hold the chunk, and stops with the overflow flag set.
#include <mutex>

#include "rz_device.cuh"

namespace rz {

constexpr uint32_t kStaticMaxTriangles = 16384;
constexpr uint32_t kStaticRecords = kStaticMaxTriangles + kStaticMaxTriangles / 4 + 4096;
constexpr uint32_t kStaticTiles = (kStaticMaxTriangles + kSetupThreads - 1) / kSetupThreads + 1;
constexpr uint32_t kStaticChunks = 65536;

// Byte layout of the scratch array (every part 256-byte aligned).
constexpr size_t kOffRecords = 0;
constexpr size_t kOffSmall = kOffRecords + (size_t)kStaticRecords * sizeof(TriRecord);
constexpr size_t kOffChunks = kOffSmall + (size_t)kStaticRecords * sizeof(TriRecord);
constexpr size_t kOffTiles = kOffChunks + (size_t)kStaticChunks * sizeof(uint32_t);
constexpr size_t kOffHeader = kOffTiles + ((kStaticTiles * sizeof(uint64_t) + 255) / 256) * 256;
constexpr size_t kOffDraw = kOffHeader + 256;
constexpr size_t kOffMvp = kOffDraw + 256;
constexpr size_t kOffFlags = kOffMvp + 256;
constexpr size_t kOffView = kOffFlags + 256;
constexpr size_t kStaticBytes = kOffView + 256;
static_assert(sizeof(ViewRec) <= 256, "view record fits its slot");
static_assert(kOffSmall % 256 == 0 && kOffChunks % 256 == 0 && kOffTiles % 256 == 0, "scratch parts are 256-byte aligned");

static __device__ __align__(256) unsigned char g_static_scratch[kStaticBytes];

struct StaticPrepArgs {
    float proj[16];
    float world[16];
    uint32_t tri_count;
    uint32_t vertex_count;
    ViewRec view;  // the target and fixed-function state of the call
};

// Clears the parts of the shared scratch that must start at zero, and writes the
// single draw and its MVP = proj * world (same arithmetic as the per-draw matrix
// of rz_render's shadow pass).
__global__ void k_static_prep(StaticPrepArgs a) {
    unsigned char* base = g_static_scratch;
    uint64_t* tiles = reinterpret_cast<uint64_t*>(base + kOffTiles);
    for (uint32_t i = threadIdx.x; i < kStaticTiles; i += blockDim.x) tiles[i] = 0;
    if (threadIdx.x == 0) {
        PassHeader* h = reinterpret_cast<PassHeader*>(base + kOffHeader);
        *h = PassHeader{};
        *reinterpret_cast<uint32_t*>(base + kOffFlags) = 0;
        DrawRec* d = reinterpret_cast<DrawRec*>(base + kOffDraw);
        *d = DrawRec{};
        d->tri_count = a.tri_count;
        d->vertex_count = a.vertex_count;
        d->material = -1;
        float C[16];
        mat4_mul(a.proj, a.world, C);
        float* mvp = reinterpret_cast<float*>(base + kOffMvp);
        for (int i = 0; i < 16; ++i) mvp[i] = C[i];
        *reinterpret_cast<ViewRec*>(base + kOffView) = a.view;
    }
}

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
unsigned char* g_static_ptr[kMaxDevices] = {};
int g_static_sms[kMaxDevices] = {};

}  // namespace

}  // namespace rz

using namespace rz;

extern "C" int rz_shadow_depth_static(const void* positions, uint32_t vertex_count, const uint32_t* indices,
                                      uint32_t index_count, const float projection[16], const float world[16],
                                      const rz_draw_config* cfg, uint32_t width, uint32_t height, float* depth_out,
                                      void* stream) {
    if (!positions || !indices || !projection || !world || !cfg || !depth_out) return RZ_INVALID_ARGUMENT;
    if (index_count % 3 != 0 || index_count / 3 > kStaticMaxTriangles) return RZ_INVALID_ARGUMENT;
    if (width == 0 || height == 0 || width > 16384 || height > 16384) return RZ_INVALID_ARGUMENT;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return RZ_ERROR;
    unsigned char* scratch = nullptr;
    int sms = 0;
    {
        std::lock_guard<std::mutex> lock(g_static_mu);
        if (!g_static_ptr[dev]) {
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_static_scratch) != cudaSuccess || !p) return RZ_ERROR;
            int n = 0;
            if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return RZ_ERROR;
            g_static_ptr[dev] = static_cast<unsigned char*>(p);
            g_static_sms[dev] = n;
        }
        scratch = g_static_ptr[dev];
        sms = g_static_sms[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const uint32_t tris = index_count / 3;
    // clear the depth target to 0 (reverse-Z far), as the shadow pass's load op does
    if (cudaMemsetAsync(depth_out, 0, (size_t)width * height * sizeof(float), s) != cudaSuccess) return RZ_ERROR;
    StaticPrepArgs a{};
    for (int i = 0; i < 16; ++i) {
        a.proj[i] = projection[i];
        a.world[i] = world[i];
    }
    a.tri_count = tris;
    a.vertex_count = vertex_count;
    a.view.shadow_w = (int)width;
    a.view.shadow_h = (int)height;
    a.view.width = (int)width;
    a.view.height = (int)height;
    a.view.cull_front = cfg->cull_enabled ? 1 : 0;
    a.view.ccw_front = cfg->reverse_winding_order_enabled ? 1 : 0;
    a.view.bias_enabled = cfg->depth_bias_enabled ? 1 : 0;
    a.view.bias_constant = cfg->depth_bias_constant;
    a.view.bias_clamp = cfg->depth_bias_clamp;
    a.view.bias_slope = cfg->depth_bias_slope_factor;
    a.view.shadow = reinterpret_cast<uint32_t*>(depth_out);
    a.view.cascades = 1;
    a.view.samples = 1;
    k_static_prep<<<1, 128, 0, s>>>(a);
    if (tris) {
        PassParams p{};
        p.draws = reinterpret_cast<const DrawRec*>(scratch + kOffDraw);
        p.draw_count = 1;
        p.tri_total = tris;
        p.chunk_stamps = kChunkStamps;
        p.small_extent = kSmallExtent;
        p.mvp = reinterpret_cast<const float*>(scratch + kOffMvp);
        p.mvp_stride = 16;
        p.pos = static_cast<const float4*>(positions);
        p.indices = indices;
        p.vertex_count = vertex_count;
        p.views = reinterpret_cast<const ViewRec*>(scratch + kOffView);
        p.write_id = 0;
        p.records = reinterpret_cast<TriRecord*>(scratch + kOffRecords);
        p.record_capacity = kStaticRecords;
        p.small_records = reinterpret_cast<TriRecord*>(scratch + kOffSmall);
        p.small_capacity = kStaticRecords;
        p.tile_status = reinterpret_cast<uint64_t*>(scratch + kOffTiles);
        p.chunk_map = reinterpret_cast<uint32_t*>(scratch + kOffChunks);
        p.chunk_capacity = kStaticChunks;
        p.header = reinterpret_cast<PassHeader*>(scratch + kOffHeader);
        p.error_flags = reinterpret_cast<uint32_t*>(scratch + kOffFlags);
        p.lookback_spins = kLookbackSpins;
        p.sample_x = 128;
        p.sample_y = 128;
        p.bb_hi = 128;
        launch_setup(p, s);
        launch_raster(p, sms, s);
    }
    if (cudaGetLastError() != cudaSuccess) return RZ_ERROR;
    uint32_t flags = 0;
    if (cudaMemcpyAsync(&flags, scratch + kOffFlags, sizeof(flags), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return RZ_ERROR;
    if (cudaStreamSynchronize(s) != cudaSuccess) return RZ_ERROR;
    if (flags & (kErrRecordOverflow | kErrStampOverflow)) return RZ_OVERFLOW;
    if (flags) return RZ_GRAPHICS_FRAME_FAILURE;
    return RZ_OK;
}
