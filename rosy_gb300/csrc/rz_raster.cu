// Geometry kernels of the shadow depth pass and the camera (visibility) pass.
//
// Reference path: the shadow draw loop (src/Engine/Graphics.cpp:5268-5288)
// running shadowVertexMain (src/shaders/shadow.slang:6-19), and the opaque
// scene draw loop (5631-5653) running the position part of vertexMain
// (src/shaders/basic.slang:116), followed by Vulkan's fixed-function clip,
// viewport, rasterisation, depth bias and GREATER_OR_EQUAL depth test with
// depth write (state at 4989-5040, 5222-5242).
//
// GB300 design:
//  * k_prep: per-draw MVP = P * W (one thread per draw).
//  * k_setup: one thread per triangle pulls its three positions, transforms,
//    clips (guard band + near/far), snaps to 8-bit sub-pixels, culls, and emits
//    64-byte records with the depth plane and bounding box. Records are
//    compacted and their 8x4-pixel stamp counts prefix-summed in the same pass
//    with a decoupled look-back across CTAs; each record also marks the work
//    chunks (kChunkStamps stamps) that start inside it.
//  * k_raster: persistent warps take chunks of stamps, so tiny and huge
//    triangles are balanced alike. A lane is a pixel of the stamp; coverage is
//    the integer edge-function test with the top-left rule, and the depth test
//    is a 64-bit atomicMax on (depth_bits << 32 | id). Because depths are
//    non-negative floats their bit patterns order like the values, so the max
//    key is exactly what a sequential GREATER_OR_EQUAL test leaves: the largest
//    depth, and among equal depths the last triangle submitted. The shadow map
//    is a 32-bit atomicMax on the depth bits.
#include <algorithm>
#include <type_traits>
#include <cstdio>

#include "rz_device.cuh"

namespace rz {

// ---------------------------------------------------------------------------
// per-draw matrices
// ---------------------------------------------------------------------------

// Also zeroes the clear list L (the pass's header and look-back words), so that
// the two need one launch.
__global__ void k_prep(const DrawRec* __restrict__ draws, uint32_t n, const rz_object* __restrict__ objects,
                       const ViewRec* __restrict__ views, float* __restrict__ out, ClearList L) {
    const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    clear_share(L);
    if (d >= n) return;
    const float* P = views[draws[d].view].scene->shadow_projection_near;
    float A[16], B[16], C[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) A[i] = P[i];
    // cascade k: the light's orthographic extent times 2^k, i.e. clip x and y scaled by 2^-k (exact)
    const float s = ldexpf(1.0f, -(int)draws[d].cascade);
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        A[c * 4 + 0] *= s;
        A[c * 4 + 1] *= s;
    }
    const float* W = objects[draws[d].object].transform;
#pragma unroll
    for (int i = 0; i < 16; ++i) B[i] = W[i];
    mat4_mul(A, B, C);
#pragma unroll
    for (int i = 0; i < 16; ++i) out[16 * d + i] = C[i];
}

namespace {
thread_local uint32_t t_launches = 0;
}  // namespace

void note_launch() { ++t_launches; }

uint32_t take_launches() {
    const uint32_t n = t_launches;
    t_launches = 0;
    return n;
}

void launch_prep(const DrawRec* draws, uint32_t n, const rz_object* objects, const ViewRec* views, float* out_mvp,
                 cudaStream_t stream, const ClearList* clear, int sm_count) {
    const ClearList none{};
    const ClearList& L = clear ? *clear : none;
    const unsigned blocks = std::max((n + 127) / 128, clear_blocks(L, sm_count, 128));
    if (blocks == 0) return;
    k_prep<<<blocks, 128, 0, stream>>>(draws, n, objects, views, out_mvp, L);
    note_launch();
}

// ---------------------------------------------------------------------------
// clears (the load-op CLEAR of the depth attachments, scratch headers)
// ---------------------------------------------------------------------------

__global__ void __launch_bounds__(256) k_clear(ClearList L) { clear_share(L); }

unsigned clear_blocks(const ClearList& list, int sm_count, unsigned threads) {
    size_t most = 0;
    for (int b = 0; b < list.count; ++b) most = list.bytes[b] > most ? list.bytes[b] : most;
    if (most == 0) return 0;
    size_t blocks = (most / 16 + threads - 1) / threads;
    const size_t cap = (size_t)sm_count * 8 * (256 / threads);
    if (blocks > cap) blocks = cap;
    return blocks ? (unsigned)blocks : 1u;
}

void launch_clear(const ClearList& list, int sm_count, cudaStream_t stream) {
    const unsigned blocks = clear_blocks(list, sm_count, 256);
    if (blocks == 0) return;
    k_clear<<<blocks, 256, 0, stream>>>(list);
    note_launch();
}

// ---------------------------------------------------------------------------
// triangle setup
// ---------------------------------------------------------------------------

struct CV {
    float x, y, z, w;
};

__device__ __forceinline__ float plane_dist(const CV& c, int p) {
    switch (p) {
        case 0: return c.z;
        case 1: return c.w - c.z;
        case 2: return fmaf(kGuardBand, c.w, c.x);
        case 3: return fmaf(kGuardBand, c.w, -c.x);
        case 4: return fmaf(kGuardBand, c.w, c.y);
        default: return fmaf(kGuardBand, c.w, -c.y);
    }
}

__device__ __forceinline__ unsigned outcode(const CV& c) {
    unsigned m = 0;
#pragma unroll
    for (int p = 0; p < 6; ++p)
        if (!(plane_dist(c, p) >= 0.0f)) m |= 1u << p;
    return m;
}

// Sutherland-Hodgman against the planes in `any` (rare path).
__device__ __noinline__ int clip_polygon(CV* poly, unsigned any) {
    CV buf[9];
    int n = 3;
    for (int p = 0; p < 6 && n > 0; ++p) {
        if (!(any & (1u << p))) continue;
        int m = 0;
        for (int i = 0; i < n; ++i) {
            const CV a = poly[i];
            const CV b = poly[(i + 1) % n];
            const float da = plane_dist(a, p);
            const float db = plane_dist(b, p);
            const bool ia = da >= 0.0f, ib = db >= 0.0f;
            if (ia) buf[m++] = a;
            if (ia != ib) {
                const float t = da / (da - db);
                CV c;
                c.x = fmaf(t, b.x - a.x, a.x);
                c.y = fmaf(t, b.y - a.y, a.y);
                c.z = fmaf(t, b.z - a.z, a.z);
                c.w = fmaf(t, b.w - a.w, a.w);
                buf[m++] = c;
            }
        }
        n = m;
        for (int i = 0; i < n; ++i) poly[i] = buf[i];
    }
    return n >= 3 ? n : 0;
}

struct SV {
    int32_t X, Y;
    float z;
};

__device__ __forceinline__ SV to_screen(const CV& c, float hw, float hh) {
    const float xn = c.x / c.w;
    const float yn = c.y / c.w;
    const float zn = c.z / c.w;
    const float xs = fmaf(xn, hw, hw);
    const float ys = fmaf(yn, hh, hh);
    SV s;
    s.X = (int32_t)rintf(xs * 256.0f);
    s.Y = (int32_t)rintf(ys * 256.0f);
    s.z = zn;
    return s;
}

__device__ __forceinline__ int64_t area2(const SV& a, const SV& b, const SV& c) {
    return (int64_t)(b.X - a.X) * (int64_t)(c.Y - a.Y) - (int64_t)(c.X - a.X) * (int64_t)(b.Y - a.Y);
}

__device__ __forceinline__ uint32_t record_stamps(const TriRecord& r) {
    const int px0 = r.p0 & 0xffff, py0 = r.p0 >> 16, px1 = r.p1 & 0xffff, py1 = r.p1 >> 16;
    return (uint32_t)((px1 - px0) / kStampW + 1) * (uint32_t)((py1 - py0) / kStampH + 1);
}

// Triangles up to this extent (pixels, each way) take the incremental 32-bit
// path: every edge value over the bounding box plus a stamp of overhang is
// below 2 * ((90 + 8) * 256)^2 < 2^31.
constexpr int kMediumExtent = 90;

// The raster facts of a large record (packed by the setup, decoded by
// load_large): the edges' top-left bias, whether the 32-bit incremental walk
// applies (medium), whether the viewport cut its box (clipped), whether float
// offsets from vertex 0 are exact over the box (near_origin), and its stamps per row.
__device__ __forceinline__ uint32_t large_facts(const TriRecord& r, int32_t bb_hi, uint32_t& nsx) {
    const int32_t X[3] = {r.X0, r.X1, r.X2}, Y[3] = {r.Y0, r.Y1, r.Y2};
    const int px0 = (int)(r.p0 & 0xffff), py0 = (int)(r.p0 >> 16), px1 = (int)(r.p1 & 0xffff), py1 = (int)(r.p1 >> 16);
    uint32_t flags = 0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int a = (i + 1) % 3, b = (i + 2) % 3;
        const int32_t dx = X[b] - X[a], dy = Y[b] - Y[a];
        if (!(dy < 0 || (dy == 0 && dx > 0))) flags |= 1u << i;
    }
    const int32_t lo_x = px0 * 256 - X[0], hi_x = px1 * 256 + 256 - X[0] + kStampW * 256;
    const int32_t lo_y = py0 * 256 - Y[0], hi_y = py1 * 256 + 256 - Y[0] + kStampH * 256;
    const int32_t lim = 1 << 23;
    const bool near_origin = lo_x > -lim && hi_x < lim && lo_y > -lim && hi_y < lim;
    const int32_t max_x = max(X[0], max(X[1], X[2])), max_y = max(Y[0], max(Y[1], Y[2]));
    const int32_t ex = max_x - min(X[0], min(X[1], X[2]));
    const int32_t ey = max_y - min(Y[0], min(Y[1], Y[2]));
    // Pixels past an uncut box edge lie outside the triangle's extent, so the edge
    // test alone rejects the stamps' overhang there; only a cut box needs the check.
    const bool clipped = ((max_x - bb_hi) >> 8) > px1 || ((max_y - bb_hi) >> 8) > py1;
    const bool medium = near_origin && ex <= kMediumExtent * 256 && ey <= kMediumExtent * 256;
    flags |= (medium ? 8u : 0u) | (clipped ? 16u : 0u) | (near_origin ? 32u : 0u);
    nsx = (uint32_t)((px1 - px0) / kStampW + 1);
    return flags;
}


// Viewport and fixed-function state of the view a triangle belongs to.
struct ViewState {
    int width, height;
    int bb_lo, bb_hi;  // largest and smallest sample offset (1/256 pixel) of the pass: box of pixels any sample may hit
    int cull_front, ccw_front;
    int bias_enabled;
    float bias_constant, bias_clamp, bias_slope;
    uint32_t view;
};

// Builds the record of a triangle ordered with S > 0. Returns 0 if its pixel
// bounding box is empty, 2 for a small triangle (extent at most kSmallExtent
// pixels each way, rasterised by one lane), 1 otherwise.
__device__ __forceinline__ int make_record(const SV& v0, const SV& v1, const SV& v2, int64_t S, const ViewState& P,
                                           bool ordered, uint32_t small_extent, uint32_t id, TriRecord& r) {
    const int32_t minX = min(v0.X, min(v1.X, v2.X)), maxX = max(v0.X, max(v1.X, v2.X));
    const int32_t minY = min(v0.Y, min(v1.Y, v2.Y)), maxY = max(v0.Y, max(v1.Y, v2.Y));
    // pixels p with minX <= 256 p + o <= maxX for some sample offset o in [bb_hi, bb_lo]
    const int px0 = max((minX - P.bb_lo + 255) >> 8, 0), px1 = min((maxX - P.bb_hi) >> 8, P.width - 1);
    const int py0 = max((minY - P.bb_lo + 255) >> 8, 0), py1 = min((maxY - P.bb_hi) >> 8, P.height - 1);
    if (px0 > px1 || py0 > py1) return 0;
    const float fX1 = (float)(v1.X - v0.X), fY1 = (float)(v1.Y - v0.Y);
    const float fX2 = (float)(v2.X - v0.X), fY2 = (float)(v2.Y - v0.Y);
    const float fS = (float)S;
    const float dz1 = v1.z - v0.z, dz2 = v2.z - v0.z;
    const float dzdx = fmaf(dz1, fY2, -(dz2 * fY1)) / fS;
    const float dzdy = fmaf(dz2, fX1, -(dz1 * fX2)) / fS;
    float o = 0.0f;
    if (P.bias_enabled) {
        // Vulkan depth bias for floating-point depth: m * slope + r * constant,
        // r = 2^(e_max - 23), then clamped.
        const float m = fmaxf(fabsf(dzdx), fabsf(dzdy)) * 256.0f;
        uint32_t e = max((__float_as_uint(fabsf(v0.z)) >> 23) & 0xffu,
                         max((__float_as_uint(fabsf(v1.z)) >> 23) & 0xffu, (__float_as_uint(fabsf(v2.z)) >> 23) & 0xffu));
        const float rr = (e >= 24u) ? __uint_as_float((e - 23u) << 23) : 0.0f;
        o = fmaf(m, P.bias_slope, rr * P.bias_constant);
        if (P.bias_clamp > 0.0f) o = fminf(o, P.bias_clamp);
        else if (P.bias_clamp < 0.0f) o = fmaxf(o, P.bias_clamp);
    }
    r.X0 = v0.X;
    r.Y0 = v0.Y;
    r.X1 = v1.X;
    r.Y1 = v1.Y;
    r.X2 = v2.X;
    r.Y2 = v2.Y;
    r.z0 = v0.z;
    r.dzdx = dzdx;
    r.dzdy = dzdy;
    r.bias = o + 0.0f;  // -0 -> +0 (biased_depth relies on it; the sums are unchanged)
    r.p0 = (uint32_t)px0 | ((uint32_t)py0 << 16);
    r.p1 = (uint32_t)px1 | ((uint32_t)py1 << 16);
    r.id = id;
    r.view = P.view;
    r.stamp_offset = 0;
    const bool small = !ordered && (maxX - minX) <= (int32_t)small_extent * 256 && (maxY - minY) <= (int32_t)small_extent * 256;
    return small ? 2 : 1;
}

// Runs the fixed-function front end for one triangle and hands each record to `emit`.
template <class Emit>
__device__ __forceinline__ void setup_triangle(const PassParams& P, uint32_t tri, Emit& emit) {
    const uint32_t d = find_draw(P.draws, P.draw_count, tri);
    const DrawRec dr = P.draws[d];
    const uint32_t t = tri - dr.tri_base;
    const uint32_t ib = dr.first_index + 3u * t;
    uint32_t vi[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) vi[k] = __ldg(&P.indices[ib + k]) + dr.vertex_base;
    if (vi[0] >= P.vertex_count || vi[1] >= P.vertex_count || vi[2] >= P.vertex_count) {
        atomicOr(P.error_flags, kErrBadIndex);
        return;
    }
    emit.source(d, vi[0] - dr.vertex_base + dr.varying_base, vi[1] - dr.vertex_base + dr.varying_base,
                vi[2] - dr.vertex_base + dr.varying_base);
    const ViewRec& VR = P.views[dr.view];
    ViewState V;
    V.view = dr.view | (dr.cascade << kViewBits);
    V.width = P.write_id ? VR.width : VR.shadow_w;
    V.height = P.write_id ? VR.height : VR.shadow_h;
    const bool msaa = P.write_id && VR.samples > 1;
    V.bb_lo = msaa ? 224 : 128;
    V.bb_hi = msaa ? 32 : 128;
    V.cull_front = P.ordered ? 0 : VR.cull_front;
    V.ccw_front = VR.ccw_front;
    V.bias_enabled = P.write_id ? 0 : VR.bias_enabled;
    V.bias_constant = VR.bias_constant;
    V.bias_clamp = VR.bias_clamp;
    V.bias_slope = VR.bias_slope;
    const float* M = P.mvp + (size_t)P.mvp_stride * d;
    float Mr[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) Mr[i] = __ldg(&M[i]);
    CV v[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float4 p = __ldg(&P.pos[vi[k]]);
        const float4 c = transform_point(Mr, p.x, p.y, p.z);
        v[k] = CV{c.x, c.y, c.z, c.w};
    }
    const unsigned o0 = outcode(v[0]), o1 = outcode(v[1]), o2 = outcode(v[2]);
    if (o0 & o1 & o2) return;
    const float hw = (float)V.width * 0.5f, hh = (float)V.height * 0.5f;
    const uint32_t id = P.write_id ? (tri + 1u) : 0u;
    if (!(o0 | o1 | o2)) {
        if (!(v[0].w > 0.0f) || !(v[1].w > 0.0f) || !(v[2].w > 0.0f)) return;
        const SV a = to_screen(v[0], hw, hh), b = to_screen(v[1], hw, hh), c = to_screen(v[2], hw, hh);
        const int64_t S = area2(a, b, c);
        if (S == 0) return;
        const bool front = V.ccw_front ? (S < 0) : (S > 0);
        if (V.cull_front && front) return;
        TriRecord r;
        const int kind = S > 0 ? make_record(a, b, c, S, V, P.ordered != 0, P.small_extent, id, r) : make_record(a, c, b, -S, V, P.ordered != 0, P.small_extent, id, r);
        if (kind) emit(r, kind == 2);
        return;
    }
    // rare path: clip against the planes the vertices violate, fan-triangulate
    CV poly[9];
    poly[0] = v[0];
    poly[1] = v[1];
    poly[2] = v[2];
    const int n = clip_polygon(poly, o0 | o1 | o2);
    if (n < 3) return;
    for (int i = 0; i < n; ++i)
        if (!(poly[i].w > 0.0f)) return;
    SV sv[9];
    for (int i = 0; i < n; ++i) sv[i] = to_screen(poly[i], hw, hh);
    int64_t S = 0;
    for (int i = 1; i + 1 < n; ++i) S += area2(sv[0], sv[i], sv[i + 1]);
    if (S == 0) return;
    const bool front = V.ccw_front ? (S < 0) : (S > 0);
    if (V.cull_front && front) return;
    for (int i = 1; i + 1 < n; ++i) {
        const int64_t si = area2(sv[0], sv[i], sv[i + 1]);
        if (si == 0 || ((si > 0) != (S > 0))) continue;
        TriRecord r;
        const int kind = si > 0 ? make_record(sv[0], sv[i], sv[i + 1], si, V, P.ordered != 0, P.small_extent, id, r)
                                : make_record(sv[0], sv[i + 1], sv[i], -si, V, P.ordered != 0, P.small_extent, id, r);
        if (kind) emit(r, kind == 2);
    }
}

__device__ __forceinline__ void store_record(TriRecord* dst, const TriRecord& r) {
    const int4* s4 = reinterpret_cast<const int4*>(&r);
    int4* d4 = reinterpret_cast<int4*>(dst);
#pragma unroll
    for (int i = 0; i < 4; ++i) d4[i] = s4[i];
}

// Phase A: count the records (small and large) a triangle produces.
struct CountEmit {
    uint32_t recs = 0;     // large
    uint64_t stamps = 0;   // of the large ones
    uint32_t small = 0;
    TriRecord first;       // the first record, kept for the common case of exactly one
    bool first_small = false;
    uint4* refs = nullptr; // opaque camera pass: where the triangle's draw and vertex records go
    uint32_t tri = 0;
    // every triangle with valid indices stores its draw and the varying records of
    // its vertices: a triangle that owns a pixel of the visibility buffer is one of
    // them, and the shading finds them here (one load instead of a search of the
    // draw list and the index buffer)
    __device__ void source(uint32_t d, uint32_t v0, uint32_t v1, uint32_t v2) {
        if (refs) refs[tri] = make_uint4(d, v0, v1, v2);
    }
    __device__ void operator()(const TriRecord& r, bool is_small) {
        if (recs + small == 0) {
            first = r;
            first_small = is_small;
        }
        if (is_small) {
            ++small;
            return;
        }
        ++recs;
        stamps += record_stamps(r);
    }
};

// Phase B: large records at their compacted index with their stamp offsets,
// small records at their slot in the small list (whose order does not matter:
// the depth test is an atomic max).
struct WriteEmit {
    const PassParams* P;
    uint32_t rec;
    uint64_t stamp;
    uint32_t small;
    __device__ void source(uint32_t, uint32_t, uint32_t, uint32_t) {}
    __device__ void operator()(TriRecord& r, bool is_small) {
        if (is_small) {
            if (small < P->small_capacity) store_record(P->small_records + small, r);
            else atomicOr(P->error_flags, kErrRecordOverflow);
            ++small;
            return;
        }
        if (rec >= P->record_capacity) {
            atomicOr(P->error_flags, kErrRecordOverflow);
            return;
        }
        uint32_t nsx;
        r.view |= large_facts(r, P->bb_hi, nsx) << kRecFlagShift;
        r.stamp_offset = stamp | ((uint64_t)nsx << kStampOffsetBits);
        store_record(P->records + rec, r);
        // chunks whose first stamp lies inside this record start here
        const uint64_t cs = P->chunk_stamps;
        uint64_t k = (stamp + cs - 1) / cs;
        const uint64_t end = stamp + record_stamps(r);
        for (; k * cs < end; ++k) {
            if (k >= P->chunk_capacity) {
                atomicOr(P->error_flags, kErrStampOverflow);
                break;
            }
            P->chunk_map[k] = rec;
        }
        ++rec;
        stamp = end;
    }
};

// Packed scan value: records in bits 40..63, stamps in bits 0..39.
constexpr int kStampBits = 40;
constexpr uint64_t kStampMask = (1ull << kStampBits) - 1;
// Look-back status word: flag (2 bits) | records (24 bits) | stamps (38 bits).
constexpr uint64_t kFlagAgg = 1ull << 62;
constexpr uint64_t kFlagIncl = 2ull << 62;
constexpr int kStatusStampBits = 38;
constexpr uint64_t kStatusStampMask = (1ull << kStatusStampBits) - 1;
constexpr uint64_t kStatusRecMask = (1ull << 24) - 1;

__device__ __forceinline__ uint64_t to_status(uint64_t recs, uint64_t stamps) {
    return (recs << kStatusStampBits) | stamps;
}

__global__ void __launch_bounds__(kSetupThreads) k_setup(PassParams P) {
    __shared__ uint32_t s_tile;
    __shared__ uint64_t s_warp[kSetupThreads / 32];
    __shared__ uint64_t s_base_recs, s_base_stamps;
    __shared__ uint32_t s_small_warp[kSetupThreads / 32];
    __shared__ uint32_t s_small_base;
    // The ordered list's look-back needs tiles numbered in the order the CTAs
    // start (a CTA only waits on tiles that have started); the unordered passes
    // wait on nobody and use the block index, sparing one same-address atomic
    // per CTA.
    if (P.ordered && threadIdx.x == 0) s_tile = atomicAdd(&P.header->ticket, 1u);
    // the pass's depth target is zeroed by the same launch: its stores overlap the
    // setup arithmetic, and the raster (the next launch) sees it cleared
    for (uint32_t b = 0; b < P.clear_count; ++b)
        zero_share(P.clear_ptr[b], P.clear_bytes[b], (size_t)blockIdx.x * blockDim.x + threadIdx.x,
                   (size_t)gridDim.x * blockDim.x);
    const uint32_t tri_ctas = (P.tri_total + kSetupThreads - 1) / kSetupThreads;
    // CTAs launched only to share the zeroing hold no triangles: done
    if (!P.ordered && blockIdx.x >= tri_ctas) return;
    __syncthreads();
    const uint32_t tile = P.ordered ? s_tile : blockIdx.x;
    const uint32_t local = tile * kSetupThreads + threadIdx.x;
    const uint32_t tri = P.tri_offset + local;

    CountEmit cnt;
    cnt.refs = P.tri_refs;
    cnt.tri = tri;
    if (local < P.tri_total) setup_triangle(P, tri, cnt);

    // CTA-wide inclusive scan of (records, stamps) packed in one 64-bit word.
    const uint64_t mine = ((uint64_t)cnt.recs << kStampBits) | cnt.stamps;
    uint64_t incl = mine;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    uint32_t small_incl = cnt.small;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, small_incl, o);
        if (lane >= o) small_incl += v;
    }
    if (lane == 31) {
        s_warp[warp] = incl;
        s_small_warp[warp] = small_incl;
    }
    __syncthreads();
    uint64_t warp_prefix = 0, total = 0;
#pragma unroll
    for (int w = 0; w < kSetupThreads / 32; ++w) {
        if (w < warp) warp_prefix += s_warp[w];
        total += s_warp[w];
    }
    const uint64_t excl = warp_prefix + incl - mine;
    uint32_t small_prefix = 0, small_total = 0;
#pragma unroll
    for (int w = 0; w < kSetupThreads / 32; ++w) {
        if (w < warp) small_prefix += s_small_warp[w];
        small_total += s_small_warp[w];
    }
    const uint32_t small_excl = small_prefix + small_incl - cnt.small;
    if (threadIdx.x == 32) s_small_base = small_total ? atomicAdd(&P.header->small_records, small_total) : 0u;

    // Unordered passes (shadow, opaque camera pass): the depth test is an atomic
    // max, so records may land in any order; one 64-bit atomicAdd per CTA
    // allocates its record slots and its stamp range. The ordered blended list
    // keeps submission order with a decoupled look-back instead.
    if (!P.ordered) {
        if (threadIdx.x == 0) {
            const uint64_t old =
                total ? atomicAdd(reinterpret_cast<unsigned long long*>(&P.header->alloc), (unsigned long long)total) : 0ull;
            s_base_recs = old >> kStampBits;
            s_base_stamps = old & kStampMask;
            __threadfence();
            if (atomicAdd(&P.header->done, 1u) == tri_ctas - 1) {
                // last CTA: publish the totals for the raster and the host
                const uint64_t fin = atomicAdd(reinterpret_cast<unsigned long long*>(&P.header->alloc), 0ull);
                const uint64_t recs = fin >> kStampBits, st = fin & kStampMask;
                uint64_t chunks = (st + P.chunk_stamps - 1) / P.chunk_stamps;
                if (chunks > P.chunk_capacity) {
                    chunks = P.chunk_capacity;
                    atomicOr(P.error_flags, kErrStampOverflow);
                }
                P.header->records = (uint32_t)(recs < (uint64_t)P.record_capacity ? recs : (uint64_t)P.record_capacity);
                P.header->stamps = st;
                P.header->chunks = (uint32_t)chunks;
                P.header->records_needed = recs > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)recs;
            }
        }
    }
    // Decoupled look-back (warp 0): publish this tile's aggregate, then sum the
    // predecessors' values 32 at a time until an inclusive prefix is found.
    if (P.ordered && warp == 0) {
        const uint64_t agg_recs = total >> kStampBits, agg_stamps = total & kStampMask;
        volatile unsigned long long* status = reinterpret_cast<volatile unsigned long long*>(P.tile_status);
        uint64_t pre_recs = 0, pre_stamps = 0;
        if (tile == 0) {
            if (lane == 0) status[0] = kFlagIncl | to_status(agg_recs, agg_stamps);
        } else {
            if (lane == 0) status[tile] = kFlagAgg | to_status(agg_recs, agg_stamps);
            int64_t base = (int64_t)tile - 1;
            uint32_t spins = 0;
            for (;;) {
                const int64_t p = base - lane;
                const uint64_t sv = p >= 0 ? (uint64_t)status[p] : kFlagIncl;
                const uint64_t flag = sv & (3ull << 62);
                const unsigned incl = __ballot_sync(0xffffffffu, flag == kFlagIncl);
                const unsigned zero = __ballot_sync(0xffffffffu, flag == 0);
                const unsigned last = incl ? (unsigned)(__ffs(incl) - 1) : 31u;
                const unsigned need = last == 31u ? 0xffffffffu : ((2u << last) - 1u);
                if (zero & need) {
                    if (++spins > P.lookback_spins) {
                        if (lane == 0) atomicOr(P.error_flags, kErrLookbackTimeout);
                        break;
                    }
                    __nanosleep(32);
                    continue;
                }
                uint64_t rr = (unsigned)lane <= last ? (sv >> kStatusStampBits) & kStatusRecMask : 0;
                uint64_t ss = (unsigned)lane <= last ? sv & kStatusStampMask : 0;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) {
                    rr += __shfl_xor_sync(0xffffffffu, rr, o);
                    ss += __shfl_xor_sync(0xffffffffu, ss, o);
                }
                pre_recs += rr;
                pre_stamps += ss;
                if (incl) break;
                base -= 32;
            }
            if (lane == 0) {
                __threadfence();
                status[tile] = kFlagIncl | to_status(pre_recs + agg_recs, pre_stamps + agg_stamps);
            }
        }
        if (lane == 0) {
            if (pre_recs + agg_recs > kStatusRecMask || pre_stamps + agg_stamps > kStatusStampMask)
                atomicOr(P.error_flags, kErrStampOverflow);
            s_base_recs = pre_recs;
            s_base_stamps = pre_stamps;
            if (tile == gridDim.x - 1) {
                const uint64_t st = pre_stamps + agg_stamps;
                uint64_t chunks = (st + P.chunk_stamps - 1) / P.chunk_stamps;
                if (chunks > P.chunk_capacity) chunks = P.chunk_capacity;
                P.header->records = (uint32_t)((pre_recs + agg_recs) < (uint64_t)P.record_capacity
                                                   ? (pre_recs + agg_recs) : (uint64_t)P.record_capacity);
                P.header->stamps = st;
                P.header->chunks = (uint32_t)chunks;
                const uint64_t need = pre_recs + agg_recs;
                P.header->records_needed = need > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)need;
            }
        }
    }
    __syncthreads();
    if (cnt.recs + cnt.small == 0) return;
    WriteEmit w{&P, (uint32_t)(s_base_recs + (excl >> kStampBits)), s_base_stamps + (excl & kStampMask),
                s_small_base + small_excl};
    if (cnt.recs + cnt.small == 1) w(cnt.first, cnt.first_small);
    else setup_triangle(P, tri, w);
}

int setup_ctas(uint32_t tri_total) { return (int)((tri_total + kSetupThreads - 1) / kSetupThreads); }

void launch_setup(const PassParams& p, cudaStream_t stream) {
    int ctas = setup_ctas(p.tri_total);
    if (ctas == 0) return;
    if (!p.ordered && p.clear_count) {
        // the depth target zeroed by this launch wants more CTAs than few triangles give
        // (about 32 KB each); the extra CTAs, past the last triangle tile, only zero
        // (the ordered list's look-back has one status word per triangle tile)
        size_t most = 0;
        for (uint32_t b = 0; b < p.clear_count; ++b) most = p.clear_bytes[b] > most ? p.clear_bytes[b] : most;
        const size_t want = std::min<size_t>(most / 32768, 4096);
        if ((size_t)ctas < want) ctas = (int)want;
    }
    k_setup<<<ctas, kSetupThreads, 0, stream>>>(p);
    note_launch();
}

// ---------------------------------------------------------------------------
// raster
// ---------------------------------------------------------------------------

// Edge e (from vertex a to vertex b of the S>0-ordered triangle) at sample P:
//   E = dx*(PY - ay) - dy*(PX - ax),   dx = bx - ax, dy = by - ay,
// covered iff E > 0, or E == 0 on a top-left edge (dy < 0, or dy == 0 and dx > 0).
// With the top-left decision folded into the constant (E' = E - 1 on the other
// edges) the test is E' >= 0 on all three edges.

// The target of a view: visibility (camera pass) or shadow map, and its row pitch.
struct Target {
    void* ptr;
    int pitch;
};

template <bool kWriteId>
__device__ __forceinline__ Target view_target(const PassParams& P, uint32_t view) {
    const ViewRec& V = P.views[view & kViewMask];
    if (kWriteId) return Target{V.vis + (size_t)P.sample_plane * (size_t)V.width * (size_t)V.height, V.width};
    return Target{V.shadow + (size_t)((view >> kViewBits) & kCascadeMask) * (size_t)V.shadow_w * (size_t)V.shadow_h,
                  V.shadow_w};
}

// The stored depth of a fragment: the interpolated z plus the record's depth bias
// (+0 in the camera pass), saturated to [0, 1] in the same instruction. The
// saturation maps NaN and every value <= 0 to +0 and every value >= 1 to 1; the
// sum is never -0 because the bias is never -0 (make_record), so this equals
// adding the bias and then clamping with NaN -> 0.
__device__ __forceinline__ float biased_depth(float z, float bias) {
    float r;
    asm("add.rn.sat.f32 %0, %1, %2;" : "=f"(r) : "f"(z), "f"(bias));
    return r;
}

// The pixel's word of the target: u64 visibility key or u32 depth bits.
template <bool kWriteId>
using TargetWord = typename std::conditional<kWriteId, unsigned long long, unsigned int>::type;

template <bool kWriteId>
__device__ __forceinline__ TargetWord<kWriteId>* target_word(const Target& T, int px, int py) {
    return reinterpret_cast<TargetWord<kWriteId>*>(T.ptr) + ((size_t)py * (size_t)T.pitch + (size_t)px);
}

// The depth test and write: atomicMax of the fragment's key (z = biased_depth).
template <bool kWriteId>
__device__ __forceinline__ void write_word(TargetWord<kWriteId>* w, float z, uint32_t id) {
    if (kWriteId) {
        const unsigned long long key = ((unsigned long long)__float_as_uint(z) << 32) | id;
        atomicMax(reinterpret_cast<unsigned long long*>(w), key);
    } else {
        atomicMax(reinterpret_cast<unsigned int*>(w), __float_as_uint(z));
    }
}

template <bool kWriteId>
__device__ __forceinline__ void write_fragment(const Target& T, int px, int py, float z, uint32_t id) {
    write_word<kWriteId>(target_word<kWriteId>(T, px, py), z, id);
}

// One lane rasterises one small triangle: its extent is at most the pass's
// small_extent (<= kMaxSmallExtent = 16 pixels = 4096 sub-pixels) each way, so
// every edge value and product stays below 2^26 and fits in 32 bits.
template <bool kWriteId>
__device__ __forceinline__ void raster_small(const PassParams& P, const TriRecord* rec) {
    const int4* src = reinterpret_cast<const int4*>(rec);
    const int4 q0 = __ldg(src), q1 = __ldg(src + 1), q2 = __ldg(src + 2), q3 = __ldg(src + 3);
    const int32_t X[3] = {q0.x, q0.z, q1.x}, Y[3] = {q0.y, q0.w, q1.y};
    const float z0 = __int_as_float(q1.z), dzdx = __int_as_float(q1.w), dzdy = __int_as_float(q2.x);
    const float bias = __int_as_float(q2.y);
    const int px0 = q2.z & 0xffff, py0 = (uint32_t)q2.z >> 16, px1 = q2.w & 0xffff, py1 = (uint32_t)q2.w >> 16;
    const uint32_t id = (uint32_t)q3.x;
    const Target T = view_target<kWriteId>(P, (uint32_t)q3.y);
    // edge constants relative to vertex 0 (all values < 2^12 sub-pixels, products < 2^24)
    int32_t dx[3], dy[3], c[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int a = (i + 1) % 3, b = (i + 2) % 3;
        dx[i] = X[b] - X[a];
        dy[i] = Y[b] - Y[a];
        const bool tl = dy[i] < 0 || (dy[i] == 0 && dx[i] > 0);
        // E' at (PX, PY) = c + dx*(PY - Y0) - dy*(PX - X0)
        c[i] = dy[i] * (X[a] - X[0]) - dx[i] * (Y[a] - Y[0]) - (tl ? 0 : 1);
    }
    for (int py = py0; py <= py1; ++py) {
        const int32_t ry = py * 256 + P.sample_y - Y[0];
        for (int px = px0; px <= px1; ++px) {
            const int32_t rx = px * 256 + P.sample_x - X[0];
            const int32_t e0 = c[0] + dx[0] * ry - dy[0] * rx;
            const int32_t e1 = c[1] + dx[1] * ry - dy[1] * rx;
            const int32_t e2 = c[2] + dx[2] * ry - dy[2] * rx;
            if ((e0 | e1 | e2) >= 0) {
                const float z = biased_depth(fmaf(dzdx, (float)rx, fmaf(dzdy, (float)ry, z0)), bias);
                write_fragment<kWriteId>(T, px, py, z, id);
            }
        }
    }
}


struct LargeRecord {
    int32_t X[3], Y[3];
    int32_t dx[3], dy[3];
    uint32_t tl_bias[3];  // 0 on top-left edges, 1 otherwise
    bool medium;          // extent <= kMediumExtent px and near_origin: incremental 32-bit walk
    bool clipped;         // the box was cut by the viewport: pixels past px1 / py1 may be inside the triangle
    bool near_origin;     // |PX - X0|, |PY - Y0| < 2^23 over the box: float offsets exact
    int32_t X0, Y0;
    float z0, dzdx, dzdy, bias;
    int px0, py0, px1, py1;
    uint32_t id, nsx, view;
    uint64_t begin, end;
};

// Decodes a large record from its four 16-byte words.
__device__ __forceinline__ void decode_large(const int4 q0, const int4 q1, const int4 q2, const int4 q3, LargeRecord& L) {
    L.X[0] = q0.x;
    L.Y[0] = q0.y;
    L.X[1] = q0.z;
    L.Y[1] = q0.w;
    L.X[2] = q1.x;
    L.Y[2] = q1.y;
    L.X0 = q0.x;
    L.Y0 = q0.y;
    L.z0 = __int_as_float(q1.z);
    L.dzdx = __int_as_float(q1.w);
    L.dzdy = __int_as_float(q2.x);
    L.bias = __int_as_float(q2.y);
    L.px0 = q2.z & 0xffff;
    L.py0 = (uint32_t)q2.z >> 16;
    L.px1 = q2.w & 0xffff;
    L.py1 = (uint32_t)q2.w >> 16;
    L.id = (uint32_t)q3.x;
    const uint32_t flags = (uint32_t)q3.y >> kRecFlagShift;
    L.view = (uint32_t)q3.y & kRecViewMask;
    L.begin = (uint64_t)(uint32_t)q3.z | ((uint64_t)((uint32_t)q3.w & 0xffu) << 32);
    L.nsx = (uint32_t)q3.w >> (kStampOffsetBits - 32);
    L.end = L.begin + (uint64_t)L.nsx * (uint32_t)((L.py1 - L.py0) / kStampH + 1);
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int a = (i + 1) % 3, b = (i + 2) % 3;
        L.dx[i] = L.X[b] - L.X[a];
        L.dy[i] = L.Y[b] - L.Y[a];
        L.tl_bias[i] = (flags >> i) & 1u;
    }
    L.medium = (flags & 8u) != 0;
    L.clipped = (flags & 16u) != 0;
    L.near_origin = (flags & 32u) != 0;
}

__device__ __forceinline__ void load_large(const TriRecord* rec, LargeRecord& L) {
    const int4* src = reinterpret_cast<const int4*>(rec);
    decode_large(__ldg(src), __ldg(src + 1), __ldg(src + 2), __ldg(src + 3), L);
}

// Record staging of the chunk walk: a warp copies the records a chunk starts
// with (one per lane, kStageRecords at most) into shared memory with cp.async
// while it rasterises the chunk before, so that a segment finds its record
// there instead of waiting for a dependent global load.
constexpr int kRasterThreads = 256;
constexpr int kStageRecords = 32;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}

// Lane `lane` copies record r0 + lane when it exists (below n_rec); one commit
// group per call, also when it copies nothing.
__device__ __forceinline__ void stage_records(int4 (*buf)[4], const TriRecord* records, uint32_t r0, uint32_t n_rec,
                                              int lane) {
    if ((uint64_t)r0 + (uint64_t)lane < (uint64_t)n_rec) {
        const int4* src = reinterpret_cast<const int4*>(records + r0 + lane);
#pragma unroll
        for (int i = 0; i < 4; ++i) cp_async16(&buf[lane][i], src + i);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}

// Edge constants of the generic (64-bit) path.
struct GenericEdges {
    int64_t c[3];                    // E' at sub-pixel (0, 0): E'(P) = c + dx*PY - dy*PX
    int64_t max_off[3], min_off[3];  // range of the lane offsets over the stamp
    bool short_edges;                // all |dx|, |dy| < 2^18: partial-edge values and lane offsets fit in 32 bits
};

__device__ __forceinline__ void generic_edges(const LargeRecord& L, GenericEdges& G) {
    bool short_edges = true;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int a = (i + 1) % 3;
        const int32_t dx = L.dx[i], dy = L.dy[i];
        G.c[i] = (int64_t)dy * L.X[a] - (int64_t)dx * L.Y[a] - L.tl_bias[i];
        G.max_off[i] = (dx > 0 ? (int64_t)dx * ((kStampH - 1) * 256) : 0) + (dy < 0 ? -(int64_t)dy * ((kStampW - 1) * 256) : 0);
        G.min_off[i] = (dx < 0 ? (int64_t)dx * ((kStampH - 1) * 256) : 0) + (dy > 0 ? -(int64_t)dy * ((kStampW - 1) * 256) : 0);
        short_edges = short_edges && abs(dx) < (1 << 18) && abs(dy) < (1 << 18);
    }
    G.short_edges = short_edges;
}

// Rasterises stamp (sx, sy) of a large record: lane = pixel (lane & 7, lane >> 3).
// Walk over the stamps of a generic record in raster order: the 64-bit edge
// values at the current stamp's origin sample, advanced by exact constant steps
// (one stamp right, or back to the row start and one stamp down).
struct GenericWalk {
    int64_t e[3], er[3];  // edge values at the current stamp's / the row's first stamp's origin sample
    int sx0, sy0;         // origin pixel of the current stamp
    uint32_t sx;
};

__device__ __forceinline__ void generic_start(const LargeRecord& L, const GenericEdges& G, uint32_t sx, uint32_t sy,
                                              int32_t ox, int32_t oy, GenericWalk& w) {
    w.sx = sx;
    w.sx0 = L.px0 + (int)sx * kStampW;
    w.sy0 = L.py0 + (int)sy * kStampH;
    const int32_t PXo = w.sx0 * 256 + ox, PYo = w.sy0 * 256 + oy, PXr = L.px0 * 256 + ox;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        w.e[i] = G.c[i] + (int64_t)L.dx[i] * PYo - (int64_t)L.dy[i] * PXo;
        w.er[i] = G.c[i] + (int64_t)L.dx[i] * PYo - (int64_t)L.dy[i] * PXr;
    }
}

__device__ __forceinline__ void generic_next(const LargeRecord& L, GenericWalk& w) {
    if (++w.sx == L.nsx) {
        w.sx = 0;
        w.sx0 = L.px0;
        w.sy0 += kStampH;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            w.er[i] += (int64_t)L.dx[i] * (kStampH * 256);
            w.e[i] = w.er[i];
        }
    } else {
        w.sx0 += kStampW;
#pragma unroll
        for (int i = 0; i < 3; ++i) w.e[i] -= (int64_t)L.dy[i] * (kStampW * 256);
    }
}

template <bool kWriteId, bool kBoxCheck>
__device__ __forceinline__ void raster_stamp(const Target& T, const LargeRecord& L, const GenericEdges& G,
                                             const GenericWalk& w, int lx, int ly, int32_t ox, int32_t oy) {
    const int sx0 = w.sx0, sy0 = w.sy0;
    const int32_t PXo = sx0 * 256 + ox, PYo = sy0 * 256 + oy;
    const int64_t* eo = w.e;
    bool reject = false, accept = true;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        reject |= eo[i] + G.max_off[i] < 0;
        accept &= eo[i] + G.min_off[i] >= 0;
    }
    if (reject) return;
    const int px = sx0 + lx, py = sy0 + ly;
    bool in = !kBoxCheck || (px <= L.px1 && py <= L.py1);
    if (!accept) {
        if (G.short_edges) {
            // partial edges: |eo| < 2^30 and the lane offset < 2^30, so 32 bits suffice
            int32_t hi = 0;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const bool edge_accept = eo[i] + G.min_off[i] >= 0;
                const int32_t e = (int32_t)eo[i] + L.dx[i] * (ly * 256) - L.dy[i] * (lx * 256);
                hi |= edge_accept ? 0 : e;
            }
            in = in && hi >= 0;
        } else {
            int32_t hi = 0;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const int64_t e = eo[i] + (int64_t)L.dx[i] * (ly * 256) - (int64_t)L.dy[i] * (lx * 256);
                hi |= (int32_t)(e >> 32);
            }
            in = in && hi >= 0;
        }
    }
    if (!in) return;
    float fx, fy;
    if (L.near_origin) {
        // exact: both terms are integers below 2^24
        fx = (float)(PXo - L.X0) + (float)(lx * 256);
        fy = (float)(PYo - L.Y0) + (float)(ly * 256);
    } else {
        fx = (float)(px * 256 + ox - L.X0);
        fy = (float)(py * 256 + oy - L.Y0);
    }
    const float z = biased_depth(fmaf(L.dzdx, fx, fmaf(L.dzdy, fy, L.z0)), L.bias);
    write_fragment<kWriteId>(T, px, py, z, L.id);
}

// Incremental walk over the stamps of a medium record in raster order. Each
// lane holds its edge values, its float offsets from vertex 0 and the address of
// its pixel's word; moving one stamp right adds a constant, moving to the next
// stamp row restarts from the row's first stamp. The float offsets stay exact
// integers below 2^24, so the depth is bit-identical to
// fma(dzdx, (float)(PX-X0), fma(dzdy, (float)(PY-Y0), z0)).
template <bool kWriteId>
struct MediumWalk {
    int32_t e[3], er[3], stepx[3], stepy[3];
    float fx, fxr, fy, zrow;
    int px, pxr, py;
    TargetWord<kWriteId>* w;   // the lane's pixel in the current stamp
    TargetWord<kWriteId>* wr;  // and in the row's first stamp
};

// Edge values relative to vertex 0 in wrapping 32-bit arithmetic: for a medium
// triangle the true value at every pixel of the walk fits in int32, so the
// wrapped result equals it.
template <bool kWriteId>
__device__ __forceinline__ void medium_start(const Target& T, const LargeRecord& L, uint32_t sx, uint32_t sy, int lx, int ly,
                                             int32_t ox, int32_t oy, MediumWalk<kWriteId>& w) {
    w.pxr = L.px0 + lx;
    w.px = w.pxr + (int)sx * kStampW;
    w.py = L.py0 + (int)sy * kStampH + ly;
    const int32_t rx = w.px * 256 + ox - L.X0, ry = w.py * 256 + oy - L.Y0, rxr = w.pxr * 256 + ox - L.X0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const int a = (i + 1) % 3;
        const uint32_t dx = (uint32_t)L.dx[i], dy = (uint32_t)L.dy[i];
        const uint32_t c = dy * (uint32_t)(L.X[a] - L.X0) - dx * (uint32_t)(L.Y[a] - L.Y0) - L.tl_bias[i];
        w.e[i] = (int32_t)(c + dx * (uint32_t)ry - dy * (uint32_t)rx);
        w.er[i] = (int32_t)(c + dx * (uint32_t)ry - dy * (uint32_t)rxr);
        w.stepx[i] = (int32_t)(0u - dy * (uint32_t)(kStampW * 256));
        w.stepy[i] = (int32_t)(dx * (uint32_t)(kStampH * 256));
    }
    w.fx = (float)rx;
    w.fxr = (float)rxr;
    w.fy = (float)ry;
    w.zrow = fmaf(L.dzdy, w.fy, L.z0);
    w.wr = target_word<kWriteId>(T, w.pxr, w.py);
    w.w = w.wr + (int)sx * kStampW;
}

// n stamps of the walk from stamp column sx: runs along a stamp row, then the
// move to the next row.
template <bool kWriteId, bool kBoxCheck>
__device__ __forceinline__ void medium_walk(const Target& T, const LargeRecord& L, uint32_t sx, uint32_t n,
                                            MediumWalk<kWriteId>& w) {
    const size_t row_step = (size_t)kStampH * (size_t)T.pitch;
    while (true) {
        const uint32_t run = min(n, L.nsx - sx);
        for (uint32_t j = 0; j < run; ++j) {
            if (((w.e[0] | w.e[1] | w.e[2]) >= 0) && (!kBoxCheck || (w.px <= L.px1 && w.py <= L.py1)))
                write_word<kWriteId>(w.w, biased_depth(fmaf(L.dzdx, w.fx, w.zrow), L.bias), L.id);
#pragma unroll
            for (int i = 0; i < 3; ++i) w.e[i] = (int32_t)((uint32_t)w.e[i] + (uint32_t)w.stepx[i]);
            w.w += kStampW;
            w.fx += (float)(kStampW * 256);
            if (kBoxCheck) w.px += kStampW;
        }
        n -= run;
        if (n == 0) return;
        sx = 0;
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            w.er[i] = (int32_t)((uint32_t)w.er[i] + (uint32_t)w.stepy[i]);
            w.e[i] = w.er[i];
        }
        w.wr += row_step;
        w.w = w.wr;
        w.fx = w.fxr;
        w.fy += (float)(kStampH * 256);
        w.zrow = fmaf(L.dzdy, w.fy, L.z0);
        if (kBoxCheck) {
            w.px = w.pxr;
            w.py += kStampH;
        }
    }
}

// Persistent raster: each warp first takes batches of 32 small records (one per
// lane), then chunks of kChunkStamps stamps of the large records, both in a
// fixed grid-stride order. (A shared cursor that every warp bumps with an
// atomic serialises on one L2 line: a raster launch with its work skipped took
// 12 us that way on the 4096^2 shadow pass of 262,144 triangles, 6 us without.)
template <bool kWriteId>
__global__ void __launch_bounds__(kRasterThreads, 3) k_raster(PassParams P) {
    __shared__ int4 s_stage[kRasterThreads / 32][2][kStageRecords][4];
    const int lane = threadIdx.x & 31;
    const int lx = lane & (kStampW - 1), ly = lane >> 3;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const uint32_t warp_id = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint64_t n_small = min(P.header->small_records, P.small_capacity);
    for (uint64_t base = (uint64_t)warp_id * 32u; base < n_small; base += (uint64_t)warps * 32u)
        if (base + lane < n_small) raster_small<kWriteId>(P, P.small_records + base + lane);
    const uint32_t chunks = P.header->chunks;
    const uint64_t total = P.header->stamps;
    const uint32_t n_rec = min(P.header->records, P.record_capacity);  // records the setup wrote
    uint32_t cur_view = 0xffffffffu;  // the view whose target T holds
    Target T{nullptr, 0};
    // chunk k's first record (r_cur, staged in buffer cb), the next chunk's (r_next)
    int cb = 0;
    uint32_t r_cur = warp_id < chunks ? P.chunk_map[warp_id] : n_rec;
    stage_records(s_stage[threadIdx.x >> 5][0], P.records, r_cur, n_rec, lane);
    uint32_t r_next = (uint64_t)warp_id + warps < chunks ? P.chunk_map[warp_id + warps] : n_rec;
    for (uint32_t k = warp_id; k < chunks; k += warps) {
        uint64_t s = (uint64_t)k * P.chunk_stamps;
        const uint64_t s_end = (s + P.chunk_stamps < total) ? (s + P.chunk_stamps) : total;
        // stage the next chunk's records while this one is rasterised, and fetch
        // the chunk map entry of the one after
        stage_records(s_stage[threadIdx.x >> 5][cb ^ 1], P.records, r_next, n_rec, lane);
        const uint64_t k_after = (uint64_t)k + 2u * (uint64_t)warps;
        const uint32_t r_after = k_after < chunks ? P.chunk_map[k_after] : n_rec;
        asm volatile("cp.async.wait_group 1;\n" ::: "memory");  // this lane's copies of chunk k
        __syncwarp();                                          // and every other lane's
        int4 (*const st)[4] = s_stage[threadIdx.x >> 5][cb];
        uint32_t r = r_cur;
        while (s < s_end) {
            if (r >= P.record_capacity) break;
            LargeRecord L;
            const uint32_t j = r - r_cur;
            if (j < (uint32_t)kStageRecords && r < n_rec) decode_large(st[j][0], st[j][1], st[j][2], st[j][3], L);
            else load_large(P.records + r, L);
            if (s < L.begin || s >= L.end) {  // cannot happen with a consistent chunk map
                atomicOr(P.error_flags, kErrStampOverflow);
                break;
            }
            const uint64_t seg_end = s_end < L.end ? s_end : L.end;
            const uint32_t n = (uint32_t)(seg_end - s);
            const uint32_t i = (uint32_t)(s - L.begin);
            const uint32_t sy = i ? i / L.nsx : 0u, sx = i - sy * L.nsx;  // a segment mostly starts at its record's first stamp
            if (L.view != cur_view) {
                T = view_target<kWriteId>(P, L.view);
                cur_view = L.view;
            }
            if (L.medium) {
                MediumWalk<kWriteId> w;
                medium_start<kWriteId>(T, L, sx, sy, lx, ly, P.sample_x, P.sample_y, w);
                if (L.clipped) medium_walk<kWriteId, true>(T, L, sx, n, w);
                else medium_walk<kWriteId, false>(T, L, sx, n, w);
            } else {
                GenericEdges G;
                generic_edges(L, G);
                GenericWalk w;
                generic_start(L, G, sx, sy, P.sample_x, P.sample_y, w);
                if (L.clipped) {
                    for (uint32_t j = 0; j < n; ++j) {
                        raster_stamp<kWriteId, true>(T, L, G, w, lx, ly, P.sample_x, P.sample_y);
                        generic_next(L, w);
                    }
                } else {
                    for (uint32_t j = 0; j < n; ++j) {
                        raster_stamp<kWriteId, false>(T, L, G, w, lx, ly, P.sample_x, P.sample_y);
                        generic_next(L, w);
                    }
                }
            }
            s = seg_end;
            ++r;
        }
        __syncwarp();  // every lane is done with this buffer before it is staged again
        r_cur = r_next;
        r_next = r_after;
        cb ^= 1;
    }
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

void launch_raster(const PassParams& p, int sm_count, cudaStream_t stream) {
    // persistent grid: as many CTAs as can be resident at once
    static int occ[2] = {0, 0};
    const int t = p.write_id ? 1 : 0;
    if (!occ[t]) {
        int n = 0;
        if (p.write_id) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_raster<true>, kRasterThreads, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_raster<false>, kRasterThreads, 0);
        occ[t] = n > 0 ? n : 1;
    }
    const int blocks = sm_count * occ[t];
    if (p.write_id) k_raster<true><<<blocks, kRasterThreads, 0, stream>>>(p);
    else k_raster<false><<<blocks, kRasterThreads, 0, stream>>>(p);
    note_launch();
}

// ---------------------------------------------------------------------------
// debug-line overlay: vertex stage, clipping and viewport of each segment
// ---------------------------------------------------------------------------

// M * (x, y, z, w) as the chain M0r*x -> fma(M1r, y) -> fma(M2r, z) -> fma(M3r, w).
__device__ __forceinline__ CV transform4(const float* __restrict__ M, const float* v) {
    CV o;
    o.x = fmaf(M[12], v[3], fmaf(M[8], v[2], fmaf(M[4], v[1], M[0] * v[0])));
    o.y = fmaf(M[13], v[3], fmaf(M[9], v[2], fmaf(M[5], v[1], M[1] * v[0])));
    o.z = fmaf(M[14], v[3], fmaf(M[10], v[2], fmaf(M[6], v[1], M[2] * v[0])));
    o.w = fmaf(M[15], v[3], fmaf(M[11], v[2], fmaf(M[7], v[1], M[3] * v[0])));
    return o;
}

// debugVertMain (src/shaders/debug.slang:5-35): flags select the space by equality.
__device__ CV debug_vertex(const rz_scene_data& sd, const rz_debug_object& d, const float* v) {
    float M[16];
    CV c;
    if (d.flags == RZ_DEBUG_TRANSFORM_IS_POINTS) return transform4(sd.view_projection, v);
    if (d.flags == RZ_DEBUG_SCREEN_SPACE) {
        const float aspect = sd.draw_extent[0] / sd.draw_extent[1];
        const float q[4] = {v[0], v[1] * aspect, v[2], v[3]};
        c = transform4(d.transform, q);
        c.z = c.w = 1.0f;
        return c;
    }
    if (d.flags == RZ_DEBUG_VIEW_SPACE) {
        mat4_mul(sd.proj, d.transform, M);
        c = transform4(M, v);
        c.z = c.w = 1.0f;
        return c;
    }
    mat4_mul(sd.view_projection, d.transform, M);
    return transform4(M, v);
}

// One thread per (view, segment). The segment is clipped against the triangle
// planes in order (an end outside one plane is replaced by the crossing
// fma(t, b-a, a), t = da/(da-db)), mapped to the viewport and snapped to
// 1/256 pixel; its pixel box is widened by half the line width.
__global__ void __launch_bounds__(128) k_debug_prep(const DebugPair* __restrict__ pairs, uint32_t count,
                                                    const rz_debug_object* __restrict__ objects,
                                                    const ViewRec* __restrict__ views, uint32_t view_count,
                                                    DebugSeg* __restrict__ out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= (uint64_t)count * view_count) return;
    const uint32_t v = (uint32_t)(i / count), k = (uint32_t)(i % count);
    const DebugPair pr = pairs[k];
    const rz_debug_object& d = objects[pr.object];
    const ViewRec& VR = views[v];
    DebugSeg s{};
    s.rgb[0] = d.color[0];
    s.rgb[1] = d.color[1];
    s.rgb[2] = d.color[2];
    CV a = debug_vertex(*VR.scene, d, pr.a), b = debug_vertex(*VR.scene, d, pr.b);
    bool live = true;
    for (int p = 0; p < 6 && live; ++p) {
        const float da = plane_dist(a, p), db = plane_dist(b, p);
        const bool ia = da >= 0.0f, ib = db >= 0.0f;
        if (!ia && !ib) {
            live = false;
        } else if (ia != ib) {
            const float t = da / (da - db);
            CV c;
            c.x = fmaf(t, b.x - a.x, a.x);
            c.y = fmaf(t, b.y - a.y, a.y);
            c.z = fmaf(t, b.z - a.z, a.z);
            c.w = fmaf(t, b.w - a.w, a.w);
            if (ia) b = c;
            else a = c;
        }
    }
    live = live && a.w > 0.0f && b.w > 0.0f;
    if (live) {
        const float hw = (float)VR.width * 0.5f, hh = (float)VR.height * 0.5f;
        const SV sa = to_screen(a, hw, hh), sb = to_screen(b, hw, hh);
        s.X0 = sa.X;
        s.Y0 = sa.Y;
        s.X1 = sb.X;
        s.Y1 = sb.Y;
        s.z0 = sa.z;
        s.z1 = sb.z;
        const int x0 = max(0, (min(sa.X, sb.X) - kDebugHalfWidth) >> 8);
        const int x1 = min(VR.width - 1, (max(sa.X, sb.X) + kDebugHalfWidth) >> 8);
        const int y0 = max(0, (min(sa.Y, sb.Y) - kDebugHalfWidth) >> 8);
        const int y1 = min(VR.height - 1, (max(sa.Y, sb.Y) + kDebugHalfWidth) >> 8);
        live = x0 <= x1 && y0 <= y1;
        if (live) {
            s.p0 = (uint32_t)x0 | ((uint32_t)y0 << 16);
            s.p1 = (uint32_t)x1 | ((uint32_t)y1 << 16);
        }
    }
    s.live = live ? 1u : 0u;
    out[i] = s;
}

void launch_debug_prep(const DebugPair* pairs, uint32_t count, const rz_debug_object* objects, const ViewRec* views,
                       uint32_t view_count, DebugSeg* out, cudaStream_t stream) {
    const uint64_t n = (uint64_t)count * view_count;
    if (n == 0) return;
    k_debug_prep<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(pairs, count, objects, views, view_count, out);
    note_launch();
}

}  // namespace rz
