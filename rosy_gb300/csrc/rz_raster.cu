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
#include <cstdio>

#include "rz_device.cuh"

namespace rz {

// ---------------------------------------------------------------------------
// per-draw matrices
// ---------------------------------------------------------------------------

__global__ void k_prep(const DrawRec* __restrict__ draws, uint32_t n, const rz_object* __restrict__ objects,
                       const float* __restrict__ P, float* __restrict__ out) {
    const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    if (d >= n) return;
    float A[16], B[16], C[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) A[i] = P[i];
    const float* W = objects[draws[d].object].transform;
#pragma unroll
    for (int i = 0; i < 16; ++i) B[i] = W[i];
    mat4_mul(A, B, C);
#pragma unroll
    for (int i = 0; i < 16; ++i) out[16 * d + i] = C[i];
}

void launch_prep(const DrawRec* draws, uint32_t n, const rz_object* objects, const float* proj16, float* out_mvp,
                 cudaStream_t stream) {
    if (n == 0) return;
    k_prep<<<(n + 127) / 128, 128, 0, stream>>>(draws, n, objects, proj16, out_mvp);
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

// Builds the record of a triangle ordered with S > 0. Returns false if its
// pixel bounding box is empty.
__device__ __forceinline__ bool make_record(const SV& v0, const SV& v1, const SV& v2, int64_t S, const PassParams& P,
                                            uint32_t id, TriRecord& r) {
    const int32_t minX = min(v0.X, min(v1.X, v2.X)), maxX = max(v0.X, max(v1.X, v2.X));
    const int32_t minY = min(v0.Y, min(v1.Y, v2.Y)), maxY = max(v0.Y, max(v1.Y, v2.Y));
    const int px0 = max((minX + 127) >> 8, 0), px1 = min((maxX - 128) >> 8, P.width - 1);
    const int py0 = max((minY + 127) >> 8, 0), py1 = min((maxY - 128) >> 8, P.height - 1);
    if (px0 > px1 || py0 > py1) return false;
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
    r.bias = o;
    r.p0 = (uint32_t)px0 | ((uint32_t)py0 << 16);
    r.p1 = (uint32_t)px1 | ((uint32_t)py1 << 16);
    r.id = id;
    const uint32_t nsx = (uint32_t)((px1 - px0) / kStampW + 1);
    const uint32_t nsy = (uint32_t)((py1 - py0) / kStampH + 1);
    r.stamps = nsx * nsy;
    r.stamp_offset = 0;
    return true;
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
    const float hw = (float)P.width * 0.5f, hh = (float)P.height * 0.5f;
    const uint32_t id = P.write_id ? (tri + 1u) : 0u;
    if (!(o0 | o1 | o2)) {
        if (!(v[0].w > 0.0f) || !(v[1].w > 0.0f) || !(v[2].w > 0.0f)) return;
        const SV a = to_screen(v[0], hw, hh), b = to_screen(v[1], hw, hh), c = to_screen(v[2], hw, hh);
        const int64_t S = area2(a, b, c);
        if (S == 0) return;
        const bool front = P.ccw_front ? (S < 0) : (S > 0);
        if (P.cull_front && front) return;
        TriRecord r;
        if (S > 0) {
            if (make_record(a, b, c, S, P, id, r)) emit(r);
        } else {
            if (make_record(a, c, b, -S, P, id, r)) emit(r);
        }
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
    const bool front = P.ccw_front ? (S < 0) : (S > 0);
    if (P.cull_front && front) return;
    for (int i = 1; i + 1 < n; ++i) {
        const int64_t si = area2(sv[0], sv[i], sv[i + 1]);
        if (si == 0 || ((si > 0) != (S > 0))) continue;
        TriRecord r;
        if (si > 0) {
            if (make_record(sv[0], sv[i], sv[i + 1], si, P, id, r)) emit(r);
        } else {
            if (make_record(sv[0], sv[i + 1], sv[i], -si, P, id, r)) emit(r);
        }
    }
}

struct CountEmit {
    uint32_t recs = 0;
    uint64_t stamps = 0;
    TriRecord first;  // kept for the common case of a single record
    __device__ void operator()(const TriRecord& r) {
        if (recs == 0) first = r;
        ++recs;
        stamps += r.stamps;
    }
};

struct WriteEmit {
    const PassParams* P;
    uint32_t rec;
    uint64_t stamp;
    __device__ void operator()(TriRecord& r) {
        if (rec >= P->record_capacity) {
            atomicOr(P->error_flags, kErrRecordOverflow);
            return;
        }
        r.stamp_offset = stamp;
        TriRecord* dst = P->records + rec;
        const int4* s4 = reinterpret_cast<const int4*>(&r);
        int4* d4 = reinterpret_cast<int4*>(dst);
#pragma unroll
        for (int i = 0; i < 4; ++i) d4[i] = s4[i];
        // chunks whose first stamp lies inside this record start here
        uint64_t k = (stamp + kChunkStamps - 1) / kChunkStamps;
        const uint64_t end = stamp + r.stamps;
        for (; k * kChunkStamps < end; ++k) {
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
    if (threadIdx.x == 0) s_tile = atomicAdd(&P.header->ticket, 1u);
    __syncthreads();
    const uint32_t tile = s_tile;
    const uint32_t tri = tile * kSetupThreads + threadIdx.x;

    CountEmit cnt;
    if (tri < P.tri_total) setup_triangle(P, tri, cnt);

    // CTA-wide inclusive scan of (records, stamps) packed in one 64-bit word.
    const uint64_t mine = ((uint64_t)cnt.recs << kStampBits) | cnt.stamps;
    uint64_t incl = mine;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint64_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    uint64_t warp_prefix = 0, total = 0;
#pragma unroll
    for (int w = 0; w < kSetupThreads / 32; ++w) {
        if (w < warp) warp_prefix += s_warp[w];
        total += s_warp[w];
    }
    const uint64_t excl = warp_prefix + incl - mine;

    // Decoupled look-back (warp 0): publish this tile's aggregate, then sum the
    // predecessors' values 32 at a time until an inclusive prefix is found.
    if (warp == 0) {
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
                    if (++spins > (1u << 22)) {
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
                uint64_t chunks = (st + kChunkStamps - 1) / kChunkStamps;
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
    if (cnt.recs == 0) return;
    WriteEmit w{&P, (uint32_t)(s_base_recs + (excl >> kStampBits)), s_base_stamps + (excl & kStampMask)};
    if (cnt.recs == 1) w(cnt.first);
    else setup_triangle(P, tri, w);
}

int setup_ctas(uint32_t tri_total) { return (int)((tri_total + kSetupThreads - 1) / kSetupThreads); }

void launch_setup(const PassParams& p, cudaStream_t stream) {
    const int ctas = setup_ctas(p.tri_total);
    if (ctas == 0) return;
    k_setup<<<ctas, kSetupThreads, 0, stream>>>(p);
}

// ---------------------------------------------------------------------------
// raster
// ---------------------------------------------------------------------------

// Edge e (from vertex a to vertex b of the S>0-ordered triangle) at sample P:
//   E = dx*(PY - ay) - dy*(PX - ax),   dx = bx - ax, dy = by - ay,
// covered iff E > 0, or E == 0 on a top-left edge (dy < 0, or dy == 0 and dx > 0).
// With the top-left decision folded into the constant (E' = E - 1 on the other
// edges) the test is E' >= 0 for all three edges. Per record each lane keeps its
// constant offset from the stamp origin; per stamp the origin value is two wide
// multiply-adds, and a stamp whose best corner fails an edge is skipped whole.
struct EdgeSetup {
    int64_t c;        // E' at the sample (0, 0) minus nothing: E'(P) = c + dx*PY - dy*PX
    int32_t dx, dy;
    int64_t lane_off; // dx*(ly*256) - dy*(lx*256) for this lane's pixel in the stamp
    int64_t max_off;  // largest lane_off over the stamp (trivial reject)
};

template <bool kWriteId>
__global__ void __launch_bounds__(256, 4) k_raster(PassParams P) {
    const uint32_t chunks = P.header->chunks;
    const uint64_t total = P.header->stamps;
    const int lane = threadIdx.x & 31;
    const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
    const int lx = lane & (kStampW - 1), ly = lane >> 3;
    for (uint32_t k = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; k < chunks; k += warps) {
        uint64_t s = (uint64_t)k * kChunkStamps;
        const uint64_t s_end = (s + kChunkStamps < total) ? (s + kChunkStamps) : total;
        uint32_t r = P.chunk_map[k];
        uint64_t r_end = 0;
        EdgeSetup e[3];
        int32_t X0 = 0, Y0 = 0;
        float z0 = 0.f, dzdx = 0.f, dzdy = 0.f, bias = 0.f;
        int px0 = 0, py0 = 0, px1 = 0, py1 = 0;
        uint32_t nsx = 1, sx = 0, sy = 0, id = 0;
        bool loaded = false;
        while (s < s_end) {
            if (!loaded || s >= r_end) {
                if (loaded) ++r;
                if (r >= P.record_capacity) break;
                const int4* src = reinterpret_cast<const int4*>(P.records + r);
                const int4 q0 = __ldg(src), q1 = __ldg(src + 1), q2 = __ldg(src + 2), q3 = __ldg(src + 3);
                const int32_t X[3] = {q0.x, q0.z, q1.x}, Y[3] = {q0.y, q0.w, q1.y};
                X0 = q0.x;
                Y0 = q0.y;
                z0 = __int_as_float(q1.z);
                dzdx = __int_as_float(q1.w);
                dzdy = __int_as_float(q2.x);
                bias = __int_as_float(q2.y);
                px0 = q2.z & 0xffff;
                py0 = (uint32_t)q2.z >> 16;
                px1 = q2.w & 0xffff;
                py1 = (uint32_t)q2.w >> 16;
                id = (uint32_t)q3.x;
                const uint32_t stamps = (uint32_t)q3.y;
                const uint64_t r_begin = (uint64_t)(uint32_t)q3.z | ((uint64_t)(uint32_t)q3.w << 32);
                r_end = r_begin + stamps;
                nsx = (uint32_t)((px1 - px0) / kStampW + 1);
#pragma unroll
                for (int i = 0; i < 3; ++i) {
                    const int a = (i + 1) % 3, b = (i + 2) % 3;
                    const int32_t dx = X[b] - X[a], dy = Y[b] - Y[a];
                    const bool tl = dy < 0 || (dy == 0 && dx > 0);
                    e[i].dx = dx;
                    e[i].dy = dy;
                    e[i].c = (int64_t)dy * X[a] - (int64_t)dx * Y[a] - (tl ? 0 : 1);
                    e[i].lane_off = (int64_t)dx * (ly * 256) - (int64_t)dy * (lx * 256);
                    e[i].max_off = (dx > 0 ? (int64_t)dx * ((kStampH - 1) * 256) : 0) +
                                   (dy < 0 ? -(int64_t)dy * ((kStampW - 1) * 256) : 0);
                }
                loaded = true;
                if (s < r_begin) {  // cannot happen with a consistent chunk map
                    atomicOr(P.error_flags, kErrStampOverflow);
                    break;
                }
                const uint32_t i = (uint32_t)(s - r_begin);
                sy = i / nsx;
                sx = i - sy * nsx;
            }
            const int sx0 = px0 + (int)sx * kStampW, sy0 = py0 + (int)sy * kStampH;
            const int32_t PXo = sx0 * 256 + 128, PYo = sy0 * 256 + 128;
            int64_t eo[3];
            bool any_out = false;
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                eo[i] = e[i].c + (int64_t)e[i].dx * PYo - (int64_t)e[i].dy * PXo;
                any_out |= (eo[i] + e[i].max_off) < 0;
            }
            if (!any_out) {
                const int px = sx0 + lx, py = sy0 + ly;
                const int64_t E0 = eo[0] + e[0].lane_off, E1 = eo[1] + e[1].lane_off, E2 = eo[2] + e[2].lane_off;
                const bool in = ((int32_t)(E0 >> 32) | (int32_t)(E1 >> 32) | (int32_t)(E2 >> 32)) >= 0;
                if (in && px <= px1 && py <= py1) {
                    const int32_t PX = px * 256 + 128, PY = py * 256 + 128;
                    float z = fmaf(dzdx, (float)(PX - X0), fmaf(dzdy, (float)(PY - Y0), z0));
                    if (!kWriteId) z = z + bias;
                    if (!(z > 0.0f)) z = 0.0f;
                    if (z > 1.0f) z = 1.0f;
                    const size_t p = (size_t)py * (size_t)P.width + (size_t)px;
                    if (kWriteId) {
                        const unsigned long long key = ((unsigned long long)__float_as_uint(z) << 32) | id;
                        atomicMax(reinterpret_cast<unsigned long long*>(P.target) + p, key);
                    } else {
                        atomicMax(reinterpret_cast<unsigned int*>(P.target) + p, __float_as_uint(z));
                    }
                }
            }
            ++s;
            if (++sx == nsx) {
                sx = 0;
                ++sy;
            }
        }
    }
}

void launch_raster(const PassParams& p, int sm_count, cudaStream_t stream) {
    const int blocks = sm_count * 8;
    if (p.write_id) k_raster<true><<<blocks, 256, 0, stream>>>(p);
    else k_raster<false><<<blocks, 256, 0, stream>>>(p);
}

}  // namespace rz
