// ORACLE — test infrastructure only (tests, smoke check, CPU baseline of the
// bench). Never linked into the renderer library.
//
// Scalar CPU restatement of Rosy's frame renderer on the shadow depth pass and
// the mesh forward pass:
//   shadowVertexMain         src/shaders/shadow.slang:6-19
//   vertexMain               src/shaders/basic.slang:16-119
//   fragmentMain             src/shaders/basic.slang:137-344
//   pcf                      src/shaders/pcf.slang:1-11
//   lighting                 src/shaders/lighting.slang:5-43
//   data layouts             src/shaders/data.slang:1-137
//   fixed-function state     src/Engine/Graphics.cpp:4989-5040 (both passes),
//                            5195-5292 (shadow pass), 5566-5691 (scene pass),
//                            5845-5879 (blit to the sRGB swapchain)
//   samplers                 src/Engine/Graphics.cpp:2697-2725, 3421-3438, 3996-4014
//   material packing         src/Engine/Graphics.cpp:4071-4150
//   debug-line overlay       src/shaders/debug.slang:5-35, src/Engine/Graphics.cpp:3222-3249 (vertex
//                            table), 5694-5738 (DRAW DEBUG)
//   draw lists               src/Engine/Graphics.cpp:4691-4735
// and, with no counterpart in the reference, the renderer's sub-pixel sources
// of the learned half-resolution path (oracle_subpixel_sources).
// The fixed-function stages (clipping, viewport, rasterisation, depth bias,
// depth test, texel filtering, depth compare, blending, sRGB conversion) follow
// the Vulkan specification's rules; the reference delegates them to the driver.
//
// Parity is unpinned by the reference (it has no tests or golden data and does
// not build here); hand-derived known-answer tests pin this file instead.
//
// Arithmetic contract of the raster (bit-exact, shared with the CUDA kernels):
//  * per-draw matrix MVP = P * W, element (c,r) = fma chain over k=0..3 of
//    P[k][r]*W[c][k] starting with a plain product (mat4_mul below);
//  * clip = MVP * (x,y,z,1) as fma(M0r,x,M3r) -> fma(M1r,y,.) -> fma(M2r,z,.);
//  * clipping only when a vertex is outside a plane: planes z>=0 (far, reverse-Z),
//    w-z>=0 (near), 64w+-x>=0, 64w+-y>=0 (guard band); Sutherland-Hodgman in
//    plane order, new vertex = fma(t, b-a, a) with t = da/(da-db);
//  * viewport: xs = fma(x/w, W/2, W/2), 8-bit sub-pixel snap rint(xs*256);
//  * facing from the integer polygon area; CW front face unless reversed;
//  * coverage: integer edge functions at pixel centres (256p+128), top-left rule;
//  * depth: plane z0 + dz/dx*(PX-X0) + dz/dy*(PY-Y0) evaluated with two fmas
//    from the first vertex of the S>0-ordered triangle;
//  * depth bias (shadow pass): m = max(|dz/dx|,|dz/dy|) per pixel,
//    r = 2^(e_max-23), o = fma(m, slope, r*constant), clamped; z+o then
//    saturated to [0,1] (NaN -> 0);
//  * depth test GREATER_OR_EQUAL in submission order.
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

constexpr float kGuardBand = 64.0f;

// ----------------------------------------------------------------------------
// fp32 geometry contract
// ----------------------------------------------------------------------------

void mat4_mul(const float* A, const float* B, float* C) {
    for (int c = 0; c < 4; ++c) {
        for (int r = 0; r < 4; ++r) {
            float acc = A[0 * 4 + r] * B[c * 4 + 0];
            acc = std::fmaf(A[1 * 4 + r], B[c * 4 + 1], acc);
            acc = std::fmaf(A[2 * 4 + r], B[c * 4 + 2], acc);
            acc = std::fmaf(A[3 * 4 + r], B[c * 4 + 3], acc);
            C[c * 4 + r] = acc;
        }
    }
}

struct CV {
    float v[4];  // clip-space x, y, z, w
};

CV transform_point(const float* M, const float* p) {
    CV o;
    for (int r = 0; r < 4; ++r) {
        float acc = std::fmaf(M[0 * 4 + r], p[0], M[3 * 4 + r]);
        acc = std::fmaf(M[1 * 4 + r], p[1], acc);
        acc = std::fmaf(M[2 * 4 + r], p[2], acc);
        o.v[r] = acc;
    }
    return o;
}

float plane_dist(const CV& c, int p) {
    switch (p) {
        case 0: return c.v[2];                                  // z >= 0 (far)
        case 1: return c.v[3] - c.v[2];                         // z <= w (near)
        case 2: return std::fmaf(kGuardBand, c.v[3], c.v[0]);   // x >= -G w
        case 3: return std::fmaf(kGuardBand, c.v[3], -c.v[0]);  // x <=  G w
        case 4: return std::fmaf(kGuardBand, c.v[3], c.v[1]);   // y >= -G w
        default: return std::fmaf(kGuardBand, c.v[3], -c.v[1]); // y <=  G w
    }
}

unsigned outcode(const CV& c) {
    unsigned m = 0;
    for (int p = 0; p < 6; ++p)
        if (!(plane_dist(c, p) >= 0.0f)) m |= 1u << p;
    return m;
}

// Clips a triangle to the planes above; returns the vertex count (0 = rejected).
int clip_triangle(const CV in[3], CV out[9]) {
    const unsigned o0 = outcode(in[0]), o1 = outcode(in[1]), o2 = outcode(in[2]);
    if (o0 & o1 & o2) return 0;
    out[0] = in[0];
    out[1] = in[1];
    out[2] = in[2];
    const unsigned any = o0 | o1 | o2;
    if (!any) return 3;
    CV buf[9];
    int n = 3;
    for (int p = 0; p < 6 && n > 0; ++p) {
        if (!(any & (1u << p))) continue;
        int m = 0;
        for (int i = 0; i < n; ++i) {
            const CV& a = out[i];
            const CV& b = out[(i + 1) % n];
            const float da = plane_dist(a, p);
            const float db = plane_dist(b, p);
            const bool ia = da >= 0.0f, ib = db >= 0.0f;
            if (ia) buf[m++] = a;
            if (ia != ib) {
                const float t = da / (da - db);
                CV c;
                for (int k = 0; k < 4; ++k) c.v[k] = std::fmaf(t, b.v[k] - a.v[k], a.v[k]);
                buf[m++] = c;
            }
        }
        n = m;
        for (int i = 0; i < n; ++i) out[i] = buf[i];
    }
    return n >= 3 ? n : 0;
}

struct SV {
    int32_t X, Y;
    float z;
};

SV to_screen(const CV& c, float hw, float hh) {
    const float xn = c.v[0] / c.v[3];
    const float yn = c.v[1] / c.v[3];
    const float zn = c.v[2] / c.v[3];
    const float xs = std::fmaf(xn, hw, hw);
    const float ys = std::fmaf(yn, hh, hh);
    SV s;
    s.X = (int32_t)std::rint(xs * 256.0f);
    s.Y = (int32_t)std::rint(ys * 256.0f);
    s.z = zn;
    return s;
}

int64_t area2(const SV& a, const SV& b, const SV& c) {
    return (int64_t)(b.X - a.X) * (int64_t)(c.Y - a.Y) - (int64_t)(c.X - a.X) * (int64_t)(b.Y - a.Y);
}

struct RasterState {
    int width = 0, height = 0;
    int32_t ox = 128, oy = 128;  // coverage sample within the pixel, 1/256 pixel (centre by default)
    int row_begin = 0, row_end = 0;  // band of rows this thread owns
    bool cull_front = false;
    bool ccw_front = false;
    bool bias = false;
    float bias_constant = 0, bias_clamp = 0, bias_slope = 0;
};

inline uint32_t fbits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}
inline float bitsf(uint32_t u) {
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

// Rasterises one triangle with S > 0 (edges V1->V2, V2->V0, V0->V1 non-negative inside).
template <class Frag>
void raster_tri(const SV& v0, const SV& v1, const SV& v2, int64_t S, const RasterState& rs, Frag&& frag) {
    const float fX1 = (float)(v1.X - v0.X), fY1 = (float)(v1.Y - v0.Y);
    const float fX2 = (float)(v2.X - v0.X), fY2 = (float)(v2.Y - v0.Y);
    const float fS = (float)S;
    const float dz1 = v1.z - v0.z, dz2 = v2.z - v0.z;
    const float dzdx = std::fmaf(dz1, fY2, -(dz2 * fY1)) / fS;
    const float dzdy = std::fmaf(dz2, fX1, -(dz1 * fX2)) / fS;
    float o = 0.0f;
    if (rs.bias) {
        const float m = std::fmax(std::fabs(dzdx), std::fabs(dzdy)) * 256.0f;
        uint32_t e = 0;
        for (float z : {v0.z, v1.z, v2.z}) e = std::max(e, (fbits(std::fabs(z)) >> 23) & 0xffu);
        const float r = (e >= 24u) ? bitsf((e - 23u) << 23) : 0.0f;
        o = std::fmaf(m, rs.bias_slope, r * rs.bias_constant);
        if (rs.bias_clamp > 0.0f) o = std::fmin(o, rs.bias_clamp);
        else if (rs.bias_clamp < 0.0f) o = std::fmax(o, rs.bias_clamp);
    }
    const int32_t minX = std::min({v0.X, v1.X, v2.X}), maxX = std::max({v0.X, v1.X, v2.X});
    const int32_t minY = std::min({v0.Y, v1.Y, v2.Y}), maxY = std::max({v0.Y, v1.Y, v2.Y});
    // pixels whose coverage sample (256 p + o) lies within the triangle's extent
    int px0 = (minX - rs.ox + 255) >> 8, px1 = (maxX - rs.ox) >> 8;
    int py0 = (minY - rs.oy + 255) >> 8, py1 = (maxY - rs.oy) >> 8;
    px0 = std::max(px0, 0);
    px1 = std::min(px1, rs.width - 1);
    py0 = std::max(py0, rs.row_begin);
    py1 = std::min(py1, rs.row_end - 1);
    if (px0 > px1 || py0 > py1) return;
    const SV* V[3] = {&v0, &v1, &v2};
    int32_t ex[3], ey[3], dxs[3], dys[3];
    bool tl[3];
    for (int i = 0; i < 3; ++i) {
        const SV& a = *V[(i + 1) % 3];
        const SV& b = *V[(i + 2) % 3];
        ex[i] = a.X;
        ey[i] = a.Y;
        dxs[i] = b.X - a.X;
        dys[i] = b.Y - a.Y;
        tl[i] = dys[i] < 0 || (dys[i] == 0 && dxs[i] > 0);
    }
    for (int py = py0; py <= py1; ++py) {
        const int32_t PY = py * 256 + rs.oy;
        for (int px = px0; px <= px1; ++px) {
            const int32_t PX = px * 256 + rs.ox;
            bool in = true;
            for (int i = 0; i < 3 && in; ++i) {
                const int64_t E = (int64_t)dxs[i] * (int64_t)(PY - ey[i]) - (int64_t)dys[i] * (int64_t)(PX - ex[i]);
                in = E > 0 || (E == 0 && tl[i]);
            }
            if (!in) continue;
            float z = std::fmaf(dzdx, (float)(PX - v0.X), std::fmaf(dzdy, (float)(PY - v0.Y), v0.z));
            if (rs.bias) z = z + o;
            if (!(z > 0.0f)) z = 0.0f;
            if (z > 1.0f) z = 1.0f;
            frag(px, py, z);
        }
    }
}

// Clip, snap, face-cull and rasterise one primitive.
template <class Frag>
void raster_primitive(const CV clip[3], const RasterState& rs, Frag&& frag) {
    CV poly[9];
    const int n = clip_triangle(clip, poly);
    if (n < 3) return;
    for (int i = 0; i < n; ++i)
        if (!(poly[i].v[3] > 0.0f)) return;
    const float hw = (float)rs.width * 0.5f, hh = (float)rs.height * 0.5f;
    SV sv[9];
    for (int i = 0; i < n; ++i) sv[i] = to_screen(poly[i], hw, hh);
    int64_t S = 0;
    for (int i = 1; i + 1 < n; ++i) S += area2(sv[0], sv[i], sv[i + 1]);
    if (S == 0) return;
    const bool front = rs.ccw_front ? (S < 0) : (S > 0);
    if (rs.cull_front && front) return;
    for (int i = 1; i + 1 < n; ++i) {
        int64_t s = area2(sv[0], sv[i], sv[i + 1]);
        if (s == 0 || ((s > 0) != (S > 0))) continue;
        if (s > 0) raster_tri(sv[0], sv[i], sv[i + 1], s, rs, frag);
        else raster_tri(sv[0], sv[i + 1], sv[i], -s, rs, frag);
    }
}

// ----------------------------------------------------------------------------
// Scene access
// ----------------------------------------------------------------------------

// gpu_material (src/Engine/Graphics.cpp:345-360) as packed at 4071-4150.
struct GpuMaterial {
    float color[4];
    float metallic_factor, roughness_factor, alpha_cutoff;
    uint32_t alpha_mode;
    uint32_t tex[4];      // color, normal, metallic, mixmap image; UINT32_MAX = absent
    uint32_t sampler[4];  // sampler index; sampler_count = the default sampler
};

struct Draw {
    uint32_t vertex_base, first_index, index_count, object, tri_base;
    int material;  // -1 = none
};

struct Ctx {
    const oracle_scene* s;
    std::vector<GpuMaterial> mats;
    std::vector<Draw> shadow, opaque, blended;
    float srgb_table[256];
};

void build_ctx(const oracle_scene* s, Ctx& c) {
    c.s = s;
    for (uint32_t i = 0; i < s->material_count; ++i) {
        const rz_material& m = s->materials[i];
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
            g.sampler[k] = s->sampler_count;  // default sampler
            if (img[k] < s->texture_count) {
                g.tex[k] = img[k];
                if (smp[k] < s->sampler_count) g.sampler[k] = smp[k];
            }
        }
        c.mats.push_back(g);
    }
    uint32_t tri_shadow = 0, tri_opaque = 0, tri_blended = 0;
    for (uint32_t i = 0; i < s->surface_count; ++i) {
        const rz_surface& sf = s->surfaces[i];
        const uint32_t* mesh = s->meshes + 4 * sf.mesh_index;
        Draw d;
        d.vertex_base = mesh[0];
        d.first_index = mesh[2] + sf.start_index;
        d.index_count = sf.index_count;
        d.object = sf.graphic_objects_offset + sf.graphics_object_index;
        d.material = sf.material_index < s->material_count ? (int)sf.material_index : -1;
        d.tri_base = tri_shadow;
        c.shadow.push_back(d);
        tri_shadow += sf.index_count / 3;
        if (sf.blended) {
            d.tri_base = tri_blended;
            c.blended.push_back(d);
            tri_blended += sf.index_count / 3;
        } else {
            d.tri_base = tri_opaque;
            c.opaque.push_back(d);
            tri_opaque += sf.index_count / 3;
        }
    }
    for (int i = 0; i < 256; ++i) {
        const double v = i / 255.0;
        c.srgb_table[i] = (float)(v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4));
    }
}

void draw_mvp(const Ctx& c, const Draw& d, const float* P, float* M) {
    mat4_mul(P, c.s->objects[d.object].transform, M);
}

void tri_clip(const Ctx& c, const Draw& d, const float* M, uint32_t t, CV out[3], uint32_t vi[3]) {
    for (int k = 0; k < 3; ++k) {
        vi[k] = d.vertex_base + c.s->indices[d.first_index + 3 * t + k];
        out[k] = transform_point(M, c.s->vertices[vi[k]].position);
    }
}

template <class F>
void parallel_rows(int rows, int threads, F&& f) {
    if (threads <= 1 || rows < 2 * threads) {
        f(0, rows);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; ++t) {
        const int r0 = (int)((int64_t)rows * t / threads), r1 = (int)((int64_t)rows * (t + 1) / threads);
        pool.emplace_back([&f, r0, r1] { f(r0, r1); });
    }
    for (auto& th : pool) th.join();
}

// Shadow pass: src/Engine/Graphics.cpp:5195-5292 with shadow.slang:6-19.
void shadow_cascade(const Ctx& c, const float* P, float* shadow, int threads);

// Camera-pass samples per pixel (1, or 4 at the standard positions (0.375, 0.125),
// (0.875, 0.375), (0.125, 0.625), (0.625, 0.875) of Vulkan's standardSampleLocations).
int samples_of(const oracle_scene* s) { return s->samples == 4 ? 4 : 1; }
constexpr int32_t kSampleX[4] = {96, 224, 32, 160};
constexpr int32_t kSampleY[4] = {32, 96, 160, 224};

// Shadow cascades: draw_config.shadow_cascades clamped to 1..4 (0 = 1, the reference's single map).
int cascades_of(const oracle_scene* s) {
    const uint32_t n = s->draw_config->shadow_cascades;
    return n < 1 ? 1 : (n > 4 ? 4 : (int)n);
}

// One shadow map per cascade, S x S each, consecutive. Cascade k rasterises with
// shadowProjNear whose clip x and y rows are scaled by 2^-k (exactly).
void shadow_pass(const Ctx& c, float* shadow, int threads) {
    const oracle_scene* s = c.s;
    const int S = (int)s->shadow_size;
    for (int k = 0; k < cascades_of(s); ++k) {
        float P[16];
        for (int i = 0; i < 16; ++i) P[i] = s->scene->shadow_projection_near[i];
        const float sc = std::ldexp(1.0f, -k);
        for (int col = 0; col < 4; ++col) {
            P[col * 4 + 0] *= sc;
            P[col * 4 + 1] *= sc;
        }
        shadow_cascade(c, P, shadow + (size_t)k * S * S, threads);
    }
}

void shadow_cascade(const Ctx& c, const float* P, float* shadow, int threads) {
    const oracle_scene* s = c.s;
    const int S = (int)s->shadow_size;
    std::fill(shadow, shadow + (size_t)S * S, 0.0f);  // clear depth to 0 (5213)
    std::vector<float> mvps(c.shadow.size() * 16);
    for (size_t i = 0; i < c.shadow.size(); ++i) draw_mvp(c, c.shadow[i], P, &mvps[16 * i]);
    parallel_rows(S, threads, [&](int r0, int r1) {
        RasterState rs;
        rs.width = S;
        rs.height = S;
        rs.row_begin = r0;
        rs.row_end = r1;
        rs.cull_front = s->draw_config->cull_enabled != 0;
        rs.ccw_front = s->draw_config->reverse_winding_order_enabled != 0;
        rs.bias = s->draw_config->depth_bias_enabled != 0;
        rs.bias_constant = s->draw_config->depth_bias_constant;
        rs.bias_clamp = s->draw_config->depth_bias_clamp;
        rs.bias_slope = s->draw_config->depth_bias_slope_factor;
        for (size_t di = 0; di < c.shadow.size(); ++di) {
            const Draw& d = c.shadow[di];
            for (uint32_t t = 0; t < d.index_count / 3; ++t) {
                CV cv[3];
                uint32_t vi[3];
                tri_clip(c, d, &mvps[16 * di], t, cv, vi);
                raster_primitive(cv, rs, [&](int px, int py, float z) {
                    float& dst = shadow[(size_t)py * S + px];
                    if (z >= dst) dst = z;  // GREATER_OR_EQUAL, write on
                });
            }
        }
    });
}

// Camera pass depth/visibility: opaque list of src/Engine/Graphics.cpp:5631-5653.
void camera_sample(const Ctx& c, float* depth, uint32_t* ids, int threads, int32_t ox, int32_t oy);

// Depth and triangle id per coverage sample: `samples` planes of W x H.
void camera_pass(const Ctx& c, float* depth, uint32_t* ids, int threads) {
    const int n = samples_of(c.s);
    const size_t plane = (size_t)c.s->width * c.s->height;
    for (int k = 0; k < n; ++k)
        camera_sample(c, depth + k * plane, ids + k * plane, threads, n > 1 ? kSampleX[k] : 128, n > 1 ? kSampleY[k] : 128);
}

void camera_sample(const Ctx& c, float* depth, uint32_t* ids, int threads, int32_t ox, int32_t oy) {
    const oracle_scene* s = c.s;
    const int W = (int)s->width, H = (int)s->height;
    std::fill(depth, depth + (size_t)W * H, 0.0f);
    std::fill(ids, ids + (size_t)W * H, 0u);
    std::vector<float> mvps(c.opaque.size() * 16);
    for (size_t i = 0; i < c.opaque.size(); ++i) draw_mvp(c, c.opaque[i], s->scene->view_projection, &mvps[16 * i]);
    parallel_rows(H, threads, [&](int r0, int r1) {
        RasterState rs;
        rs.width = W;
        rs.height = H;
        rs.ox = ox;
        rs.oy = oy;
        rs.row_begin = r0;
        rs.row_end = r1;
        rs.cull_front = s->draw_config->cull_enabled != 0;
        rs.ccw_front = s->draw_config->reverse_winding_order_enabled != 0;
        for (size_t di = 0; di < c.opaque.size(); ++di) {
            const Draw& d = c.opaque[di];
            for (uint32_t t = 0; t < d.index_count / 3; ++t) {
                CV cv[3];
                uint32_t vi[3];
                tri_clip(c, d, &mvps[16 * di], t, cv, vi);
                const uint32_t id = d.tri_base + t + 1;
                raster_primitive(cv, rs, [&](int px, int py, float z) {
                    const size_t p = (size_t)py * W + px;
                    if (z >= depth[p]) {
                        depth[p] = z;
                        ids[p] = id;
                    }
                });
            }
        }
    });
}

// ----------------------------------------------------------------------------
// Shading (templated: T = float is the graded pipeline, T = double the FP64 reference)
// ----------------------------------------------------------------------------

template <class T>
struct V3 {
    T x, y, z;
};
template <class T> V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> V3<T> mul3(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> T length(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> V3<T> normalize(V3<T> a) {
    const T l = length(a);
    return {a.x / l, a.y / l, a.z / l};
}
template <class T> T fmaxT(T a, T b) { return std::fmax(a, b); }
template <class T> T fminT(T a, T b) { return std::fmin(a, b); }
template <class T> T clamp01(T x) { return fminT<T>(fmaxT<T>(x, T(0)), T(1)); }

// y = M * (v, w) for a column-major 4x4 float matrix, generic precision.
template <class T> void mulm4v(const float* M, const T v[4], T out[4]) {
    for (int r = 0; r < 4; ++r)
        out[r] = (T)M[0 * 4 + r] * v[0] + (T)M[1 * 4 + r] * v[1] + (T)M[2 * 4 + r] * v[2] + (T)M[3 * 4 + r] * v[3];
}
template <class T> void mulm4m4(const T* A, const float* B, T* C) {
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r)
            C[c * 4 + r] = A[0 * 4 + r] * (T)B[c * 4 + 0] + A[1 * 4 + r] * (T)B[c * 4 + 1] +
                           A[2 * 4 + r] * (T)B[c * 4 + 2] + A[3 * 4 + r] * (T)B[c * 4 + 3];
}
template <class T> V3<T> mulm3v(const float* N, V3<T> v) {
    return {(T)N[0] * v.x + (T)N[3] * v.y + (T)N[6] * v.z, (T)N[1] * v.x + (T)N[4] * v.y + (T)N[7] * v.z,
            (T)N[2] * v.x + (T)N[5] * v.y + (T)N[8] * v.z};
}

// BasicVertex varyings (src/shaders/data.slang:10-22) + CSM + clip position.
template <class T>
struct VsOut {
    V3<T> vertex, normal, worldNormal, viewDir, lightDir, tangent, bitangent;
    T color[4];
    T uv[2];
    T sigma;
    T csm[4];
    T clip[4];
};

inline bool valid_index(uint32_t i) { return i < 4294967295u; }

// vertexMain, src/shaders/basic.slang:16-119.
template <class T>
void vertex_main(const Ctx& c, const Draw& d, uint32_t vi, VsOut<T>& o) {
    const rz_scene_data& sd = *c.s->scene;
    const rz_object& gd = c.s->objects[d.object];
    const rz_vertex& v = c.s->vertices[vi];
    const float* worldMat = gd.transform;
    T nt[4] = {(T)v.tangent[0], (T)v.tangent[1], (T)v.tangent[2], (T)v.tangent[3]};
    if (sd.ignore_asset_tangent_sign == 1) nt[3] = T(1);
    if (sd.flip_tangents[0] == 1) nt[0] = nt[0] * T(-1);
    if (sd.flip_tangents[1] == 1) nt[1] = nt[1] * T(-1);
    if (sd.flip_tangents[2] == 1) nt[2] = nt[2] * T(-1);
    if (sd.flip_tangents[3] == 1) nt[3] = nt[3] * T(-1);
    bool tse = sd.tangent_space_enabled == 1;
    if (d.material >= 0 && !valid_index(c.mats[d.material].tex[1])) tse = false;
    const V3<T> vpos{(T)v.position[0], (T)v.position[1], (T)v.position[2]};
    V3<T> normal{(T)v.normal[0], (T)v.normal[1], (T)v.normal[2]};
    V3<T> tangent{nt[0], nt[1], nt[2]};
    V3<T> bitangent = cross(normal, tangent) * nt[3];
    if (sd.ensure_orthogonal_bitangent == 1) {
        const V3<T> normal_projection = bitangent * dot(normal, bitangent);
        const V3<T> ortho_n = normalize(normal - normal_projection);
        const V3<T> tangent_projection = normal_projection - bitangent * dot(tangent, bitangent);
        const V3<T> ortho_t = normalize(tangent - tangent_projection);
        bitangent = cross(ortho_n, ortho_t) * nt[3];
    }
    const T p4[4] = {vpos.x, vpos.y, vpos.z, T(1)};
    T wp[4];
    mulm4v(worldMat, p4, wp);
    V3<T> viewDir{(T)sd.camera_position[0] - wp[0], (T)sd.camera_position[1] - wp[1], (T)sd.camera_position[2] - wp[2]};
    V3<T> lightDir{(T)sd.sun_position[0] - wp[0], (T)sd.sun_position[1] - wp[1], (T)sd.sun_position[2] - wp[2]};
    if (tse) {
        const T cam[4] = {(T)sd.camera_position[0], (T)sd.camera_position[1], (T)sd.camera_position[2], (T)sd.camera_position[3]};
        const T sun[4] = {(T)sd.sun_position[0], (T)sd.sun_position[1], (T)sd.sun_position[2], (T)sd.sun_position[3]};
        T co[4], so[4];
        mulm4v(gd.to_object_space_transform, cam, co);
        mulm4v(gd.to_object_space_transform, sun, so);
        viewDir = V3<T>{co[0], co[1], co[2]} - vpos;
        lightDir = V3<T>{so[0], so[1], so[2]} - vpos;
    } else {
        normal = normalize(mulm3v<T>(gd.normal_transform, V3<T>{(T)v.normal[0], (T)v.normal[1], (T)v.normal[2]}));
        tangent = normalize(mulm3v<T>(gd.normal_transform, V3<T>{nt[0], nt[1], nt[2]}));
        tangent = normalize(tangent - normal * dot(normal, tangent));
    }
    if (sd.flip_lights[0] == 1) lightDir.x = lightDir.x * T(-1);
    if (sd.flip_lights[1] == 1) lightDir.y = lightDir.y * T(-1);
    if (sd.flip_lights[2] == 1) lightDir.z = lightDir.z * T(-1);
    o.vertex = V3<T>{wp[0] / wp[3], wp[1] / wp[3], wp[2] / wp[3]};
    o.normal = normal;
    o.worldNormal = mulm3v<T>(gd.normal_transform, V3<T>{(T)v.normal[0], (T)v.normal[1], (T)v.normal[2]});
    for (int k = 0; k < 4; ++k) o.color[k] = (T)v.color[k];
    o.tangent = V3<T>{nt[0], nt[1], nt[2]};
    o.bitangent = bitangent;
    o.viewDir = viewDir;
    o.lightDir = lightDir;
    o.sigma = nt[3];
    o.uv[0] = (T)v.uv[0];
    o.uv[1] = (T)v.uv[1];
    // csm.near = ((ndc_to_tc * shadowProjNear) * worldMat) * pos; ndc_to_tc rows
    // (0.5,0,0,0.5), (0,0.5,0,0.5), (0,0,1,0), (0,0,0,1) (basic.slang:24).
    {
        const float* P = sd.shadow_projection_near;
        T A[16];
        for (int col = 0; col < 4; ++col) {
            const T x = (T)P[col * 4 + 0], y = (T)P[col * 4 + 1], z = (T)P[col * 4 + 2], w = (T)P[col * 4 + 3];
            A[col * 4 + 0] = T(0.5) * x + T(0.5) * w;
            A[col * 4 + 1] = T(0.5) * y + T(0.5) * w;
            A[col * 4 + 2] = z;
            A[col * 4 + 3] = w;
        }
        T B[16];
        mulm4m4(A, worldMat, B);
        for (int r = 0; r < 4; ++r) o.csm[r] = B[0 * 4 + r] * p4[0] + B[1 * 4 + r] * p4[1] + B[2 * 4 + r] * p4[2] + B[3 * 4 + r];
    }
}

// Clip position through the fp32 raster contract (identical to what rasterised the pixel).
template <class T>
void clip_position(const Ctx& c, const Draw& d, uint32_t vi, T out[4]) {
    if constexpr (sizeof(T) == 4) {
        float M[16];
        mat4_mul(c.s->scene->view_projection, c.s->objects[d.object].transform, M);
        const CV cv = transform_point(M, c.s->vertices[vi].position);
        for (int k = 0; k < 4; ++k) out[k] = cv.v[k];
    } else {
        T VP[16];
        for (int k = 0; k < 16; ++k) VP[k] = (T)c.s->scene->view_projection[k];
        T M[16];
        mulm4m4(VP, c.s->objects[d.object].transform, M);
        const float* p = c.s->vertices[vi].position;
        for (int r = 0; r < 4; ++r) out[r] = M[0 * 4 + r] * (T)p[0] + M[1 * 4 + r] * (T)p[1] + M[2 * 4 + r] * (T)p[2] + M[3 * 4 + r];
    }
}

// Perspective-correct barycentrics at pixel centre (px, py) from clip positions
// (2D homogeneous form; equals the Vulkan perspective interpolation weights).
template <class T>
void barycentrics(const T c0[4], const T c1[4], const T c2[4], int px, int py, int W, int H, T b[3]) {
    const T xn = (T)(2 * px + 1 - W) / (T)W;
    const T yn = (T)(2 * py + 1 - H) / (T)H;
    const V3<T> v0{c0[0], c0[1], c0[3]}, v1{c1[0], c1[1], c1[3]}, v2{c2[0], c2[1], c2[3]};
    const V3<T> p{xn, yn, T(1)};
    const T b0 = dot(cross(v1, v2), p), b1 = dot(cross(v2, v0), p), b2 = dot(cross(v0, v1), p);
    const T inv = T(1) / (b0 + b1 + b2);
    b[0] = b0 * inv;
    b[1] = b1 * inv;
    b[2] = b2 * inv;
}

template <class T>
struct Frag {
    V3<T> normal, worldNormal, viewDir, lightDir, tangent, bitangent;
    T color[4];
    T uv[2];
    T sigma;
    T csm[4];
    T duvdx[2], duvdy[2];
};

template <class T> V3<T> lerp3(const V3<T>* a, const T b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

template <class T>
void interpolate(const VsOut<T> v[3], const T b[3], Frag<T>& f) {
    V3<T> t[3];
    for (int k = 0; k < 3; ++k) t[k] = v[k].normal;
    f.normal = lerp3(t, b);
    for (int k = 0; k < 3; ++k) t[k] = v[k].worldNormal;
    f.worldNormal = lerp3(t, b);
    for (int k = 0; k < 3; ++k) t[k] = v[k].viewDir;
    f.viewDir = lerp3(t, b);
    for (int k = 0; k < 3; ++k) t[k] = v[k].lightDir;
    f.lightDir = lerp3(t, b);
    for (int k = 0; k < 3; ++k) t[k] = v[k].tangent;
    f.tangent = lerp3(t, b);
    for (int k = 0; k < 3; ++k) t[k] = v[k].bitangent;
    f.bitangent = lerp3(t, b);
    for (int i = 0; i < 4; ++i) f.color[i] = v[0].color[i] * b[0] + v[1].color[i] * b[1] + v[2].color[i] * b[2];
    for (int i = 0; i < 2; ++i) f.uv[i] = v[0].uv[i] * b[0] + v[1].uv[i] * b[1] + v[2].uv[i] * b[2];
    f.sigma = v[0].sigma * b[0] + v[1].sigma * b[1] + v[2].sigma * b[2];
    for (int i = 0; i < 4; ++i) f.csm[i] = v[0].csm[i] * b[0] + v[1].csm[i] * b[1] + v[2].csm[i] * b[2];
}

// --- texture sampling (Vulkan texel filtering restated) ---

struct SamplerState {
    bool min_linear, mag_linear, mip_linear;
    int wrap_u, wrap_v;  // 0 clamp-to-edge, 1 mirrored repeat, 2 repeat
};

SamplerState sampler_state(const Ctx& c, uint32_t idx) {
    SamplerState st;
    if (idx >= c.s->sampler_count) {  // default sampler, src/Engine/Graphics.cpp:3421-3438
        st.min_linear = st.mag_linear = true;
        st.mip_linear = false;
        st.wrap_u = st.wrap_v = 2;
        return st;
    }
    const rz_sampler& s = c.s->samplers[idx];  // src/Engine/Graphics.cpp:250-278, 3996-4014
    st.min_linear = !(s.min_filter <= 2);
    st.mag_linear = !(s.mag_filter <= 2);
    st.mip_linear = true;
    st.wrap_u = s.wrap_s == 0 ? 0 : (s.wrap_s == 1 ? 1 : 2);
    st.wrap_v = s.wrap_t == 0 ? 0 : (s.wrap_t == 1 ? 1 : 2);
    return st;
}

inline int wrap_coord(int i, int size, int mode) {
    if (mode == 0) return std::min(std::max(i, 0), size - 1);
    if (mode == 2) {
        int m = i % size;
        return m < 0 ? m + size : m;
    }
    // mirrored repeat: (size-1) - mirror((i mod 2size) - size), mirror(a) = a>=0 ? a : -(1+a)
    int t = i % (2 * size);
    if (t < 0) t += 2 * size;
    int a = t - size;
    a = a >= 0 ? a : -(1 + a);
    return size - 1 - a;
}

struct TexMarks {
    std::vector<std::vector<uint8_t>> levels;  // per texture: concatenated per-texel marks
};

template <class T>
struct Sampling {
    const Ctx* c;
    TexMarks* marks;  // may be null

    void texel(const rz_texture& t, uint32_t tex_index, size_t level_off_texels, int w, int i, int j, T out[4]) const {
        const size_t idx = level_off_texels + (size_t)j * w + i;
        const uint8_t* p = (const uint8_t*)t.texels + idx * 4;
        if (marks) __atomic_store_n(&marks->levels[tex_index][idx], (uint8_t)1, __ATOMIC_RELAXED);
        const bool srgb = t.image_type != RZ_IMAGE_NORMAL_MAP;
        for (int k = 0; k < 3; ++k) {
            if (srgb) {
                if constexpr (sizeof(T) == 4) out[k] = c->srgb_table[p[k]];
                else {
                    const double v = p[k] / 255.0;
                    out[k] = v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4);
                }
            } else {
                out[k] = (T)p[k] / T(255);
            }
        }
        out[3] = (T)p[3] / T(255);
    }

    void sample_level(const rz_texture& t, uint32_t ti, int level, bool linear, const SamplerState& st, T u, T v, T out[4]) const {
        const int w = std::max(1, (int)(t.width >> level)), h = std::max(1, (int)(t.height >> level));
        size_t off = 0;
        for (int l = 0; l < level; ++l) off += (size_t)std::max(1u, t.width >> l) * std::max(1u, t.height >> l);
        if (!linear) {
            const int i = (int)std::floor(u * (T)w), j = (int)std::floor(v * (T)h);
            texel(t, ti, off, w, wrap_coord(i, w, st.wrap_u), wrap_coord(j, h, st.wrap_v), out);
            return;
        }
        const T uu = u * (T)w - T(0.5), vv = v * (T)h - T(0.5);
        const T fi = std::floor(uu), fj = std::floor(vv);
        const T a = uu - fi, b = vv - fj;
        const int i0 = (int)fi, j0 = (int)fj;
        const int x0 = wrap_coord(i0, w, st.wrap_u), x1 = wrap_coord(i0 + 1, w, st.wrap_u);
        const int y0 = wrap_coord(j0, h, st.wrap_v), y1 = wrap_coord(j0 + 1, h, st.wrap_v);
        T t00[4], t10[4], t01[4], t11[4];
        texel(t, ti, off, w, x0, y0, t00);
        texel(t, ti, off, w, x1, y0, t10);
        texel(t, ti, off, w, x0, y1, t01);
        texel(t, ti, off, w, x1, y1, t11);
        for (int k = 0; k < 4; ++k) {
            const T top = t00[k] + a * (t10[k] - t00[k]);
            const T bot = t01[k] + a * (t11[k] - t01[k]);
            out[k] = top + b * (bot - top);
        }
    }

    // texture2D.Sample with implicit derivatives.
    void sample(uint32_t tex_index, uint32_t sampler_index, const Frag<T>& f, T out[4]) const {
        if (tex_index >= c->s->texture_count) {  // absent image: robust null descriptor reads 0
            out[0] = out[1] = out[2] = out[3] = T(0);
            return;
        }
        const rz_texture& t = c->s->textures[tex_index];
        const SamplerState st = sampler_state(*c, sampler_index);
        const T w0 = (T)t.width, h0 = (T)t.height;
        const T ax = f.duvdx[0] * w0, ay = f.duvdx[1] * h0, bx = f.duvdy[0] * w0, by = f.duvdy[1] * h0;
        const T rx2 = ax * ax + ay * ay, ry2 = bx * bx + by * by;
        const T rho2 = fmaxT<T>(rx2, ry2);
        const int q = (int)t.levels - 1;
        if (!(rho2 > T(1))) {  // lambda <= 0: magnification, level 0
            sample_level(t, tex_index, 0, st.mag_linear, st, f.uv[0], f.uv[1], out);
            return;
        }
        if (!st.mip_linear) {
            // nearest mip: d = ceil(lambda + 0.5) - 1, i.e. the count of k >= 1 with rho^2 > 2^(2k-1)
            int d = 0;
            T thr = T(2);
            while (d < q && rho2 > thr) {
                ++d;
                thr = thr * T(4);
            }
            sample_level(t, tex_index, d, st.min_linear, st, f.uv[0], f.uv[1], out);
            return;
        }
        const T lambda = T(0.5) * std::log2(rho2);
        const T dp = fminT<T>(lambda, (T)q);
        const int dlo = (int)std::floor(dp);
        const int dhi = std::min(dlo + 1, q);
        const T delta = dp - (T)dlo;
        T a[4], b[4];
        sample_level(t, tex_index, dlo, st.min_linear, st, f.uv[0], f.uv[1], a);
        if (delta > T(0) && dhi != dlo) {
            sample_level(t, tex_index, dhi, st.min_linear, st, f.uv[0], f.uv[1], b);
            for (int k = 0; k < 4; ++k) out[k] = a[k] + delta * (b[k] - a[k]);
        } else {
            for (int k = 0; k < 4; ++k) out[k] = a[k];
        }
    }
};

// SampleCmpLevelZero with the shadow sampler of src/Engine/Graphics.cpp:2697-2725:
// linear filter, clamp-to-edge, compare GREATER_OR_EQUAL (Dref >= texel passes).
template <class T>
T sample_cmp(const float* shadow, int S, T u, T v, T dref, std::vector<uint8_t>* marks) {
    const T uu = u * (T)S - T(0.5), vv = v * (T)S - T(0.5);
    const T fi = std::floor(uu), fj = std::floor(vv);
    const T a = uu - fi, b = vv - fj;
    const int i0 = (int)std::max<T>(std::min<T>(fi, (T)(S + 1)), T(-2)), j0 = (int)std::max<T>(std::min<T>(fj, (T)(S + 1)), T(-2));
    const int x0 = std::min(std::max(i0, 0), S - 1), x1 = std::min(std::max(i0 + 1, 0), S - 1);
    const int y0 = std::min(std::max(j0, 0), S - 1), y1 = std::min(std::max(j0 + 1, 0), S - 1);
    auto cmp = [&](int x, int y) -> T {
        if (marks) __atomic_store_n(&(*marks)[(size_t)y * S + x], (uint8_t)1, __ATOMIC_RELAXED);
        return dref >= (T)shadow[(size_t)y * S + x] ? T(1) : T(0);
    };
    const T c00 = cmp(x0, y0), c10 = cmp(x1, y0), c01 = cmp(x0, y1), c11 = cmp(x1, y1);
    const T top = c00 + a * (c10 - c00);
    const T bot = c01 + a * (c11 - c01);
    return top + b * (bot - top);
}

// pcf, src/shaders/pcf.slang:1-11 (5 taps) and the 3x3 option.
template <class T>
T pcf(const float* shadow, int S, const T csm[4], uint32_t mode, std::vector<uint8_t>* marks) {
    T result = T(0);
    if (mode == RZ_PCF_3X3) {
        const T o = T(1) / (T)S;
        for (int j = -1; j <= 1; ++j)
            for (int i = -1; i <= 1; ++i)
                result += sample_cmp<T>(shadow, S, csm[0] + (T)i * o, csm[1] + (T)j * o, csm[2], marks);
        return result * (T(1) / T(9));
    }
    const T o = T(0.00025);
    result += sample_cmp<T>(shadow, S, csm[0] - o, csm[1] - o, csm[2], marks);
    result += sample_cmp<T>(shadow, S, csm[0] + o * T(2), csm[1], csm[2], marks);
    result += sample_cmp<T>(shadow, S, csm[0], csm[1] + o * T(2), csm[2], marks);
    result += sample_cmp<T>(shadow, S, csm[0] + o * T(2), csm[1] + o * T(2), csm[2], marks);
    result += sample_cmp<T>(shadow, S, csm[0] - o * T(2), csm[1] - o * T(2), csm[2], marks);
    return result * (T(1) / T(5));
}

// lighting.slang:5-43
template <class T> V3<T> schlick_fresnel(T vDotH, V3<T> f0) {
    const T p = std::pow(clamp01<T>(T(1) - vDotH), T(5));
    return {f0.x + (T(1) - f0.x) * p, f0.y + (T(1) - f0.y) * p, f0.z + (T(1) - f0.z) * p};
}
template <class T> T distribution_ggx(V3<T> N, V3<T> H, T roughness) {
    const T PI = T(3.14159265359);
    const T a = roughness * roughness;
    const T a2 = a * a;
    const T NdotH = fmaxT<T>(dot(N, H), T(0));
    const T NdotH2 = NdotH * NdotH;
    T denom = (NdotH2 * (a2 - T(1)) + T(1));
    denom = PI * denom * denom;
    return a2 / denom;
}
template <class T> T geometry_schlick_ggx(T NdotV, T roughness) {
    const T r = roughness + T(1);
    const T k = (r * r) / T(8);
    return NdotV / (NdotV * (T(1) - k) + k);
}
template <class T> T geometry_smith(V3<T> N, V3<T> V, V3<T> L, T roughness) {
    const T NdotV = fmaxT<T>(dot(N, V), T(0));
    const T NdotL = fmaxT<T>(dot(N, L), T(0));
    return geometry_schlick_ggx(NdotL, roughness) * geometry_schlick_ggx(NdotV, roughness);
}

// fragmentMain, src/shaders/basic.slang:137-344. Returns false on discard.
template <class T>
bool fragment_main(const Ctx& c, const Draw& d, const Frag<T>& bv, const float* shadow, const Sampling<T>& smp,
                   std::vector<uint8_t>* shadow_marks, T out[4]) {
    const rz_scene_data& sd = *c.s->scene;
    const V3<T> ambientLight{(T)sd.ambient_color[0], (T)sd.ambient_color[1], (T)sd.ambient_color[2]};
    T outFragColor[4] = {bv.color[0], bv.color[1], bv.color[2], bv.color[3]};
    T imageTextureColor[4] = {outFragColor[0], outFragColor[1], outFragColor[2], outFragColor[3]};
    T alpha = bv.color[3];
    T sampledRoughness = T(0), sampledMetallic = T(0);
    T roughness = T(0), metallic = T(0);
    const bool hasMaterial = d.material >= 0;
    V3<T> lightNormal = normalize(bv.normal);
    const V3<T> lightDir = normalize(bv.lightDir);
    const V3<T> bitangent = bv.bitangent;
    const GpuMaterial* md = hasMaterial ? &c.mats[d.material] : nullptr;
    if (hasMaterial) {
        for (int k = 0; k < 4; ++k) outFragColor[k] = (T)md->color[k];
        for (int k = 0; k < 4; ++k) imageTextureColor[k] = outFragColor[k];
        alpha = fminT<T>((T)md->color[3], alpha);
        if (sd.normal_maps_enabled == 1 && valid_index(md->tex[1])) {
            T s[4];
            smp.sample(md->tex[1], md->sampler[1], bv, s);
            const V3<T> m{s[0] * T(2) - T(1), s[1] * T(2) - T(1), s[2] * T(2) - T(1)};
            const V3<T> n = normalize(bv.normal);
            const V3<T> t = normalize(bv.tangent - n * dot(bv.tangent, n));
            const V3<T> b = normalize(cross(bv.normal, bv.tangent) * bv.sigma);
            lightNormal = normalize(t * m.x + b * m.y + n * m.z);
        }
        if (valid_index(md->tex[0])) {
            smp.sample(md->tex[0], md->sampler[0], bv, imageTextureColor);
            alpha = fminT<T>(imageTextureColor[3], alpha);
        }
        const bool hasMixmap = valid_index(md->tex[3]);
        T s[4];
        if (hasMixmap) smp.sample(md->tex[3], md->sampler[3], bv, s);
        else smp.sample(md->tex[2], md->sampler[2], bv, s);  // sampled even when absent (basic.slang:210-221)
        sampledRoughness = s[1];
        sampledMetallic = s[2];
    }
    const V3<T> V = normalize(bv.viewDir);
    const V3<T> L = lightDir;
    const V3<T> N = lightNormal;
    const V3<T> H = normalize(L + V);
    const T cosTheta = clamp01<T>(dot(L, N));
    const T cosPhi = clamp01<T>(dot(H, N));
    const T lDotN = cosTheta;
    const T lDotH = clamp01<T>(dot(L, H));
    const T nDotV = clamp01<T>(dot(N, V));
    auto set3 = [&](V3<T> v) {
        outFragColor[0] = v.x;
        outFragColor[1] = v.y;
        outFragColor[2] = v.z;
        outFragColor[3] = alpha;
    };
    const T half = T(0.5);
    auto enc = [&](V3<T> v) { return V3<T>{v.x * half + half, v.y * half + half, v.z * half + half}; };
    switch (sd.fragment_output) {
        case 0: set3({imageTextureColor[0], imageTextureColor[1], imageTextureColor[2]}); break;
        case 1: set3(enc(normalize(bv.worldNormal))); break;
        case 2: set3(enc(normalize(bv.tangent))); break;
        case 3: set3(enc(normalize(bv.lightDir))); break;
        case 4: set3(enc(normalize(bv.viewDir))); break;
        case 5: set3({bv.color[0], bv.color[1], bv.color[2]}); break;
        case 6: set3(enc(lightNormal)); break;
        case 7: set3(enc(bitangent)); break;
        case 8: set3(enc({cosTheta, cosTheta, cosTheta})); break;
        case 9: set3(enc({cosPhi, cosPhi, cosPhi})); break;
        case 10: set3(enc({lDotH, lDotH, lDotH})); break;
        case 11: set3(enc({nDotV, nDotV, nDotV})); break;
        case 12: set3({bv.uv[0], bv.uv[1], T(0)}); break;
        case 13: set3({sampledRoughness, T(0.05f), T(0.05f)}); break;
        case 14: set3({sampledMetallic, T(0.05f), T(0.05f)}); break;
        case 15: set3({T(1) - alpha, T(0.05f), T(0.05f)}); break;
        default: break;
    }
    if (sd.light_enabled > 0) {
        T shadowFactor = T(1);
        if (sd.shadows_enabled == 1)
        {
            // the finest cascade whose coordinates keep the PCF footprint inside the map
            const int S = (int)c.s->shadow_size;
            const int n = cascades_of(c.s);
            T cc[4] = {bv.csm[0], bv.csm[1], bv.csm[2], bv.csm[3]};
            int k = 0;
            if (n > 1) {
                const T m = (T)(2.0f / (float)S);
                const T hi = T(1) - m;
                for (k = 0; k < n; ++k) {
                    T x = bv.csm[0], y = bv.csm[1];
                    if (k > 0) {
                        const T sc = (T)std::ldexp(1.0f, -k);
                        x = (bv.csm[0] - T(0.5)) * sc + T(0.5);
                        y = (bv.csm[1] - T(0.5)) * sc + T(0.5);
                    }
                    if ((x >= m && x <= hi && y >= m && y <= hi) || k == n - 1) {
                        cc[0] = x;
                        cc[1] = y;
                        break;
                    }
                }
            }
            shadowFactor = pcf<T>(shadow + (size_t)k * S * S, S, cc, c.s->draw_config->pcf_mode,
                                  shadow_marks);
        }
        if (sd.brdf_lighting_enabled == 0) {
            const T ml = fmaxT<T>(cosTheta, T(0));
            const V3<T> sunLight{(T)sd.sunlight_color[0] * ml, (T)sd.sunlight_color[1] * ml, (T)sd.sunlight_color[2] * ml};
            outFragColor[0] = outFragColor[0] * fmaxT<T>(ambientLight.x, sunLight.x * shadowFactor);
            outFragColor[1] = outFragColor[1] * fmaxT<T>(ambientLight.y, sunLight.y * shadowFactor);
            outFragColor[2] = outFragColor[2] * fmaxT<T>(ambientLight.z, sunLight.z * shadowFactor);
            outFragColor[3] = outFragColor[3] * alpha;
        } else {
            roughness = sampledRoughness;
            metallic = sampledMetallic;
            const T f04 = T(0.04f);
            // lerp(f0, color, metallic) = f0*(1-m) + color*m
            const V3<T> f0{f04 * (T(1) - metallic) + outFragColor[0] * metallic,
                           f04 * (T(1) - metallic) + outFragColor[1] * metallic,
                           f04 * (T(1) - metallic) + outFragColor[2] * metallic};
            const T ndf = distribution_ggx(N, H, roughness);
            const T g = geometry_smith(N, V, L, roughness);
            const V3<T> f = schlick_fresnel(fmaxT<T>(dot(H, V), T(0)), f0);
            const V3<T> kS = f;
            V3<T> kD{T(1) - kS.x, T(1) - kS.y, T(1) - kS.z};
            kD = kD * (T(1) - metallic);
            const V3<T> numerator = f * (ndf * g);
            const T denominator = T(4) * nDotV * lDotN + T(0.0001f);
            const V3<T> specular{numerator.x / denominator, numerator.y / denominator, numerator.z / denominator};
            const T pi = T(3.14159265f);
            const V3<T> diffuse{outFragColor[0] / pi, outFragColor[1] / pi, outFragColor[2] / pi};
            const T li = (T)sd.light_intensity;
            const V3<T> sunLight{(T)sd.sunlight_color[0] * li, (T)sd.sunlight_color[1] * li, (T)sd.sunlight_color[2] * li};
            V3<T> brdf = mul3(mul3(kD, diffuse) + specular, sunLight) * lDotN;
            brdf = V3<T>{fmaxT<T>(ambientLight.x * diffuse.x, brdf.x * shadowFactor),
                         fmaxT<T>(ambientLight.y * diffuse.y, brdf.y * shadowFactor),
                         fmaxT<T>(ambientLight.z * diffuse.z, brdf.z * shadowFactor)};
            outFragColor[0] = brdf.x;
            outFragColor[1] = brdf.y;
            outFragColor[2] = brdf.z;
            outFragColor[3] = alpha;
        }
    }
    if (hasMaterial) {
        if (md->alpha_mode == 1 && alpha < (T)md->alpha_cutoff) return false;
        outFragColor[3] = alpha;
    }
    for (int k = 0; k < 4; ++k) out[k] = outFragColor[k];
    return true;
}

// float -> IEEE binary16 (round to nearest even) -> float: the RGBA16F draw image.
float to_half_and_back(float f) {
    const uint32_t x = fbits(f);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const uint32_t ax = x & 0x7fffffffu;
    uint16_t h;
    if (ax >= 0x7f800000u) {
        h = (uint16_t)(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
    } else if (ax >= 0x477ff000u) {  // rounds to >= 65520 -> inf
        h = (uint16_t)(sign | 0x7c00u);
    } else if (ax < 0x38800000u) {  // below the smallest normal half (2^-14): subnormal or zero
        if (ax < 0x33000000u) {      // < 2^-25: rounds to zero (2^-25 ties to even 0)
            h = (uint16_t)sign;
        } else {
            const uint32_t e = ax >> 23;
            const uint32_t m = (ax & 0x7fffffu) | 0x800000u;
            const uint32_t shift = 126u - e;  // value = m * 2^(e-150); half subnormal unit 2^-24
            // h_m = m * 2^(e-150+24) = m >> (126 - e)
            uint32_t hm = m >> shift;
            const uint32_t rem = m & ((1u << shift) - 1u);
            const uint32_t halfway = 1u << (shift - 1u);
            if (rem > halfway || (rem == halfway && (hm & 1u))) ++hm;
            h = (uint16_t)(sign | hm);
        }
    } else {
        uint32_t e = (ax >> 23) - 112u;  // rebias 127 -> 15
        uint32_t m = ax & 0x7fffffu;
        uint32_t hm = m >> 13;
        const uint32_t rem = m & 0x1fffu;
        uint32_t hv = (e << 10) | hm;
        if (rem > 0x1000u || (rem == 0x1000u && (hv & 1u))) ++hv;
        h = (uint16_t)(sign | hv);
    }
    // back to float
    const uint32_t hs = (uint32_t)(h & 0x8000u) << 16;
    const uint32_t he = (h >> 10) & 0x1fu;
    const uint32_t hm = h & 0x3ffu;
    uint32_t r;
    if (he == 0) {
        if (hm == 0) r = hs;
        else {
            const float v = (float)hm * (1.0f / 16777216.0f);
            r = hs | fbits(v);
        }
    } else if (he == 31) {
        r = hs | 0x7f800000u | (hm << 13);
    } else {
        r = hs | ((he + 112u) << 23) | (hm << 13);
    }
    return bitsf(r);
}

// Vulkan float -> sRGB-encoded 8-bit UNORM (the blit to the B8G8R8A8_SRGB swapchain).
uint8_t encode_srgb8(float c) {
    if (!(c > 0.0f)) c = 0.0f;
    if (c > 1.0f) c = 1.0f;
    const float s = c <= 0.0031308f ? c * 12.92f : 1.055f * std::pow(c, 1.0f / 2.4f) - 0.055f;
    return (uint8_t)std::floor(s * 255.0f + 0.5f);
}
uint8_t encode_unorm8(float c) {
    if (!(c > 0.0f)) c = 0.0f;
    if (c > 1.0f) c = 1.0f;
    return (uint8_t)std::floor(c * 255.0f + 0.5f);
}

// Shade one fragment of triangle t of draw d at pixel (px, py).
template <class T>
bool shade(const Ctx& c, const Draw& d, uint32_t t, int px, int py, const float* shadow, const Sampling<T>& smp,
           std::vector<uint8_t>* shadow_marks, T out[4]) {
    const int W = (int)c.s->width, H = (int)c.s->height;
    uint32_t vi[3];
    VsOut<T> vs[3];
    for (int k = 0; k < 3; ++k) {
        vi[k] = d.vertex_base + c.s->indices[d.first_index + 3 * t + k];
        vertex_main<T>(c, d, vi[k], vs[k]);
        clip_position<T>(c, d, vi[k], vs[k].clip);
    }
    T b[3], bq0[3], bqx[3], bqy[3];
    barycentrics<T>(vs[0].clip, vs[1].clip, vs[2].clip, px, py, W, H, b);
    const int qx = px & ~1, qy = py & ~1;
    barycentrics<T>(vs[0].clip, vs[1].clip, vs[2].clip, qx, qy, W, H, bq0);
    barycentrics<T>(vs[0].clip, vs[1].clip, vs[2].clip, qx + 1, qy, W, H, bqx);
    barycentrics<T>(vs[0].clip, vs[1].clip, vs[2].clip, qx, qy + 1, W, H, bqy);
    Frag<T> f;
    interpolate(vs, b, f);
    for (int i = 0; i < 2; ++i) {
        const T u0 = vs[0].uv[i] * bq0[0] + vs[1].uv[i] * bq0[1] + vs[2].uv[i] * bq0[2];
        const T ux = vs[0].uv[i] * bqx[0] + vs[1].uv[i] * bqx[1] + vs[2].uv[i] * bqx[2];
        const T uy = vs[0].uv[i] * bqy[0] + vs[1].uv[i] * bqy[1] + vs[2].uv[i] * bqy[2];
        f.duvdx[i] = ux - u0;
        f.duvdy[i] = uy - u0;
    }
    return fragment_main<T>(c, d, f, shadow, smp, shadow_marks, out);
}

const Draw& find_draw(const std::vector<Draw>& list, uint32_t tri) {
    size_t lo = 0, hi = list.size();
    while (hi - lo > 1) {
        const size_t mid = (lo + hi) / 2;
        if (list[mid].tri_base <= tri) lo = mid;
        else hi = mid;
    }
    return list[lo];
}

template <class T>
void shading_pass(const Ctx& c, const float* shadow, const float* depth, const uint32_t* ids, float* color16,
                  double* out64, int threads, TexMarks* marks, std::vector<uint8_t>* shadow_marks) {
    const int W = (int)c.s->width, H = (int)c.s->height;
    const int n = samples_of(c.s);
    const size_t plane = (size_t)W * H;
    const float clear[4] = {0.0f, 0.05f, 0.1f, 1.0f};  // src/Engine/Graphics.cpp:5416-5419
    Sampling<T> smp{&c, marks};
    // Opaque list. With multisampling each distinct triangle of a pixel's samples
    // is shaded once at the pixel centre and its colour goes to the samples it covers.
    parallel_rows(H, threads, [&](int r0, int r1) {
        for (int py = r0; py < r1; ++py) {
            for (int px = 0; px < W; ++px) {
                const size_t p = (size_t)py * W + px;
                T cs[4][4];
                for (int k = 0; k < n; ++k) {
                    const uint32_t id = ids[k * plane + p];
                    int same = -1;
                    for (int j = 0; j < k && same < 0; ++j)
                        if (ids[j * plane + p] == id) same = j;
                    if (same >= 0) {
                        for (int i = 0; i < 4; ++i) cs[k][i] = cs[same][i];
                        continue;
                    }
                    T col[4] = {(T)clear[0], (T)clear[1], (T)clear[2], (T)clear[3]};
                    if (id != 0) {
                        const uint32_t tri = id - 1;
                        const Draw& d = find_draw(c.opaque, tri);
                        T o[4];
                        if (shade<T>(c, d, tri - d.tri_base, px, py, shadow, smp, shadow_marks, o))
                            for (int i = 0; i < 4; ++i) col[i] = o[i];
                    }
                    for (int i = 0; i < 4; ++i) cs[k][i] = col[i];
                }
                for (int k = 0; k < n; ++k)
                    for (int i = 0; i < 4; ++i) {
                        if constexpr (sizeof(T) == 4) color16[4 * (k * plane + p) + i] = to_half_and_back((float)cs[k][i]);
                        else out64[4 * (k * plane + p) + i] = (double)cs[k][i];
                    }
            }
        }
    });
    // Blended list, in submission order: blend on, depth write off, cull none (5654-5691),
    // per coverage sample against that sample's opaque depth.
    if (c.blended.empty()) return;
    std::vector<float> mvps(c.blended.size() * 16);
    for (size_t i = 0; i < c.blended.size(); ++i) draw_mvp(c, c.blended[i], c.s->scene->view_projection, &mvps[16 * i]);
    for (int k = 0; k < n; ++k) {
        const float* dk = depth + k * plane;
        parallel_rows(H, threads, [&](int r0, int r1) {
            RasterState rs;
            rs.width = W;
            rs.height = H;
            rs.row_begin = r0;
            rs.row_end = r1;
            rs.ox = n > 1 ? kSampleX[k] : 128;
            rs.oy = n > 1 ? kSampleY[k] : 128;
            rs.cull_front = false;
            rs.ccw_front = c.s->draw_config->reverse_winding_order_enabled != 0;
            for (size_t di = 0; di < c.blended.size(); ++di) {
                const Draw& d = c.blended[di];
                for (uint32_t t = 0; t < d.index_count / 3; ++t) {
                    CV cv[3];
                    uint32_t vi[3];
                    tri_clip(c, d, &mvps[16 * di], t, cv, vi);
                    raster_primitive(cv, rs, [&](int px, int py, float z) {
                        const size_t p = (size_t)py * W + px;
                        if (!(z >= dk[p])) return;
                        T s[4];
                        if (!shade<T>(c, d, t, px, py, shadow, smp, shadow_marks, s)) return;
                        // SRC_ALPHA / ONE_MINUS_SRC_ALPHA on colour, ONE / ZERO on alpha
                        const T a = s[3];
                        const size_t q = 4 * (k * plane + p);
                        if constexpr (sizeof(T) == 4) {
                            for (int i = 0; i < 3; ++i) {
                                const float dst = color16[q + i];
                                color16[q + i] = to_half_and_back((float)(s[i] * a + (T)dst * (T(1) - a)));
                            }
                            color16[q + 3] = to_half_and_back((float)a);
                        } else {
                            for (int i = 0; i < 3; ++i) out64[q + i] = s[i] * a + out64[q + i] * (T(1) - a);
                            out64[q + 3] = a;
                        }
                    });
                }
            }
        });
    }
}

// ----------------------------------------------------------------------------
// Debug-line overlay: DRAW DEBUG of src/Engine/Graphics.cpp:5694-5738 with the
// vertex stage of src/shaders/debug.slang:5-35 and the vertex table of
// Graphics.cpp:3222-3249. Contract shared with k_debug_prep / k_blend:
//  * vertex: flags == 4 -> view_projection * point (the transform's columns 0
//    and 1); flags == 1 -> transform * (x, y*aspect, z, w), z = w = 1;
//    flags == 2 -> (proj * transform) * v, z = w = 1; else
//    (view_projection * transform) * v; M * v is the chain M0r*x -> fma(M1r, y)
//    -> fma(M2r, z) -> fma(M3r, w);
//  * clipping against the triangle planes in order; when exactly one end is
//    outside, the point fma(t, b-a, a) with t = da/(da-db) replaces it;
//  * viewport and 8-bit sub-pixel snap as for triangles;
//  * coverage of a sample: 0 <= along < |d|^2 and -(w/2)|d| < perp <= (w/2)|d|
//    (exact integers; the rectangle of Vulkan's strict lines, width 5);
//  * depth fma(along/|d|^2, z1 - z0, z0) clamped to [0,1], tested
//    GREATER_OR_EQUAL against the opaque depth, never written;
//  * the sample takes the line's colour (alpha 1: SRC_ALPHA blending keeps
//    only the source), rounded to RGBA16F.
// ----------------------------------------------------------------------------

constexpr int64_t kDebugHalfWidth2 = 640 * 640;  // (2.5 px in 1/256 px)^2

struct DebugPair {
    float a[4], b[4];
    uint32_t object;
};

std::vector<DebugPair> debug_pairs(const rz_debug_object* objs, uint32_t n) {
    // unit circle of the vertex table: 101 vertex pairs from angle step, step 4*pi/100
    const float target = (float)3.141592653589793 * 4.0f;
    const float step = target / 100.0f;
    std::vector<DebugPair> out;
    for (uint32_t o = 0; o < n; ++o) {
        const rz_debug_object& d = objs[o];
        if (d.flags == RZ_DEBUG_TRANSFORM_IS_POINTS) {
            DebugPair p{};
            for (int k = 0; k < 4; ++k) {
                p.a[k] = d.transform[k];
                p.b[k] = d.transform[4 + k];
            }
            p.object = o;
            out.push_back(p);
        } else if (d.type == RZ_DEBUG_CIRCLE) {
            for (int i = 0; i < 50; ++i) {
                const float cur = step * (float)(i + 1), next = cur + step;
                out.push_back(DebugPair{{std::sin(cur), std::cos(cur), 0.0f, 1.0f},
                                        {std::sin(next), std::cos(next), 0.0f, 1.0f}, o});
            }
        } else {
            out.push_back(DebugPair{{0.0f, 0.0f, 0.0f, 1.0f}, {0.0f, 0.0f, 1.0f, 1.0f}, o});
        }
    }
    return out;
}

CV transform4(const float* M, const float* p) {
    CV o;
    for (int r = 0; r < 4; ++r) {
        float acc = M[0 * 4 + r] * p[0];
        acc = std::fmaf(M[1 * 4 + r], p[1], acc);
        acc = std::fmaf(M[2 * 4 + r], p[2], acc);
        acc = std::fmaf(M[3 * 4 + r], p[3], acc);
        o.v[r] = acc;
    }
    return o;
}

CV debug_vertex(const rz_scene_data& sd, const rz_debug_object& d, const float* v) {
    float M[16];
    CV c;
    if (d.flags == RZ_DEBUG_TRANSFORM_IS_POINTS) return transform4(sd.view_projection, v);
    if (d.flags == RZ_DEBUG_SCREEN_SPACE) {
        const float aspect = sd.draw_extent[0] / sd.draw_extent[1];
        const float q[4] = {v[0], v[1] * aspect, v[2], v[3]};
        c = transform4(d.transform, q);
        c.v[2] = c.v[3] = 1.0f;
        return c;
    }
    if (d.flags == RZ_DEBUG_VIEW_SPACE) {
        mat4_mul(sd.proj, d.transform, M);
        c = transform4(M, v);
        c.v[2] = c.v[3] = 1.0f;
        return c;
    }
    mat4_mul(sd.view_projection, d.transform, M);
    return transform4(M, v);
}

struct DebugSeg {
    bool live = false;
    SV a{}, b{};
};

DebugSeg debug_segment(const rz_scene_data& sd, const rz_debug_object& d, const DebugPair& pr, int W, int H) {
    CV a = debug_vertex(sd, d, pr.a), b = debug_vertex(sd, d, pr.b);
    DebugSeg s;
    for (int p = 0; p < 6; ++p) {
        const float da = plane_dist(a, p), db = plane_dist(b, p);
        const bool ia = da >= 0.0f, ib = db >= 0.0f;
        if (!ia && !ib) return s;
        if (ia != ib) {
            const float t = da / (da - db);
            CV c;
            for (int k = 0; k < 4; ++k) c.v[k] = std::fmaf(t, b.v[k] - a.v[k], a.v[k]);
            if (ia) b = c;
            else a = c;
        }
    }
    if (!(a.v[3] > 0.0f) || !(b.v[3] > 0.0f)) return s;
    const float hw = (float)W * 0.5f, hh = (float)H * 0.5f;
    s.a = to_screen(a, hw, hh);
    s.b = to_screen(b, hw, hh);
    s.live = true;
    return s;
}

bool debug_covers(const DebugSeg& s, int32_t PX, int32_t PY, float& z) {
    const int64_t dx = (int64_t)s.b.X - s.a.X, dy = (int64_t)s.b.Y - s.a.Y;
    const int64_t len2 = dx * dx + dy * dy;
    if (len2 == 0) return false;
    const int64_t ex = (int64_t)PX - s.a.X, ey = (int64_t)PY - s.a.Y;
    const int64_t along = ex * dx + ey * dy;
    if (along < 0 || along >= len2) return false;
    const int64_t perp = dx * ey - dy * ex;
    const __int128 lhs = (__int128)perp * perp, rhs = (__int128)kDebugHalfWidth2 * len2;
    if (perp >= 0 ? lhs > rhs : lhs >= rhs) return false;
    const float t = (float)along / (float)len2;
    float zz = std::fmaf(t, s.b.z - s.a.z, s.a.z);
    if (!(zz > 0.0f)) zz = 0.0f;
    if (zz > 1.0f) zz = 1.0f;
    z = zz;
    return true;
}

// Draws the overlay over the per-sample draw image (color16 with T = float,
// FP64 values in out64 with T = double); depth holds each sample's opaque depth.
template <class T>
void debug_overlay(const Ctx& c, const float* depth, float* color16, double* out64, int threads) {
    const oracle_scene* sc = c.s;
    if (!sc->debug_objects || sc->debug_object_count == 0) return;
    const int W = (int)sc->width, H = (int)sc->height, n = samples_of(sc);
    const size_t plane = (size_t)W * H;
    const std::vector<DebugPair> pairs = debug_pairs(sc->debug_objects, sc->debug_object_count);
    std::vector<DebugSeg> segs(pairs.size());
    for (size_t i = 0; i < pairs.size(); ++i)
        segs[i] = debug_segment(*sc->scene, sc->debug_objects[pairs[i].object], pairs[i], W, H);
    parallel_rows(H, threads, [&](int r0, int r1) {
        for (size_t i = 0; i < segs.size(); ++i) {
            const DebugSeg& s = segs[i];
            if (!s.live) continue;
            const float* col = sc->debug_objects[pairs[i].object].color;
            const int x0 = std::max(0, (std::min(s.a.X, s.b.X) - 640) >> 8);
            const int x1 = std::min(W - 1, (std::max(s.a.X, s.b.X) + 640) >> 8);
            const int y0 = std::max(r0, (std::min(s.a.Y, s.b.Y) - 640) >> 8);
            const int y1 = std::min(r1 - 1, (std::max(s.a.Y, s.b.Y) + 640) >> 8);
            for (int py = y0; py <= y1; ++py)
                for (int px = x0; px <= x1; ++px)
                    for (int k = 0; k < n; ++k) {
                        const int32_t PX = px * 256 + (n > 1 ? kSampleX[k] : 128);
                        const int32_t PY = py * 256 + (n > 1 ? kSampleY[k] : 128);
                        float z;
                        const size_t q = k * plane + (size_t)py * W + px;
                        if (!debug_covers(s, PX, PY, z) || !(z >= depth[q])) continue;
                        for (int ch = 0; ch < 3; ++ch) {
                            if constexpr (sizeof(T) == 4) color16[4 * q + ch] = to_half_and_back(col[ch]);
                            else out64[4 * q + ch] = (double)col[ch];
                        }
                        if constexpr (sizeof(T) == 4) color16[4 * q + 3] = 1.0f;
                        else out64[4 * q + 3] = 1.0;
                    }
        }
    });
}

int threads_or_default(int threads) {
    if (threads > 0) return threads;
    const unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 1;
}

}  // namespace

extern "C" int oracle_raster(const oracle_scene* s, oracle_out* out, int threads) {
    if (!s || !out) return 3;
    threads = threads_or_default(threads);
    Ctx c;
    build_ctx(s, c);
    std::vector<float> shadow_local, depth_local;
    std::vector<uint32_t> ids_local;
    float* shadow = out->shadow;
    if (!shadow) {
        shadow_local.resize((size_t)cascades_of(s) * s->shadow_size * s->shadow_size);
        shadow = shadow_local.data();
    }
    float* depth = out->depth;
    if (!depth) {
        depth_local.resize((size_t)samples_of(s) * s->width * s->height);
        depth = depth_local.data();
    }
    uint32_t* ids = out->ids;
    if (!ids) {
        ids_local.resize((size_t)samples_of(s) * s->width * s->height);
        ids = ids_local.data();
    }
    shadow_pass(c, shadow, threads);
    camera_pass(c, depth, ids, threads);
    return 0;
}

// ---- sub-pixel sources of the learned path's triangle-aware x2 base -----------
// (the renderer's k_subpixel_sources, restated; the reference has no such pass)

namespace {

struct SubTri {
    float X[3], Y[3], Z[3];  // screen position (pixels) and NDC depth z / w of each vertex
    float inv_area;          // 1 / twice the signed screen area (0 when degenerate)
    bool valid;              // every w > 0
};

SubTri sub_triangle(const Ctx& c, uint32_t id, float hw, float hh) {
    const uint32_t tri = id - 1;
    const Draw& d = find_draw(c.opaque, tri);
    const uint32_t t = tri - d.tri_base;
    SubTri g;
    g.valid = true;
    for (int k = 0; k < 3; ++k) {
        const uint32_t vi = d.vertex_base + c.s->indices[d.first_index + 3 * t + k];
        float cp[4];
        clip_position<float>(c, d, vi, cp);
        g.valid = g.valid && cp[3] > 0.0f;
        const float rw = 1.0f / cp[3];
        g.X[k] = (cp[0] * rw) * hw + hw;
        g.Y[k] = (cp[1] * rw) * hh + hh;
        g.Z[k] = cp[2] * rw;
    }
    const float area = (g.X[1] - g.X[0]) * (g.Y[2] - g.Y[0]) - (g.X[2] - g.X[0]) * (g.Y[1] - g.Y[0]);
    g.inv_area = area != 0.0f ? 1.0f / area : 0.0f;
    return g;
}

uint16_t subpixel_mask(const Ctx& c, const uint32_t* ids, int W, int H, int x, int y, float hw, float hh) {
    uint32_t nb[9];
    int n9 = 0;
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
            const int yy = std::min(std::max(y + dy, 0), H - 1), xx = std::min(std::max(x + dx, 0), W - 1);
            nb[n9++] = ids[(size_t)yy * W + xx];
        }
    const uint32_t own = nb[4];
    bool same = true;
    for (int i = 0; i < 9; ++i) same = same && nb[i] == own;
    if (same) return 0xFFFF;
    uint32_t cand[9];
    int n = 0;
    for (int i = 0; i < 9; ++i) {
        bool seen = nb[i] == 0;
        for (int j = 0; j < n; ++j) seen = seen || cand[j] == nb[i];
        if (!seen) cand[n++] = nb[i];
    }
    uint32_t best[4] = {0, 0, 0, 0};
    float best_z[4] = {-INFINITY, -INFINITY, -INFINITY, -INFINITY};
    for (int ci = 0; ci < n; ++ci) {
        const SubTri g = sub_triangle(c, cand[ci], hw, hh);
        for (int k = 0; k < 4; ++k) {
            const float sx = (float)x + ((k & 1) ? 0.75f : 0.25f), sy = (float)y + ((k >> 1) ? 0.75f : 0.25f);
            bool inside;
            float z;
            if (!g.valid) {  // a vertex behind the eye: only the pixel's own triangle, behind every other
                inside = cand[ci] == own;
                z = -3.0e38f;
            } else {
                const float e0 = (g.X[2] - g.X[1]) * (sy - g.Y[1]) - (g.Y[2] - g.Y[1]) * (sx - g.X[1]);
                const float e1 = (g.X[0] - g.X[2]) * (sy - g.Y[2]) - (g.Y[0] - g.Y[2]) * (sx - g.X[2]);
                const float e2 = (g.X[1] - g.X[0]) * (sy - g.Y[0]) - (g.Y[1] - g.Y[0]) * (sx - g.X[0]);
                inside = g.inv_area != 0.0f &&
                         ((e0 >= 0.0f && e1 >= 0.0f && e2 >= 0.0f) || (e0 <= 0.0f && e1 <= 0.0f && e2 <= 0.0f));
                z = ((e0 * g.Z[0] + e1 * g.Z[1]) + e2 * g.Z[2]) * g.inv_area;
            }
            if (inside && z > best_z[k]) {  // reverse-Z: larger is nearer, as in the depth test
                best[k] = cand[ci];
                best_z[k] = z;
            }
        }
    }
    uint16_t mask = 0;
    for (int k = 0; k < 4; ++k) {
        const int xs = std::min(std::max(x + ((k & 1) ? 1 : -1), 0), W - 1);
        const int ys = std::min(std::max(y + ((k >> 1) ? 1 : -1), 0), H - 1);
        const uint32_t src[4] = {ids[(size_t)y * W + x], ids[(size_t)y * W + xs], ids[(size_t)ys * W + x],
                                 ids[(size_t)ys * W + xs]};
        for (int s = 0; s < 4; ++s)
            if (src[s] == best[k]) mask |= (uint16_t)(1u << (4 * k + s));
    }
    return mask;
}

}  // namespace

extern "C" int oracle_subpixel_sources(const oracle_scene* s, const uint32_t* ids, uint16_t* out, int threads) {
    if (!s || !ids || !out) return 3;
    threads = threads_or_default(threads);
    Ctx c;
    build_ctx(s, c);
    const int W = (int)s->width, H = (int)s->height;
    const float hw = (float)W * 0.5f, hh = (float)H * 0.5f;
    parallel_rows(H, threads, [&](int r0, int r1) {
        for (int y = r0; y < r1; ++y)
            for (int x = 0; x < W; ++x) out[(size_t)y * W + x] = subpixel_mask(c, ids, W, H, x, y, hw, hh);
    });
    return 0;
}

static int render_rgba8(const oracle_scene* s, oracle_out* out, int threads);

// BC7 textures are decoded to RGBA8 level by level first, as the renderer does
// when it uploads them; the frame is then rendered from RGBA8 texels only.
extern "C" int oracle_render(const oracle_scene* s, oracle_out* out, int threads) {
    if (!s || !out) return 3;
    bool any_bc7 = false;
    for (uint32_t i = 0; i < s->texture_count; ++i) any_bc7 = any_bc7 || s->textures[i].format == RZ_TEXELS_BC7;
    if (!any_bc7) return render_rgba8(s, out, threads);
    std::vector<rz_texture> tex(s->textures, s->textures + s->texture_count);
    std::vector<std::vector<uint8_t>> texels(s->texture_count);
    for (uint32_t i = 0; i < s->texture_count; ++i) {
        rz_texture& t = tex[i];
        if (t.format != RZ_TEXELS_BC7) continue;
        size_t n = 0;
        for (uint32_t l = 0; l < t.levels; ++l) n += (size_t)std::max(1u, t.width >> l) * std::max(1u, t.height >> l);
        texels[i].resize(n * 4);
        const uint8_t* blocks = static_cast<const uint8_t*>(t.texels);
        size_t texel_off = 0, block_off = 0;
        for (uint32_t l = 0; l < t.levels; ++l) {
            const uint32_t w = std::max(1u, t.width >> l), h = std::max(1u, t.height >> l);
            oracle_bc7_decode(blocks + block_off, w, h, texels[i].data() + 4 * texel_off);
            texel_off += (size_t)w * h;
            block_off += (size_t)((w + 3) / 4) * ((h + 3) / 4) * 16;
        }
        t.texels = texels[i].data();
        t.format = RZ_TEXELS_RGBA8;
    }
    oracle_scene decoded = *s;
    decoded.textures = tex.data();
    return render_rgba8(&decoded, out, threads);
}

static int render_rgba8(const oracle_scene* s, oracle_out* out, int threads) {
    if (!s || !out) return 3;
    threads = threads_or_default(threads);
    Ctx c;
    build_ctx(s, c);
    const size_t np = (size_t)s->width * s->height;
    const int ns = samples_of(s);
    std::vector<float> shadow((size_t)cascades_of(s) * s->shadow_size * s->shadow_size), depth(np * ns);
    std::vector<uint32_t> ids(np * ns);
    shadow_pass(c, shadow.data(), threads);
    camera_pass(c, depth.data(), ids.data(), threads);
    TexMarks marks;
    std::vector<uint8_t> shadow_marks;
    TexMarks* mp = nullptr;
    std::vector<uint8_t>* smp = nullptr;
    if (out->texel_bytes) {
        marks.levels.resize(s->texture_count);
        for (uint32_t i = 0; i < s->texture_count; ++i) {
            size_t n = 0;
            for (uint32_t l = 0; l < s->textures[i].levels; ++l)
                n += (size_t)std::max(1u, s->textures[i].width >> l) * std::max(1u, s->textures[i].height >> l);
            marks.levels[i].assign(n, 0);
        }
        shadow_marks.assign(shadow.size(), 0);
        mp = &marks;
        smp = &shadow_marks;
    }
    std::vector<float> color16(np * 4 * ns);
    shading_pass<float>(c, shadow.data(), depth.data(), ids.data(), color16.data(), nullptr, threads, mp, smp);
    debug_overlay<float>(c, depth.data(), color16.data(), nullptr, threads);
    // AVERAGE resolve of the samples into the RGBA16F draw image ((s0 + s1) + (s2 + s3)) / 4
    // (src/Engine/Graphics.cpp:5571-5572), then the blit to sRGB 8-bit
    auto resolved = [&](size_t p, int k) -> float {
        if (ns == 1) return color16[4 * p + k];
        const float* q = color16.data() + 4 * p + k;
        return to_half_and_back(((q[0] + q[4 * np]) + (q[8 * np] + q[12 * np])) * 0.25f);
    };
    if (out->color) {
        for (size_t p = 0; p < np; ++p) {
            for (int k = 0; k < 3; ++k) out->color[4 * p + k] = encode_srgb8(resolved(p, k));
            out->color[4 * p + 3] = encode_unorm8(resolved(p, 3));
        }
    }
    if (out->color_f64) {
        std::vector<double> c64(np * 4 * ns);
        shading_pass<double>(c, shadow.data(), depth.data(), ids.data(), nullptr, c64.data(), threads, nullptr, nullptr);
        debug_overlay<double>(c, depth.data(), nullptr, c64.data(), threads);
        for (size_t p = 0; p < np; ++p)
            for (int k = 0; k < 4; ++k) {
                const double* q = c64.data() + 4 * p + k;
                out->color_f64[4 * p + k] = ns == 1 ? q[0] : ((q[0] + q[4 * np]) + (q[8 * np] + q[12 * np])) * 0.25;
            }
        for (size_t p = 0; p < np; ++p) {
            for (int k = 0; k < 4; ++k) {
                double v = out->color_f64[4 * p + k];
                if (!(v > 0.0)) v = 0.0;
                if (v > 1.0) v = 1.0;
                if (k < 3) v = v <= 0.0031308 ? v * 12.92 : 1.055 * std::pow(v, 1.0 / 2.4) - 0.055;
                out->color_f64[4 * p + k] = v;
            }
        }
    }
    if (out->texel_bytes) {
        uint64_t n = 0;
        for (auto& l : marks.levels)
            for (uint8_t m : l) n += m;
        for (uint8_t m : shadow_marks) n += m;
        *out->texel_bytes = 4 * n;
    }
    if (out->depth) std::copy(depth.begin(), depth.end(), out->depth);
    if (out->ids) std::copy(ids.begin(), ids.end(), out->ids);
    if (out->shadow) std::copy(shadow.begin(), shadow.end(), out->shadow);
    return 0;
}
