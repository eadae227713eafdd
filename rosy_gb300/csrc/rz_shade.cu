// Deferred-style shading of the camera pass.
//
// Reference path: vertexMain (src/shaders/basic.slang:16-119) and fragmentMain
// (137-344) with pcf (src/shaders/pcf.slang:1-11) and the BRDF helpers
// (src/shaders/lighting.slang:5-43), evaluated once per pixel for the triangle
// that won the depth test, then the RGBA16F draw image (Graphics.cpp:1905-1908)
// and the blit to the sRGB swapchain (5845-5879).
//
// The vertex stage runs once per (draw, mesh vertex) in k_vertex, pulling the
// 64-byte vertex records as the reference does through buffer device addresses,
// and writes a 128-byte varying record. k_shade then shades each pixel once for
// the triangle that won its depth test: it gathers the three varying records
// and interpolates them with perspective-correct barycentrics computed from the
// clip positions in 2D homogeneous form. Texture level selection uses the
// derivative of the interpolated uv across the pixel's 2x2 quad (the value at
// the quad's top-left, right and lower neighbours, which is what a helper
// invocation would compute).
//
// The file is built with -fmad=false. Everything that feeds a discrete
// decision - barycentrics, the interpolated uv and its quad derivatives, level
// selection, texel addresses and filter weights, the shadow-map coordinate and
// depth compared in PCF - follows the oracle's fp32 operation order and is
// bit-identical to it (log2f of the trilinear fraction aside). The lighting
// arithmetic downstream is continuous and uses reciprocal square roots and
// approximate division; its output stays within the 1/255 bound.
#include <cuda_fp16.h>

#include <algorithm>

#include "rz_device.cuh"

namespace rz {

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 mul3(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
__device__ __forceinline__ V3 normalize(V3 a) {
    const float l = sqrtf(dot(a, a));
    return {a.x / l, a.y / l, a.z / l};
}
__device__ __forceinline__ float clamp01(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }
// Lighting-only forms (continuous quantities graded within 1/255): reciprocal
// square root and approximate division instead of IEEE sqrt/div.
__device__ __forceinline__ V3 fnormalize(V3 a) {
    const float r = rsqrtf(dot(a, a));
    return {a.x * r, a.y * r, a.z * r};
}
__device__ __forceinline__ float fdiv(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ V3 mulm3v(const float* N, V3 v) {
    return {N[0] * v.x + N[3] * v.y + N[6] * v.z, N[1] * v.x + N[4] * v.y + N[7] * v.z, N[2] * v.x + N[5] * v.y + N[8] * v.z};
}

// ---------------------------------------------------------------------------
// per-draw constants
// ---------------------------------------------------------------------------

// Also zeroes the clear list L (the camera pass's headers and look-back words),
// so that the two need one launch.
__global__ void k_prep_camera(const DrawRec* __restrict__ draws, uint32_t n, const rz_object* __restrict__ objects,
                              const ViewRec* __restrict__ views, DrawConsts* __restrict__ out, ClearList L) {
    const uint32_t d = blockIdx.x * blockDim.x + threadIdx.x;
    clear_share(L);
    if (d >= n) return;
    const rz_scene_data* sd = views[draws[d].view].scene;
    const rz_object& gd = objects[draws[d].object];
    float W[16], VP[16], C[16];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        W[i] = gd.transform[i];
        VP[i] = sd->view_projection[i];
    }
    mat4_mul(VP, W, C);
    DrawConsts& o = out[d];
#pragma unroll
    for (int i = 0; i < 16; ++i) o.mvp[i] = C[i];
    // (ndc_to_tc * shadowProjNear) * W, ndc_to_tc rows (0.5,0,0,0.5) (0,0.5,0,0.5) (0,0,1,0) (0,0,0,1)
    float A[16];
    const float* P = sd->shadow_projection_near;
#pragma unroll
    for (int col = 0; col < 4; ++col) {
        const float x = P[col * 4 + 0], y = P[col * 4 + 1], z = P[col * 4 + 2], w = P[col * 4 + 3];
        A[col * 4 + 0] = 0.5f * x + 0.5f * w;
        A[col * 4 + 1] = 0.5f * y + 0.5f * w;
        A[col * 4 + 2] = z;
        A[col * 4 + 3] = w;
    }
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int r = 0; r < 4; ++r)
            o.csm[c * 4 + r] = A[0 * 4 + r] * W[c * 4 + 0] + A[1 * 4 + r] * W[c * 4 + 1] + A[2 * 4 + r] * W[c * 4 + 2] +
                               A[3 * 4 + r] * W[c * 4 + 3];
    const float* T = gd.to_object_space_transform;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        o.cam_obj[r] = T[0 * 4 + r] * sd->camera_position[0] + T[1 * 4 + r] * sd->camera_position[1] +
                       T[2 * 4 + r] * sd->camera_position[2] + T[3 * 4 + r] * sd->camera_position[3];
        o.sun_obj[r] = T[0 * 4 + r] * sd->sun_position[0] + T[1 * 4 + r] * sd->sun_position[1] +
                       T[2 * 4 + r] * sd->sun_position[2] + T[3 * 4 + r] * sd->sun_position[3];
    }
}

void launch_prep_camera(const DrawRec* draws, uint32_t n, const rz_object* objects, const ViewRec* views,
                        DrawConsts* out, cudaStream_t stream, const ClearList* clear, int sm_count) {
    const ClearList none{};
    const ClearList& L = clear ? *clear : none;
    const unsigned blocks = std::max((n + 127) / 128, clear_blocks(L, sm_count, 128));
    if (blocks == 0) return;
    k_prep_camera<<<blocks, 128, 0, stream>>>(draws, n, objects, views, out, L);
    note_launch();
}

// ---------------------------------------------------------------------------
// vertex stage
// ---------------------------------------------------------------------------

struct VsOut {
    V3 normal, worldNormal, viewDir, lightDir, tangent, bitangent;
    float color[4];
    float uv[2];
    float sigma;
    float csm[4];
};

// vertexMain, src/shaders/basic.slang:16-119 (outputs used by fragmentMain).
__device__ __forceinline__ void vertex_main(const rz_scene_data& sd, const rz_object& gd, const DrawConsts& dc,
                                            bool has_material, bool material_has_normal_map, const rz_vertex& v, VsOut& o) {
    float nt[4] = {v.tangent[0], v.tangent[1], v.tangent[2], v.tangent[3]};
    if (sd.ignore_asset_tangent_sign == 1) nt[3] = 1.0f;
    if (sd.flip_tangents[0] == 1) nt[0] = nt[0] * -1.0f;
    if (sd.flip_tangents[1] == 1) nt[1] = nt[1] * -1.0f;
    if (sd.flip_tangents[2] == 1) nt[2] = nt[2] * -1.0f;
    if (sd.flip_tangents[3] == 1) nt[3] = nt[3] * -1.0f;
    bool tse = sd.tangent_space_enabled == 1;
    if (has_material && !material_has_normal_map) tse = false;
    const V3 vpos{v.position[0], v.position[1], v.position[2]};
    V3 normal{v.normal[0], v.normal[1], v.normal[2]};
    V3 tangent{nt[0], nt[1], nt[2]};
    V3 bitangent = cross(normal, tangent) * nt[3];
    if (sd.ensure_orthogonal_bitangent == 1) {
        const V3 normal_projection = bitangent * dot(normal, bitangent);
        const V3 ortho_n = normalize(normal - normal_projection);
        const V3 tangent_projection = normal_projection - bitangent * dot(tangent, bitangent);
        const V3 ortho_t = normalize(tangent - tangent_projection);
        bitangent = cross(ortho_n, ortho_t) * nt[3];
    }
    V3 viewDir, lightDir;
    if (tse) {
        viewDir = V3{dc.cam_obj[0], dc.cam_obj[1], dc.cam_obj[2]} - vpos;
        lightDir = V3{dc.sun_obj[0], dc.sun_obj[1], dc.sun_obj[2]} - vpos;
    } else {
        const float* M = gd.transform;
        float wp[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) wp[r] = M[0 * 4 + r] * vpos.x + M[1 * 4 + r] * vpos.y + M[2 * 4 + r] * vpos.z + M[3 * 4 + r] * 1.0f;
        viewDir = V3{sd.camera_position[0] - wp[0], sd.camera_position[1] - wp[1], sd.camera_position[2] - wp[2]};
        lightDir = V3{sd.sun_position[0] - wp[0], sd.sun_position[1] - wp[1], sd.sun_position[2] - wp[2]};
        normal = normalize(mulm3v(gd.normal_transform, V3{v.normal[0], v.normal[1], v.normal[2]}));
        tangent = normalize(mulm3v(gd.normal_transform, V3{nt[0], nt[1], nt[2]}));
        tangent = normalize(tangent - normal * dot(normal, tangent));
    }
    if (sd.flip_lights[0] == 1) lightDir.x = lightDir.x * -1.0f;
    if (sd.flip_lights[1] == 1) lightDir.y = lightDir.y * -1.0f;
    if (sd.flip_lights[2] == 1) lightDir.z = lightDir.z * -1.0f;
    o.normal = normal;
    o.worldNormal = mulm3v(gd.normal_transform, V3{v.normal[0], v.normal[1], v.normal[2]});
#pragma unroll
    for (int k = 0; k < 4; ++k) o.color[k] = v.color[k];
    o.tangent = V3{nt[0], nt[1], nt[2]};
    o.bitangent = bitangent;
    o.viewDir = viewDir;
    o.lightDir = lightDir;
    o.sigma = nt[3];
    o.uv[0] = v.uv[0];
    o.uv[1] = v.uv[1];
    const float* B = dc.csm;
#pragma unroll
    for (int r = 0; r < 4; ++r)
        o.csm[r] = B[0 * 4 + r] * vpos.x + B[1 * 4 + r] * vpos.y + B[2 * 4 + r] * vpos.z + B[3 * 4 + r];
}

// Perspective-correct barycentrics at pixel centre (px, py), 2D homogeneous form.
// Normalised device coordinate of pixel centre i of an extent of n pixels.
__device__ __forceinline__ float ndc(int i, int n) { return (float)(2 * i + 1 - n) / (float)n; }

// The normalised coordinates a pixel's barycentrics use: its centre (xp, yp) and
// its quad's (xq, yq), (xq1 = column + 1, yq1 = row + 1).
struct PixelNdc {
    float xp, yp, xq, yq, xq1, yq1;
};

__device__ __forceinline__ void barycentrics_n(const float4& c0, const float4& c1, const float4& c2, float xn, float yn,
                                               float b[3]) {
    const V3 v0{c0.x, c0.y, c0.w}, v1{c1.x, c1.y, c1.w}, v2{c2.x, c2.y, c2.w};
    const V3 p{xn, yn, 1.0f};
    const float b0 = dot(cross(v1, v2), p), b1 = dot(cross(v2, v0), p), b2 = dot(cross(v0, v1), p);
    const float inv = 1.0f / (b0 + b1 + b2);
    b[0] = b0 * inv;
    b[1] = b1 * inv;
    b[2] = b2 * inv;
}

__device__ __forceinline__ void barycentrics(const float4& c0, const float4& c1, const float4& c2, int px, int py, int W,
                                             int H, float b[3]) {
    barycentrics_n(c0, c1, c2, ndc(px, W), ndc(py, H), b);
}

struct Frag {
    V3 normal, worldNormal, viewDir, lightDir, tangent, bitangent;
    float color[4];
    float uv[2];
    float sigma;
    float csm[4];
    float duvdx[2], duvdy[2];
};

// ---------------------------------------------------------------------------
// textures
// ---------------------------------------------------------------------------

__device__ __forceinline__ int wrap_coord(int i, int size, int mode) {
    if (mode == 0) return min(max(i, 0), size - 1);
    if (mode == 2 && (size & (size - 1)) == 0) return i & (size - 1);  // == i mod size for powers of two
    if (mode == 2) {
        int m = i % size;
        return m < 0 ? m + size : m;
    }
    int t = i % (2 * size);
    if (t < 0) t += 2 * size;
    int a = t - size;
    a = a >= 0 ? a : -(1 + a);
    return size - 1 - a;
}

// Where a texture.Sample call reads: the level(s), the wrapped texel columns
// and rows and the filter weights. It depends only on the texture's size and
// level count, the sampler and the uv/derivatives, so textures that share those
// share one SampleCoords (the three material textures usually do).
struct LevelCoords {
    uint32_t off;   // texel offset of the level
    int w;          // level width (row pitch)
    int x0, x1, y0, y1;
    float a, b;     // bilinear weights (unused for nearest)
};

struct SampleCoords {
    uint32_t width, height, levels;
    SamplerBits st;
    bool valid;
    bool linear;    // filter within the level(s)
    bool two;       // blend two levels
    float delta;
    LevelCoords l0, l1;
};

__device__ __forceinline__ void level_coords(const TexDesc& t, int level, bool linear, SamplerBits st, float u, float v,
                                             LevelCoords& c) {
    const int w = max(1, (int)(t.width >> level)), h = max(1, (int)(t.height >> level));
    c.off = t.level_off[level];
    c.w = w;
    const int wu = (st >> 4) & 3, wv = (st >> 6) & 3;
    if (!linear) {
        const int i = (int)floorf(u * (float)w), j = (int)floorf(v * (float)h);
        c.x0 = wrap_coord(i, w, wu);
        c.y0 = wrap_coord(j, h, wv);
        c.x1 = c.x0;
        c.y1 = c.y0;
        c.a = c.b = 0.0f;
        return;
    }
    const float uu = u * (float)w - 0.5f, vv = v * (float)h - 0.5f;
    const float fi = floorf(uu), fj = floorf(vv);
    c.a = uu - fi;
    c.b = vv - fj;
    const int i0 = (int)fi, j0 = (int)fj;
    c.x0 = wrap_coord(i0, w, wu);
    c.x1 = wrap_coord(i0 + 1, w, wu);
    c.y0 = wrap_coord(j0, h, wv);
    c.y1 = wrap_coord(j0 + 1, h, wv);
}

// Level selection of texture.Sample with implicit derivatives (Vulkan LOD rules).
__device__ __forceinline__ void sample_coords(const TexDesc& t, SamplerBits st, const float uv[2], const float duvdx[2],
                                              const float duvdy[2], SampleCoords& c) {
    c.width = t.width;
    c.height = t.height;
    c.levels = t.levels;
    c.st = st;
    c.valid = true;
    const float w0 = (float)t.width, h0 = (float)t.height;
    const float ax = duvdx[0] * w0, ay = duvdx[1] * h0, bx = duvdy[0] * w0, by = duvdy[1] * h0;
    const float rx2 = ax * ax + ay * ay, ry2 = bx * bx + by * by;
    const float rho2 = fmaxf(rx2, ry2);
    const int q = (int)t.levels - 1;
    c.two = false;
    c.delta = 0.0f;
    if (!(rho2 > 1.0f)) {  // magnification: level 0
        c.linear = (st & 2u) != 0;
        level_coords(t, 0, c.linear, st, uv[0], uv[1], c.l0);
        return;
    }
    c.linear = (st & 1u) != 0;
    if (!(st & 4u)) {  // nearest mip: d = ceil(lambda + 0.5) - 1
        int d = 0;
        float thr = 2.0f;
        while (d < q && rho2 > thr) {
            ++d;
            thr = thr * 4.0f;
        }
        level_coords(t, d, c.linear, st, uv[0], uv[1], c.l0);
        return;
    }
    const float lambda = 0.5f * log2f(rho2);
    const float dp = fminf(lambda, (float)q);
    const int dlo = (int)floorf(dp);
    const int dhi = min(dlo + 1, q);
    const float delta = dp - (float)dlo;
    level_coords(t, dlo, c.linear, st, uv[0], uv[1], c.l0);
    if (delta > 0.0f && dhi != dlo) {
        c.two = true;
        c.delta = delta;
        level_coords(t, dhi, c.linear, st, uv[0], uv[1], c.l1);
    }
}

// byte / 255 rounded to nearest: the product with the rounded reciprocal and one
// residual step, exact for every byte (it equals the IEEE quotient, as a table
// of (float)b / 255.0f would, without the shared-memory lookup and its bank
// conflicts).
__device__ __forceinline__ float unorm8(uint32_t b) {
    const float x = (float)b, r = 1.0f / 255.0f;
    const float q = x * r;
    return fmaf(fmaf(-q, 255.0f, x), r, q);
}

struct Sampler {
    const ShadeParams* P;
    const float* srgb;   // shared-memory table: sRGB byte -> linear

    __device__ __forceinline__ void texel(const TexDesc& t, uint32_t off, int w, int i, int j, float out[4]) const {
        const uint32_t v = __ldg(reinterpret_cast<const uint32_t*>(t.base) + off + (uint32_t)j * (uint32_t)w + (uint32_t)i);
        const uint32_t r = v & 0xffu, g = (v >> 8) & 0xffu, b = (v >> 16) & 0xffu, a = v >> 24;
        if (t.srgb) {
            out[0] = srgb[r];
            out[1] = srgb[g];
            out[2] = srgb[b];
        } else {
            out[0] = unorm8(r);
            out[1] = unorm8(g);
            out[2] = unorm8(b);
        }
        out[3] = unorm8(a);
    }

    __device__ __forceinline__ void fetch_level(const TexDesc& t, const LevelCoords& c, bool linear, float out[4]) const {
        if (!linear) {
            texel(t, c.off, c.w, c.x0, c.y0, out);
            return;
        }
        float t00[4], t10[4], t01[4], t11[4];
        texel(t, c.off, c.w, c.x0, c.y0, t00);
        texel(t, c.off, c.w, c.x1, c.y0, t10);
        texel(t, c.off, c.w, c.x0, c.y1, t01);
        texel(t, c.off, c.w, c.x1, c.y1, t11);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float top = t00[k] + c.a * (t10[k] - t00[k]);
            const float bot = t01[k] + c.a * (t11[k] - t01[k]);
            out[k] = top + c.b * (bot - top);
        }
    }

    // texture.Sample(sampler, uv) with implicit derivatives. `cache` holds the
    // coordinates of the previous call and is reused when the texture's size,
    // levels and sampler match.
    __device__ void sample(uint32_t tex_index, uint32_t sampler_index, const Frag& f, SampleCoords& cache, float out[4]) const {
        if (tex_index >= P->texture_count) {  // absent image: robust null descriptor reads 0
            out[0] = out[1] = out[2] = out[3] = 0.0f;
            return;
        }
        const TexDesc& t = P->textures[tex_index];
        const SamplerBits st = P->samplers[min(sampler_index, P->sampler_count)];
        if (!(cache.valid && cache.width == t.width && cache.height == t.height && cache.levels == t.levels &&
              cache.st == st))
            sample_coords(t, st, f.uv, f.duvdx, f.duvdy, cache);
        fetch_level(t, cache.l0, cache.linear, out);
        if (cache.two) {
            float b[4];
            fetch_level(t, cache.l1, cache.linear, b);
#pragma unroll
            for (int k = 0; k < 4; ++k) out[k] = out[k] + cache.delta * (b[k] - out[k]);
        }
    }
};

// SampleCmpLevelZero, linear, clamp-to-edge, GREATER_OR_EQUAL (Graphics.cpp:2697-2725).
__device__ __forceinline__ float sample_cmp(const float* __restrict__ shadow, int S, float u, float v, float dref) {
    const float uu = u * (float)S - 0.5f, vv = v * (float)S - 0.5f;
    const float fi = floorf(uu), fj = floorf(vv);
    const float a = uu - fi, b = vv - fj;
    const int i0 = (int)fmaxf(fminf(fi, (float)(S + 1)), -2.0f), j0 = (int)fmaxf(fminf(fj, (float)(S + 1)), -2.0f);
    const int x0 = min(max(i0, 0), S - 1), x1 = min(max(i0 + 1, 0), S - 1);
    const int y0 = min(max(j0, 0), S - 1), y1 = min(max(j0 + 1, 0), S - 1);
    const float c00 = dref >= __ldg(&shadow[(size_t)y0 * S + x0]) ? 1.0f : 0.0f;
    const float c10 = dref >= __ldg(&shadow[(size_t)y0 * S + x1]) ? 1.0f : 0.0f;
    const float c01 = dref >= __ldg(&shadow[(size_t)y1 * S + x0]) ? 1.0f : 0.0f;
    const float c11 = dref >= __ldg(&shadow[(size_t)y1 * S + x1]) ? 1.0f : 0.0f;
    const float top = c00 + a * (c10 - c00);
    const float bot = c01 + a * (c11 - c01);
    return top + b * (bot - top);
}

// 3x3 PCF: nine bilinear compare taps one texel apart. The taps' texel
// positions are computed one by one (as the single-tap path would), and when
// they fall on consecutive columns/rows - the usual case - the 16 compares of
// the shared 4x4 block are done once; otherwise each tap reads its own texels.
__device__ float pcf3x3(const float* __restrict__ shadow, int S, const float csm[4]) {
    const float o = 1.0f / (float)S;
    int xi[3], yj[3];
    float a[3], b[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float uu = (csm[0] + (float)(k - 1) * o) * (float)S - 0.5f;
        const float vv = (csm[1] + (float)(k - 1) * o) * (float)S - 0.5f;
        const float fi = floorf(uu), fj = floorf(vv);
        a[k] = uu - fi;
        b[k] = vv - fj;
        xi[k] = (int)fmaxf(fminf(fi, (float)(S + 1)), -2.0f);
        yj[k] = (int)fmaxf(fminf(fj, (float)(S + 1)), -2.0f);
    }
    const float dref = csm[2];
    float result = 0.0f;
    if (xi[1] == xi[0] + 1 && xi[2] == xi[0] + 2 && yj[1] == yj[0] + 1 && yj[2] == yj[0] + 2) {
        float c[4][4];
#pragma unroll
        for (int y = 0; y < 4; ++y) {
            const size_t row = (size_t)min(max(yj[0] + y, 0), S - 1) * S;
#pragma unroll
            for (int x = 0; x < 4; ++x)
                c[y][x] = dref >= __ldg(&shadow[row + min(max(xi[0] + x, 0), S - 1)]) ? 1.0f : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < 3; ++j) {
#pragma unroll
            for (int i = 0; i < 3; ++i) {
                const float top = c[j][i] + a[i] * (c[j][i + 1] - c[j][i]);
                const float bot = c[j + 1][i] + a[i] * (c[j + 1][i + 1] - c[j + 1][i]);
                result += top + b[j] * (bot - top);
            }
        }
        return result * (1.0f / 9.0f);
    }
    for (int j = -1; j <= 1; ++j)
        for (int i = -1; i <= 1; ++i)
            result += sample_cmp(shadow, S, csm[0] + (float)i * o, csm[1] + (float)j * o, csm[2]);
    return result * (1.0f / 9.0f);
}

// pcf.slang:1-11 (5 taps) and the 3x3 option.
__device__ float pcf(const float* __restrict__ shadow, int S, const float csm[4], uint32_t mode) {
    float result = 0.0f;
    if (mode == RZ_PCF_3X3) return pcf3x3(shadow, S, csm);
    const float o = 0.00025f;
    result += sample_cmp(shadow, S, csm[0] - o, csm[1] - o, csm[2]);
    result += sample_cmp(shadow, S, csm[0] + o * 2.0f, csm[1], csm[2]);
    result += sample_cmp(shadow, S, csm[0], csm[1] + o * 2.0f, csm[2]);
    result += sample_cmp(shadow, S, csm[0] + o * 2.0f, csm[1] + o * 2.0f, csm[2]);
    result += sample_cmp(shadow, S, csm[0] - o * 2.0f, csm[1] - o * 2.0f, csm[2]);
    return result * (1.0f / 5.0f);
}

// lighting.slang:5-43
__device__ __forceinline__ V3 schlick_fresnel(float vDotH, V3 f0) {
    const float x = clamp01(1.0f - vDotH);
    const float x2 = x * x;
    const float p = x2 * x2 * x;  // pow(x, 5)
    return {f0.x + (1.0f - f0.x) * p, f0.y + (1.0f - f0.y) * p, f0.z + (1.0f - f0.z) * p};
}
__device__ __forceinline__ float distribution_ggx(V3 N, V3 H, float roughness) {
    const float PI = 3.14159265359f;
    const float a = roughness * roughness;
    const float a2 = a * a;
    const float NdotH = fmaxf(dot(N, H), 0.0f);
    const float NdotH2 = NdotH * NdotH;
    float denom = (NdotH2 * (a2 - 1.0f) + 1.0f);
    denom = PI * denom * denom;
    return fdiv(a2, denom);
}
__device__ __forceinline__ float geometry_schlick_ggx(float NdotV, float roughness) {
    const float r = roughness + 1.0f;
    const float k = (r * r) * 0.125f;
    return fdiv(NdotV, NdotV * (1.0f - k) + k);
}
__device__ __forceinline__ float geometry_smith(V3 N, V3 V, V3 L, float roughness) {
    const float NdotV = fmaxf(dot(N, V), 0.0f);
    const float NdotL = fmaxf(dot(N, L), 0.0f);
    return geometry_schlick_ggx(NdotL, roughness) * geometry_schlick_ggx(NdotV, roughness);
}

// The shadow map a fragment samples: with one cascade the view's map and csm
// unchanged; with n > 1 the finest cascade k whose coordinates
// (csm.xy - 0.5) * 2^-k + 0.5 keep the PCF footprint (2 texels) inside the map,
// else the coarsest. Writes the coordinates in that cascade to cc.
__device__ __forceinline__ const float* select_cascade(const ViewRec& VR, const float csm[4], float cc[4]) {
#pragma unroll
    for (int i = 0; i < 4; ++i) cc[i] = csm[i];
    const float* base = reinterpret_cast<const float*>(VR.shadow);
    const int n = VR.cascades;
    if (n <= 1) return base;
    const float m = 2.0f / (float)VR.shadow_w;
    const float hi = 1.0f - m;
    int k = 0;
    for (; k < n; ++k) {
        float x = csm[0], y = csm[1];
        if (k > 0) {
            const float sc = ldexpf(1.0f, -k);
            x = (csm[0] - 0.5f) * sc + 0.5f;
            y = (csm[1] - 0.5f) * sc + 0.5f;
        }
        if ((x >= m && x <= hi && y >= m && y <= hi) || k == n - 1) {
            cc[0] = x;
            cc[1] = y;
            break;
        }
    }
    return base + (size_t)k * (size_t)VR.shadow_w * (size_t)VR.shadow_h;
}

// fragmentMain, src/shaders/basic.slang:137-344. Returns false on discard.
// kLit: the caller has checked that the view renders the default output
// (fragment_output 0) with the light, its shadow and the BRDF on, so those
// branches are taken without testing them and the debug outputs are not
// compiled into this copy. A view takes the same branches at every pixel, and
// the shading kernel runs the specialised copy for such views: the code its
// warps execute is then smaller (fewer instruction-fetch stalls).
template <bool kLit = false>
__device__ bool fragment_main(const ViewRec& VR, const rz_scene_data& sd, const GpuMaterial* md, const Frag& bv,
                              const Sampler& smp, float out[4], float* albedo = nullptr) {
    const V3 ambientLight{sd.ambient_color[0], sd.ambient_color[1], sd.ambient_color[2]};
    float outFragColor[4] = {bv.color[0], bv.color[1], bv.color[2], bv.color[3]};
    float imageTextureColor[4] = {outFragColor[0], outFragColor[1], outFragColor[2], outFragColor[3]};
    float alpha = bv.color[3];
    float sampledRoughness = 0.0f, sampledMetallic = 0.0f;
    V3 lightNormal = fnormalize(bv.normal);
    const V3 lightDir = fnormalize(bv.lightDir);
    const V3 bitangent = bv.bitangent;
    SampleCoords cache;
    cache.valid = false;
    if (md) {
#pragma unroll
        for (int k = 0; k < 4; ++k) outFragColor[k] = md->color[k];
#pragma unroll
        for (int k = 0; k < 4; ++k) imageTextureColor[k] = outFragColor[k];
        alpha = fminf(md->color[3], alpha);
        if (sd.normal_maps_enabled == 1 && md->tex[1] != RZ_INVALID_INDEX) {
            float s[4];
            smp.sample(md->tex[1], md->sampler[1], bv, cache, s);
            const V3 m{s[0] * 2.0f - 1.0f, s[1] * 2.0f - 1.0f, s[2] * 2.0f - 1.0f};
            const V3 n = fnormalize(bv.normal);
            const V3 t = fnormalize(bv.tangent - n * dot(bv.tangent, n));
            const V3 b = fnormalize(cross(bv.normal, bv.tangent) * bv.sigma);
            lightNormal = fnormalize(t * m.x + b * m.y + n * m.z);
        }
        if (md->tex[0] != RZ_INVALID_INDEX) {
            smp.sample(md->tex[0], md->sampler[0], bv, cache, imageTextureColor);
            alpha = fminf(imageTextureColor[3], alpha);
        }
        float s[4];
        if (md->tex[3] != RZ_INVALID_INDEX) smp.sample(md->tex[3], md->sampler[3], bv, cache, s);
        else smp.sample(md->tex[2], md->sampler[2], bv, cache, s);
        sampledRoughness = s[1];
        sampledMetallic = s[2];
    }
    if (albedo) {
#pragma unroll
        for (int k = 0; k < 3; ++k) albedo[k] = imageTextureColor[k];
    }
    const V3 V = fnormalize(bv.viewDir);
    const V3 L = lightDir;
    const V3 N = lightNormal;
    const V3 H = fnormalize(L + V);
    const float cosTheta = clamp01(dot(L, N));
    const float cosPhi = clamp01(dot(H, N));
    const float lDotN = cosTheta;
    const float lDotH = clamp01(dot(L, H));
    const float nDotV = clamp01(dot(N, V));
    V3 c3;
    bool set = true;
    switch (kLit ? 0u : sd.fragment_output) {
        case 0: c3 = V3{imageTextureColor[0], imageTextureColor[1], imageTextureColor[2]}; break;
        case 1: c3 = fnormalize(bv.worldNormal) * 0.5f + V3{0.5f, 0.5f, 0.5f}; break;
        case 2: c3 = fnormalize(bv.tangent) * 0.5f + V3{0.5f, 0.5f, 0.5f}; break;
        case 3: c3 = fnormalize(bv.lightDir) * 0.5f + V3{0.5f, 0.5f, 0.5f}; break;
        case 4: c3 = fnormalize(bv.viewDir) * 0.5f + V3{0.5f, 0.5f, 0.5f}; break;
        case 5: c3 = V3{bv.color[0], bv.color[1], bv.color[2]}; break;
        case 6: c3 = lightNormal * 0.5f + V3{0.5f, 0.5f, 0.5f}; break;
        case 7: c3 = bitangent * 0.5f + V3{0.5f, 0.5f, 0.5f}; break;
        case 8: c3 = V3{cosTheta, cosTheta, cosTheta} * 0.5f + V3{0.5f, 0.5f, 0.5f}; break;
        case 9: c3 = V3{cosPhi, cosPhi, cosPhi} * 0.5f + V3{0.5f, 0.5f, 0.5f}; break;
        case 10: c3 = V3{lDotH, lDotH, lDotH} * 0.5f + V3{0.5f, 0.5f, 0.5f}; break;
        case 11: c3 = V3{nDotV, nDotV, nDotV} * 0.5f + V3{0.5f, 0.5f, 0.5f}; break;
        case 12: c3 = V3{bv.uv[0], bv.uv[1], 0.0f}; break;
        case 13: c3 = V3{sampledRoughness, 0.05f, 0.05f}; break;
        case 14: c3 = V3{sampledMetallic, 0.05f, 0.05f}; break;
        case 15: c3 = V3{1.0f - alpha, 0.05f, 0.05f}; break;
        default: set = false; break;
    }
    if (set) {
        outFragColor[0] = c3.x;
        outFragColor[1] = c3.y;
        outFragColor[2] = c3.z;
        outFragColor[3] = alpha;
    }
    if (kLit || sd.light_enabled > 0) {
        float shadowFactor = 1.0f;
        if (kLit || sd.shadows_enabled == 1)
        {
            float cc[4];
            const float* map = select_cascade(VR, bv.csm, cc);
            shadowFactor = pcf(map, VR.shadow_w, cc, VR.pcf_mode);
        }
        if (!kLit && sd.brdf_lighting_enabled == 0) {
            const float ml = fmaxf(cosTheta, 0.0f);
            const V3 sunLight{sd.sunlight_color[0] * ml, sd.sunlight_color[1] * ml, sd.sunlight_color[2] * ml};
            outFragColor[0] = outFragColor[0] * fmaxf(ambientLight.x, sunLight.x * shadowFactor);
            outFragColor[1] = outFragColor[1] * fmaxf(ambientLight.y, sunLight.y * shadowFactor);
            outFragColor[2] = outFragColor[2] * fmaxf(ambientLight.z, sunLight.z * shadowFactor);
            outFragColor[3] = outFragColor[3] * alpha;
        } else {
            const float roughness = sampledRoughness;
            const float metallic = sampledMetallic;
            const float f04 = 0.04f;
            const V3 f0{f04 * (1.0f - metallic) + outFragColor[0] * metallic, f04 * (1.0f - metallic) + outFragColor[1] * metallic,
                        f04 * (1.0f - metallic) + outFragColor[2] * metallic};
            const float ndf = distribution_ggx(N, H, roughness);
            const float g = geometry_smith(N, V, L, roughness);
            const V3 f = schlick_fresnel(fmaxf(dot(H, V), 0.0f), f0);
            V3 kD{1.0f - f.x, 1.0f - f.y, 1.0f - f.z};
            kD = kD * (1.0f - metallic);
            const V3 numerator = f * (ndf * g);
            const float denominator = 4.0f * nDotV * lDotN + 0.0001f;
            const float inv_den = fdiv(1.0f, denominator);
            const V3 specular{numerator.x * inv_den, numerator.y * inv_den, numerator.z * inv_den};
            const float inv_pi = 1.0f / 3.14159265f;
            const V3 diffuse{outFragColor[0] * inv_pi, outFragColor[1] * inv_pi, outFragColor[2] * inv_pi};
            const float li = sd.light_intensity;
            const V3 sunLight{sd.sunlight_color[0] * li, sd.sunlight_color[1] * li, sd.sunlight_color[2] * li};
            V3 brdf = mul3(mul3(kD, diffuse) + specular, sunLight) * lDotN;
            brdf = V3{fmaxf(ambientLight.x * diffuse.x, brdf.x * shadowFactor), fmaxf(ambientLight.y * diffuse.y, brdf.y * shadowFactor),
                      fmaxf(ambientLight.z * diffuse.z, brdf.z * shadowFactor)};
            outFragColor[0] = brdf.x;
            outFragColor[1] = brdf.y;
            outFragColor[2] = brdf.z;
            outFragColor[3] = alpha;
        }
    }
    if (md) {
        if (md->alpha_mode == 1 && alpha < md->alpha_cutoff) return false;
        outFragColor[3] = alpha;
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = outFragColor[k];
    return true;
}

__device__ __forceinline__ uint32_t encode_srgb8(float c) {
    if (!(c > 0.0f)) c = 0.0f;
    if (c > 1.0f) c = 1.0f;
    const float s = c <= 0.0031308f ? c * 12.92f : 1.055f * __powf(c, 1.0f / 2.4f) - 0.055f;
    return (uint32_t)floorf(s * 255.0f + 0.5f);
}
__device__ __forceinline__ uint32_t encode_unorm8(float c) {
    if (!(c > 0.0f)) c = 0.0f;
    if (c > 1.0f) c = 1.0f;
    return (uint32_t)floorf(c * 255.0f + 0.5f);
}
__device__ __forceinline__ float half_round(float x) { return __half2float(__float2half_rn(x)); }

// Varying record of one (draw, vertex): the vertex-stage outputs the fragment
// stage reads plus the clip position, 32 floats:
//   0-2 normal, 3-5 viewDir, 6-8 lightDir, 9-11 tangent, 12 sigma, 13-16 color,
//   17-18 uv, 19-22 csm.near, 23-25 worldNormal, 26-28 bitangent, 29-31 clip x, y, w.
constexpr int kVaryingF4 = 8;

__device__ __forceinline__ uint32_t find_draw_by_varying(const DrawRec* __restrict__ draws, uint32_t n, uint32_t i) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&draws[mid].varying_base) <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// The vertex stage, once per (draw, mesh vertex): records [first, varying_count).
__global__ void __launch_bounds__(256) k_vertex(ShadeParams P, uint32_t first) {
    const uint32_t i = first + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.varying_count) return;
    const uint32_t d = find_draw_by_varying(P.draws, P.draw_count, i);
    const DrawRec dr = P.draws[d];
    const DrawConsts& dc = P.consts[d];
    const rz_object& gd = P.objects[dr.object];
    const GpuMaterial* md = dr.material >= 0 ? &P.materials[dr.material] : nullptr;
    const bool has_nm = md ? (md->tex[1] != RZ_INVALID_INDEX) : false;
    // the 64-byte vertex record as four 16-byte loads
    const float4* vp = reinterpret_cast<const float4*>(P.vertices + dr.vertex_base + (i - dr.varying_base));
    const float4 q0 = __ldg(vp), q1 = __ldg(vp + 1), q2 = __ldg(vp + 2), q3 = __ldg(vp + 3);
    rz_vertex v;
    v.position[0] = q0.x; v.position[1] = q0.y; v.position[2] = q0.z;
    v.normal[0] = q0.w; v.normal[1] = q1.x; v.normal[2] = q1.y;
    v.tangent[0] = q1.z; v.tangent[1] = q1.w; v.tangent[2] = q2.x; v.tangent[3] = q2.y;
    v.color[0] = q2.z; v.color[1] = q2.w; v.color[2] = q3.x; v.color[3] = q3.y;
    v.uv[0] = q3.z; v.uv[1] = q3.w;
    VsOut o;
    vertex_main(*P.views[dr.view].scene, gd, dc, md != nullptr, has_nm, v, o);
    const float4 clip = transform_point(dc.mvp, v.position[0], v.position[1], v.position[2]);
    float4* dst = P.varyings + (size_t)i * kVaryingF4;
    dst[0] = make_float4(o.normal.x, o.normal.y, o.normal.z, o.viewDir.x);
    dst[1] = make_float4(o.viewDir.y, o.viewDir.z, o.lightDir.x, o.lightDir.y);
    dst[2] = make_float4(o.lightDir.z, o.tangent.x, o.tangent.y, o.tangent.z);
    dst[3] = make_float4(o.sigma, o.color[0], o.color[1], o.color[2]);
    dst[4] = make_float4(o.color[3], o.uv[0], o.uv[1], o.csm[0]);
    dst[5] = make_float4(o.csm[1], o.csm[2], o.csm[3], o.worldNormal.x);
    dst[6] = make_float4(o.worldNormal.y, o.worldNormal.z, o.bitangent.x, o.bitangent.y);
    dst[7] = make_float4(o.bitangent.z, clip.x, clip.y, clip.w);
}

void launch_vertex(const ShadeParams& p, cudaStream_t stream) {
    if (p.varying_count == 0 || p.draw_count == 0) return;
    k_vertex<<<(p.varying_count + 255) / 256, 256, 0, stream>>>(p, 0u);
    note_launch();
}

void launch_vertex_range(const ShadeParams& p, uint32_t first, cudaStream_t stream) {
    if (p.varying_count <= first || p.draw_count == 0) return;
    k_vertex<<<(p.varying_count - first + 255) / 256, 256, 0, stream>>>(p, first);
    note_launch();
}

// Shade triangle `tri` (pass-global id) at pixel (px, py) from the varying
// records of its three vertices.
// With `aux` non-null it also returns the G-buffer values: albedo (the sampled
// base colour, rgb) and the interpolated world-space normal (normalised, xyz).
// With `pn` non-null the pixel-centre coordinates come from there (see pixel_ndc).
template <bool kLit = false>
__device__ bool shade_pixel(const ShadeParams& P, const ViewRec& VR, const rz_scene_data& sd, const Sampler& smp, uint32_t tri,
                            int px, int py, float out[4], float* aux = nullptr, const PixelNdc* pn = nullptr) {
    uint32_t d;
    const float4* rec[3];
    if (P.tri_refs) {  // the opaque list: the camera setup recorded the draw and the vertices
        const uint4 r = __ldg(&P.tri_refs[tri]);
        d = r.x;
        rec[0] = P.varyings + (size_t)r.y * kVaryingF4;
        rec[1] = P.varyings + (size_t)r.z * kVaryingF4;
        rec[2] = P.varyings + (size_t)r.w * kVaryingF4;
    } else {
        d = find_draw(P.draws, P.draw_count, tri);
        const DrawRec& dl = P.draws[d];
        const uint32_t t = tri - dl.tri_base;
#pragma unroll
        for (int k = 0; k < 3; ++k)
            rec[k] = P.varyings + (size_t)(__ldg(&P.indices[dl.first_index + 3u * t + k]) + dl.varying_base) * kVaryingF4;
    }
    const int32_t material = __ldg(&P.draws[d].material);
    const GpuMaterial* md = material >= 0 ? &P.materials[material] : nullptr;
    float4 clip[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float4 q = __ldg(rec[k] + 7);
        clip[k] = make_float4(q.y, q.z, 0.0f, q.w);
    }
    float b[3], bq0[3], bqx[3], bqy[3];
    const int qx = px & ~1, qy = py & ~1;
    float xp, yp, xq, yq, xq1, yq1;  // ndc of px, py, qx, qy, qx + 1, qy + 1
    if (pn) {
        xp = pn->xp;
        yp = pn->yp;
        xq = pn->xq;
        yq = pn->yq;
        xq1 = pn->xq1;
        yq1 = pn->yq1;
    } else {
        xp = ndc(px, VR.width);
        yp = ndc(py, VR.height);
        xq = ndc(qx, VR.width);
        yq = ndc(qy, VR.height);
        xq1 = ndc(qx + 1, VR.width);
        yq1 = ndc(qy + 1, VR.height);
    }
    barycentrics_n(clip[0], clip[1], clip[2], xp, yp, b);
    barycentrics_n(clip[0], clip[1], clip[2], xq, yq, bq0);
    barycentrics_n(clip[0], clip[1], clip[2], xq1, yq, bqx);
    barycentrics_n(clip[0], clip[1], clip[2], xq, yq1, bqy);
    const bool debug_extra = (!kLit && (sd.fragment_output == 1 || sd.fragment_output == 7)) || aux != nullptr;
    Frag f;
    float u0[2], ux[2], uy[2];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float4 a0 = __ldg(rec[k] + 0), a1 = __ldg(rec[k] + 1), a2 = __ldg(rec[k] + 2);
        const float4 a3 = __ldg(rec[k] + 3), a4 = __ldg(rec[k] + 4), a5 = __ldg(rec[k] + 5);
        float4 a6 = make_float4(0.f, 0.f, 0.f, 0.f), a7 = make_float4(0.f, 0.f, 0.f, 0.f);
        if (debug_extra) {
            a6 = __ldg(rec[k] + 6);
            a7 = __ldg(rec[k] + 7);
        }
        const V3 normal{a0.x, a0.y, a0.z}, viewDir{a0.w, a1.x, a1.y}, lightDir{a1.z, a1.w, a2.x};
        const V3 tangent{a2.y, a2.z, a2.w}, worldNormal{a5.w, a6.x, a6.y}, bitangent{a6.z, a6.w, a7.x};
        const float sigma = a3.x;
        const float color[4] = {a3.y, a3.z, a3.w, a4.x};
        const float uv[2] = {a4.y, a4.z};
        const float csm[4] = {a4.w, a5.x, a5.y, a5.z};
        const float w = b[k];
        if (k == 0) {
            f.normal = normal * w;
            f.worldNormal = worldNormal * w;
            f.viewDir = viewDir * w;
            f.lightDir = lightDir * w;
            f.tangent = tangent * w;
            f.bitangent = bitangent * w;
#pragma unroll
            for (int i = 0; i < 4; ++i) f.color[i] = color[i] * w;
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                f.uv[i] = uv[i] * w;
                u0[i] = uv[i] * bq0[0];
                ux[i] = uv[i] * bqx[0];
                uy[i] = uv[i] * bqy[0];
            }
            f.sigma = sigma * w;
#pragma unroll
            for (int i = 0; i < 4; ++i) f.csm[i] = csm[i] * w;
        } else {
            f.normal = f.normal + normal * w;
            f.worldNormal = f.worldNormal + worldNormal * w;
            f.viewDir = f.viewDir + viewDir * w;
            f.lightDir = f.lightDir + lightDir * w;
            f.tangent = f.tangent + tangent * w;
            f.bitangent = f.bitangent + bitangent * w;
#pragma unroll
            for (int i = 0; i < 4; ++i) f.color[i] = f.color[i] + color[i] * w;
#pragma unroll
            for (int i = 0; i < 2; ++i) {
                f.uv[i] = f.uv[i] + uv[i] * w;
                u0[i] = u0[i] + uv[i] * bq0[k];
                ux[i] = ux[i] + uv[i] * bqx[k];
                uy[i] = uy[i] + uv[i] * bqy[k];
            }
            f.sigma = f.sigma + sigma * w;
#pragma unroll
            for (int i = 0; i < 4; ++i) f.csm[i] = f.csm[i] + csm[i] * w;
        }
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        f.duvdx[i] = ux[i] - u0[i];
        f.duvdy[i] = uy[i] - u0[i];
    }
    if (aux) {
        const V3 n = fnormalize(f.worldNormal);
        aux[3] = n.x;
        aux[4] = n.y;
        aux[5] = n.z;
    }
    return fragment_main<kLit>(VR, sd, md, f, smp, out, aux);
}

// Whether a view renders the default output with the light, its shadow and the
// BRDF on (the branches fragment_main<true> takes without testing).
__device__ __forceinline__ bool lit_view(const rz_scene_data& sd) {
    return sd.fragment_output == 0 && sd.light_enabled > 0 && sd.shadows_enabled == 1 && sd.brdf_lighting_enabled != 0;
}

// Octahedral encoding of a unit vector into two f16 (x in the low half).
__device__ __forceinline__ uint32_t encode_octahedral(float x, float y, float z) {
    const float s = fabsf(x) + fabsf(y) + fabsf(z);
    float u = 0.0f, v = 0.0f;
    if (s > 0.0f) {
        u = x / s;
        v = y / s;
        if (z < 0.0f) {
            const float au = 1.0f - fabsf(v), av = 1.0f - fabsf(u);
            u = u >= 0.0f ? au : -au;
            v = v >= 0.0f ? av : -av;
        }
    }
    const __half2 h = __floats2half2_rn(u, v);
    return *reinterpret_cast<const uint32_t*>(&h);
}

// The view a 16x16 shading tile belongs to (tiles are numbered view by view).
__device__ __forceinline__ uint32_t tile_view(const ViewRec* __restrict__ views, uint32_t n, uint32_t tile) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&views[mid].shade_block_base) <= tile) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Average of four RGBA16F sample values ((s0 + s1) + (s2 + s3)) / 4, rounded
// to RGBA16F: the AVERAGE resolve of the multisampled draw image
// (src/Engine/Graphics.cpp:5571-5572).
__device__ __forceinline__ float resolve4(float a, float b, float c, float d) {
    return half_round(((a + b) + (c + d)) * 0.25f);
}

// One pixel of a 4x multisampled view: each distinct triangle among its samples
// is shaded once at the pixel centre (no sample shading, as the reference's
// pipeline), its colour is rounded to RGBA16F and given to the samples it
// covers; uncovered samples keep the clear colour. Without blended surfaces the
// samples are resolved and encoded here; with them they go to the RGBA16F
// sample planes for k_blend. The depth output is sample 0's.
template <bool kLit>
__device__ __forceinline__ void shade_msaa(const ShadeParams& P, const ViewRec& VR, const float* s_srgb,
                                           const PixelNdc& pn, int px, int py, size_t p) {
    const size_t plane = (size_t)VR.width * VR.height;
    uint32_t ids[kMsaaSamples];
    unsigned long long key0 = 0;
#pragma unroll
    for (int k = 0; k < kMsaaSamples; ++k) {
        const unsigned long long key = VR.vis[p + k * plane];
        if (k == 0) key0 = key;
        ids[k] = (uint32_t)key;
    }
    float cs[kMsaaSamples][4];
    const Sampler smp{&P, s_srgb};
    const bool gbuffer = VR.gb_albedo != nullptr;
    float gs[kMsaaSamples][6];  // G-buffer values per sample (albedo rgb, normal xyz)
#pragma unroll
    for (int k = 0; k < kMsaaSamples; ++k) {
        float c[4] = {0.0f, 0.05f, 0.1f, 1.0f};  // clear colour, src/Engine/Graphics.cpp:5416-5419
        float aux[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        int same = -1;
#pragma unroll
        for (int j = 0; j < k; ++j)
            if (same < 0 && ids[j] == ids[k]) same = j;
        if (same >= 0) {
#pragma unroll
            for (int i = 0; i < 4; ++i) cs[k][i] = cs[same][i];
#pragma unroll
            for (int i = 0; i < 6; ++i) gs[k][i] = gs[same][i];
            continue;
        }
        if (ids[k] != 0) {
            float o[4];
            if (shade_pixel<kLit>(P, VR, *VR.scene, smp, ids[k] - 1u, px, py, o, gbuffer ? aux : nullptr, &pn)) {
#pragma unroll
                for (int i = 0; i < 4; ++i) c[i] = o[i];
            }
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) cs[k][i] = half_round(c[i]);
#pragma unroll
        for (int i = 0; i < 6; ++i) gs[k][i] = aux[i];
    }
    if (gbuffer) {
        // G-buffer of a multisampled pixel: albedo and normal averaged over the samples,
        // coverage = covered samples / 4 in the albedo's alpha
        float g[6];
#pragma unroll
        for (int i = 0; i < 6; ++i) g[i] = ((gs[0][i] + gs[1][i]) + (gs[2][i] + gs[3][i])) * 0.25f;
        uint32_t covered = 0;
#pragma unroll
        for (int k = 0; k < kMsaaSamples; ++k) covered += ids[k] != 0 ? 1u : 0u;
        VR.gb_albedo[p] = encode_srgb8(half_round(g[0])) | (encode_srgb8(half_round(g[1])) << 8) |
                          (encode_srgb8(half_round(g[2])) << 16) | (encode_unorm8((float)covered * 0.25f) << 24);
        const float len2 = g[3] * g[3] + g[4] * g[4] + g[5] * g[5];
        const float inv = len2 > 0.0f ? rsqrtf(len2) : 0.0f;
        VR.gb_normal[p] = encode_octahedral(g[3] * inv, g[4] * inv, g[5] * inv);
    }
    VR.depth[p] = __uint_as_float((uint32_t)(key0 >> 32));
    if (P.blended) {
#pragma unroll
        for (int k = 0; k < kMsaaSamples; ++k) {
            const __half2 rg = __floats2half2_rn(cs[k][0], cs[k][1]), ba = __floats2half2_rn(cs[k][2], cs[k][3]);
            VR.color16[p + k * plane] =
                make_uint2(*reinterpret_cast<const uint32_t*>(&rg), *reinterpret_cast<const uint32_t*>(&ba));
        }
        return;
    }
    float r[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) r[i] = resolve4(cs[0][i], cs[1][i], cs[2][i], cs[3][i]);
    VR.color[p] = encode_srgb8(r[0]) | (encode_srgb8(r[1]) << 8) | (encode_srgb8(r[2]) << 16) | (encode_unorm8(r[3]) << 24);
}

// The pixel (px, py) of this thread in the block's 16x16 tile, and its
// pixel-centre coordinates. Each lane of a warp (16 columns, 2 rows) computes its
// column's and its row's coordinate (the values ndc() gives) and takes its quad's
// from the lanes of its quad's first column and of the two rows, so the tile needs
// no shared table and no second block barrier. All lanes take part (shuffles).
__device__ __forceinline__ PixelNdc pixel_ndc(const ShadeParams& P, const ViewRec& VR, int& px, int& py) {
    const uint32_t lt = blockIdx.x + P.block_offset - VR.shade_block_base;
    const uint32_t tiles_x = ((uint32_t)VR.width + 15) / 16;
    px = (int)(lt % tiles_x) * 16 + (int)threadIdx.x;
    py = (int)(lt / tiles_x) * 16 + (int)threadIdx.y;
    const int lane = (int)(threadIdx.x + 16 * (threadIdx.y & 1));
    PixelNdc pn;
    pn.xp = ndc(px, VR.width);
    pn.yp = ndc(py, VR.height);
    pn.xq = __shfl_sync(0xffffffffu, pn.xp, lane & 14);
    pn.xq1 = __shfl_sync(0xffffffffu, pn.xp, (lane & 14) + 1);
    pn.yq = __shfl_sync(0xffffffffu, pn.yp, lane & 15);
    pn.yq1 = __shfl_sync(0xffffffffu, pn.yp, (lane & 15) + 16);
    return pn;
}

__global__ void __launch_bounds__(256, 4) k_shade(ShadeParams P) {
    __shared__ float s_srgb[256];
    __shared__ uint32_t s_view;
    {
        const int t = threadIdx.y * blockDim.x + threadIdx.x;
        s_srgb[t] = P.srgb_table[t];
        if (t == 0) s_view = tile_view(P.views, P.view_count, blockIdx.x + P.block_offset);
    }
    __syncthreads();
    const ViewRec& VR = P.views[s_view];
    int px, py;
    const PixelNdc pn = pixel_ndc(P, VR, px, py);
    if (px >= VR.width || py >= VR.height) return;
    const size_t p = (size_t)py * VR.width + px;
    const unsigned long long key = VR.vis[p];
    const uint32_t id = (uint32_t)key;
    float col[4] = {0.0f, 0.05f, 0.1f, 1.0f};  // clear colour, src/Engine/Graphics.cpp:5416-5419
    const bool gbuffer = VR.gb_albedo != nullptr;
    float aux[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    if (id != 0) {
        const Sampler smp{&P, s_srgb};
        float o[4];
        const rz_scene_data& sd = *VR.scene;
        float* const ax = gbuffer ? aux : nullptr;
        if (lit_view(sd) ? shade_pixel<true>(P, VR, sd, smp, id - 1u, px, py, o, ax, &pn)
                         : shade_pixel<false>(P, VR, sd, smp, id - 1u, px, py, o, ax, &pn)) {
#pragma unroll
            for (int k = 0; k < 4; ++k) col[k] = o[k];
        }
    }
    if (gbuffer) {
        VR.gb_albedo[p] = encode_srgb8(half_round(aux[0])) | (encode_srgb8(half_round(aux[1])) << 8) |
                          (encode_srgb8(half_round(aux[2])) << 16) | ((id != 0 ? 255u : 0u) << 24);
        VR.gb_normal[p] = encode_octahedral(aux[3], aux[4], aux[5]);
    }
    VR.depth[p] = __uint_as_float((uint32_t)(key >> 32));
    if (P.blended) {  // blended surfaces follow: keep the RGBA16F draw image
        const __half2 rg = __floats2half2_rn(col[0], col[1]), ba = __floats2half2_rn(col[2], col[3]);
        VR.color16[p] = make_uint2(*reinterpret_cast<const uint32_t*>(&rg), *reinterpret_cast<const uint32_t*>(&ba));
        return;
    }
    const uint32_t r = encode_srgb8(half_round(col[0]));
    const uint32_t g = encode_srgb8(half_round(col[1]));
    const uint32_t b = encode_srgb8(half_round(col[2]));
    const uint32_t a = encode_unorm8(half_round(col[3]));
    VR.color[p] = r | (g << 8) | (b << 16) | (a << 24);
}

// k_shade for 4x multisampled views.
__global__ void __launch_bounds__(256, 4) k_shade_msaa(ShadeParams P) {
    __shared__ float s_srgb[256];
    __shared__ uint32_t s_view;
    {
        const int t = threadIdx.y * blockDim.x + threadIdx.x;
        s_srgb[t] = P.srgb_table[t];
        if (t == 0) s_view = tile_view(P.views, P.view_count, blockIdx.x + P.block_offset);
    }
    __syncthreads();
    const ViewRec& VR = P.views[s_view];
    int px, py;
    const PixelNdc pn = pixel_ndc(P, VR, px, py);
    if (px >= VR.width || py >= VR.height) return;
    const size_t p = (size_t)py * VR.width + px;
    if (lit_view(*VR.scene)) shade_msaa<true>(P, VR, s_srgb, pn, px, py, p);
    else shade_msaa<false>(P, VR, s_srgb, pn, px, py, p);
}

void launch_shade(const ShadeParams& p, cudaStream_t stream) {
    if (p.shade_blocks == 0) return;
    note_launch();
    if (p.samples > 1) {
        k_shade_msaa<<<p.shade_blocks, dim3(16, 16), 0, stream>>>(p);
        return;
    }
    k_shade<<<p.shade_blocks, dim3(16, 16), 0, stream>>>(p);
}

// ---------------------------------------------------------------------------
// sub-pixel sources of the learned half-resolution path (G-buffer)
// ---------------------------------------------------------------------------

// Screen position (pixels) and NDC depth of the three vertices of an opaque
// triangle: the clip position the vertex stage computes (the draw's MVP times
// the mesh position), divided by w.
struct SubTri {
    float X[3], Y[3], Z[3];
    float inv_area;  // 1 / twice the signed screen area (0 when degenerate)
    bool valid;      // every w > 0
};

__device__ __forceinline__ SubTri sub_triangle(const ShadeParams& P, uint32_t id, float hw, float hh) {
    const uint32_t tri = id - 1u;
    const uint32_t d = find_draw(P.draws, P.draw_count, tri);
    const DrawRec dr = P.draws[d];
    const uint32_t t = tri - dr.tri_base;
    const float* M = P.consts[d].mvp;
    SubTri g;
    g.valid = true;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const uint32_t vi = __ldg(&P.indices[dr.first_index + 3u * t + k]) + dr.vertex_base;
        const float* pos = P.vertices[vi].position;
        const float4 c = transform_point(M, __ldg(pos), __ldg(pos + 1), __ldg(pos + 2));
        g.valid = g.valid && c.w > 0.0f;
        const float rw = 1.0f / c.w;
        g.X[k] = (c.x * rw) * hw + hw;
        g.Y[k] = (c.y * rw) * hh + hh;
        g.Z[k] = c.z * rw;
    }
    const float area = (g.X[1] - g.X[0]) * (g.Y[2] - g.Y[0]) - (g.X[2] - g.X[0]) * (g.Y[1] - g.Y[0]);
    g.inv_area = area != 0.0f ? 1.0f / area : 0.0f;
    return g;
}

// Shared-memory table of a tile's distinct triangles (open addressing, 128
// slots): each triangle's geometry is computed once per tile, not once per
// pixel that considers it. Key 0 marks an empty slot (ids are >= 1).
constexpr int kSubSlots = 128;

__device__ __forceinline__ uint32_t sub_slot(uint32_t id) { return (id * 2654435761u) >> 25; }

__device__ __forceinline__ void sub_insert(uint32_t* keys, uint32_t id) {
    uint32_t h = sub_slot(id);
    for (int i = 0; i < kSubSlots; ++i) {
        const uint32_t prev = atomicCAS(&keys[h], 0u, id);
        if (prev == 0u || prev == id) return;
        h = (h + 1) & (kSubSlots - 1);
    }  // table full: pixels that need this triangle compute its geometry themselves
}

__device__ __forceinline__ int sub_find(const uint32_t* keys, uint32_t id) {
    uint32_t h = sub_slot(id);
    for (int i = 0; i < kSubSlots; ++i) {
        const uint32_t k = keys[h];
        if (k == id) return (int)h;
        if (k == 0u) return -1;
        h = (h + 1) & (kSubSlots - 1);
    }
    return -1;
}

// For the x2 reconstruction of the learned path: which triangle is in front at
// each of the four points (x + 0.25 / 0.75, y + 0.25 / 0.75) that the pixel's
// four full-resolution pixels sample, among the triangles visible at the 3x3
// neighbourhood's pixel centres (covered by the float edge functions, front-most
// by the depth plane through the vertices' z / w, larger nearer as in the depth
// test), and which of each point's bilinear sources (own, horizontal, vertical,
// diagonal neighbour, clamped at the borders) show it: bit 4k + s,
// k = 2 * (y half) + (x half). A pixel whose neighbourhood shows one triangle
// (or none) keeps every source (0xFFFF). The arithmetic is plain float without
// contraction, restated by the oracle bit for bit. The reference has no learned
// path; nothing here follows a reference file.
__global__ void __launch_bounds__(256) k_subpixel_sources(ShadeParams P) {
    __shared__ uint32_t s_view;
    __shared__ uint32_t s_ids[18][18];  // the tile's triangle ids with a one-pixel border (clamped)
    __shared__ uint32_t s_keys[kSubSlots];
    __shared__ SubTri s_geo[kSubSlots];
    __shared__ uint32_t s_edge_count;
    __shared__ uint8_t s_edges[256];  // the tile's pixels whose neighbourhood shows more than one triangle
    const int tid = threadIdx.y * 16 + threadIdx.x;
    if (tid == 0) {
        s_view = tile_view(P.views, P.view_count, blockIdx.x + P.block_offset);
        s_edge_count = 0u;
    }
    if (tid < kSubSlots) s_keys[tid] = 0u;
    __syncthreads();
    const ViewRec& VR = P.views[s_view];
    if (!VR.gb_sources) return;  // uniform over the block
    const uint32_t lt = blockIdx.x + P.block_offset - VR.shade_block_base;
    const uint32_t tiles_x = ((uint32_t)VR.width + 15) / 16;
    const int x0 = (int)(lt % tiles_x) * 16, y0 = (int)(lt / tiles_x) * 16;
    const int W = VR.width, H = VR.height;
    const float hw = (float)W * 0.5f, hh = (float)H * 0.5f;
    for (int i = tid; i < 18 * 18; i += 256) {
        const int yy = min(max(y0 + i / 18 - 1, 0), H - 1), xx = min(max(x0 + i % 18 - 1, 0), W - 1);
        s_ids[i / 18][i % 18] = (uint32_t)VR.vis[(size_t)yy * W + xx];
    }
    __syncthreads();
    {
        const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
        bool same = true;
#pragma unroll
        for (int dy = 0; dy < 3; ++dy)
#pragma unroll
            for (int dx = 0; dx < 3; ++dx) same = same && s_ids[threadIdx.y + dy][threadIdx.x + dx] == s_ids[threadIdx.y + 1][threadIdx.x + 1];
        if (x < W && y < H) {
            if (same) {
                VR.gb_sources[(size_t)y * W + x] = 0xFFFFu;
            } else {  // the distinct triangles the edge pixels consider (geometry once each), and the pixel
#pragma unroll
                for (int dy = 0; dy < 3; ++dy)
#pragma unroll
                    for (int dx = 0; dx < 3; ++dx)
                        if (s_ids[threadIdx.y + dy][threadIdx.x + dx] != 0u) sub_insert(s_keys, s_ids[threadIdx.y + dy][threadIdx.x + dx]);
                s_edges[atomicAdd(&s_edge_count, 1u)] = (uint8_t)tid;
            }
        }
    }
    __syncthreads();
    if (tid < kSubSlots && s_keys[tid] != 0u) s_geo[tid] = sub_triangle(P, s_keys[tid], hw, hh);
    __syncthreads();
    // the edge pixels, packed onto the first lanes of the block
    const uint32_t n_edges = s_edge_count;
    if ((uint32_t)tid >= n_edges) return;
    const int ex = s_edges[tid] & 15, ey = s_edges[tid] >> 4;
    const int x = x0 + ex, y = y0 + ey;
    uint32_t nb[9];
#pragma unroll
    for (int dy = 0; dy < 3; ++dy)
#pragma unroll
        for (int dx = 0; dx < 3; ++dx) nb[dy * 3 + dx] = s_ids[ey + dy][ex + dx];
    const uint32_t own = nb[4];
    uint32_t mask;
    {
        uint32_t best[4] = {0u, 0u, 0u, 0u};
        float best_z[4] = {-INFINITY, -INFINITY, -INFINITY, -INFINITY};
        for (int ci = 0; ci < 9; ++ci) {
            const uint32_t id = nb[ci];
            bool seen = id == 0u;
            for (int j = 0; j < ci; ++j) seen = seen || nb[j] == id;
            if (seen) continue;  // candidates: distinct triangles in neighbourhood order
            const int slot = sub_find(s_keys, id);
            const SubTri g = slot >= 0 ? s_geo[slot] : sub_triangle(P, id, hw, hh);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float sx = (float)x + ((k & 1) ? 0.75f : 0.25f), sy = (float)y + ((k >> 1) ? 0.75f : 0.25f);
                bool inside;
                float z;
                if (!g.valid) {  // a vertex behind the eye: only the pixel's own triangle, behind every other
                    inside = id == own;
                    z = -3.0e38f;
                } else {
                    const float e0 = (g.X[2] - g.X[1]) * (sy - g.Y[1]) - (g.Y[2] - g.Y[1]) * (sx - g.X[1]);
                    const float e1 = (g.X[0] - g.X[2]) * (sy - g.Y[2]) - (g.Y[0] - g.Y[2]) * (sx - g.X[2]);
                    const float e2 = (g.X[1] - g.X[0]) * (sy - g.Y[0]) - (g.Y[1] - g.Y[0]) * (sx - g.X[0]);
                    inside = g.inv_area != 0.0f &&
                             ((e0 >= 0.0f && e1 >= 0.0f && e2 >= 0.0f) || (e0 <= 0.0f && e1 <= 0.0f && e2 <= 0.0f));
                    z = ((e0 * g.Z[0] + e1 * g.Z[1]) + e2 * g.Z[2]) * g.inv_area;
                }
                if (inside && z > best_z[k]) {
                    best[k] = id;
                    best_z[k] = z;
                }
            }
        }
        mask = 0u;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            // sources of point k: own, horizontal, vertical and diagonal neighbour (the 3x3 entries)
            const int hx = (k & 1) ? 2 : 0, vy = (k >> 1) ? 2 : 0;
            const uint32_t src[4] = {own, nb[3 + hx], nb[vy * 3 + 1], nb[vy * 3 + hx]};
#pragma unroll
            for (int s = 0; s < 4; ++s)
                if (src[s] == best[k]) mask |= 1u << (4 * k + s);
        }
    }
    VR.gb_sources[(size_t)y * W + x] = (uint16_t)mask;
}

void launch_subpixel_sources(const ShadeParams& p, cudaStream_t stream) {
    if (p.shade_blocks == 0 || p.samples > 1) return;
    k_subpixel_sources<<<p.shade_blocks, dim3(16, 16), 0, stream>>>(p);
    note_launch();
}

// ---------------------------------------------------------------------------
// blended list
// ---------------------------------------------------------------------------

// One CTA per 16x16 tile. The blended records overlapping the tile are
// compacted into shared memory in submission order, then every pixel walks
// them in that order: coverage with the raster's integer edge test, the
// GREATER_OR_EQUAL test against the opaque depth (no write), fragmentMain
// (discard honoured), and SRC_ALPHA / ONE_MINUS_SRC_ALPHA on colour, ONE / ZERO
// on alpha, rounded to the RGBA16F draw image after each blend
// (src/Engine/Graphics.cpp:5654-5691). Then the sRGB blit.
constexpr int kBlendBatch = 1024;

// Ordered compaction of the items [start, min(start + kBlendBatch, n)) that `hit`
// selects (4 consecutive items per thread) into s_list, in item order; returns
// their count. Every thread of the 256-thread CTA calls it.
template <class Hit>
__device__ __forceinline__ uint32_t compact_batch(uint32_t start, uint32_t n, int tid, uint32_t* s_list,
                                                  uint32_t* s_count, Hit hit) {
    const int lane = tid & 31, warp = tid >> 5;
    uint32_t mask = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const uint32_t r = start + 4 * tid + k;
        if (r < n && hit(r)) mask |= 1u << k;
    }
    const uint32_t cnt = __popc(mask);
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    __syncthreads();
    if (lane == 31) s_count[warp] = incl;
    __syncthreads();
    uint32_t base = 0, total = 0;
    for (int w = 0; w < 8; ++w) {
        if (w < warp) base += s_count[w];
        total += s_count[w];
    }
    uint32_t pos = base + incl - cnt;
#pragma unroll
    for (int k = 0; k < 4; ++k)
        if (mask & (1u << k)) s_list[pos++] = start + 4 * tid + k;
    __syncthreads();
    return total;
}

// Whether the 5-pixel line `s` covers the sample at (PX, PY) (1/256 pixel), and
// its depth there: the rectangle 0 <= along < |d|^2, -(w/2)|d| < perp <= (w/2)|d|
// in exact integers; depth fma(along/|d|^2, z1 - z0, z0) clamped to [0, 1].
__device__ __forceinline__ bool debug_covers(const DebugSeg& s, int32_t PX, int32_t PY, float& z) {
    const long long dx = (long long)s.X1 - s.X0, dy = (long long)s.Y1 - s.Y0;
    const long long len2 = dx * dx + dy * dy;
    if (len2 == 0) return false;
    const long long ex = (long long)PX - s.X0, ey = (long long)PY - s.Y0;
    const long long along = ex * dx + ey * dy;
    if (along < 0 || along >= len2) return false;
    const long long perp = dx * ey - dy * ex;
    const __int128 lhs = (__int128)perp * perp, rhs = (__int128)kDebugHalfWidth2 * len2;
    if (perp >= 0 ? lhs > rhs : lhs >= rhs) return false;
    const float t = (float)along / (float)len2;
    float zz = fmaf(t, s.z1 - s.z0, s.z0);
    if (!(zz > 0.0f)) zz = 0.0f;
    if (zz > 1.0f) zz = 1.0f;
    z = zz;
    return true;
}

__global__ void __launch_bounds__(256) k_blend(BlendParams B) {
    __shared__ float s_srgb[256];
    __shared__ uint32_t s_list[kBlendBatch];
    __shared__ uint32_t s_count[256 / 32 + 1];
    __shared__ uint32_t s_view;
    const ShadeParams& P = B.sh;
    const int tid = threadIdx.y * blockDim.x + threadIdx.x;
    s_srgb[tid] = P.srgb_table[tid];
    if (tid == 0) s_view = tile_view(P.views, P.view_count, blockIdx.x + P.block_offset);
    __syncthreads();
    const uint32_t view = s_view;
    const ViewRec& VR = P.views[view];
    const uint32_t lt = blockIdx.x + P.block_offset - VR.shade_block_base;
    const uint32_t tiles_x = ((uint32_t)VR.width + 15) / 16;
    const int tx0 = (int)(lt % tiles_x) * 16, ty0 = (int)(lt / tiles_x) * 16;
    const int px = tx0 + threadIdx.x, py = ty0 + threadIdx.y;
    const bool inside = px < VR.width && py < VR.height;
    const size_t p = inside ? (size_t)py * VR.width + px : 0;
    const size_t plane = (size_t)VR.width * VR.height;
    const int nsamples = VR.samples > 1 ? kMsaaSamples : 1;
    // per coverage sample: the RGBA16F value and the opaque depth it is tested against
    float col[kMsaaSamples][4];
    float dst_depth[kMsaaSamples];
#pragma unroll
    for (int k = 0; k < kMsaaSamples; ++k) {
        dst_depth[k] = 0.f;
#pragma unroll
        for (int i = 0; i < 4; ++i) col[k][i] = 0.f;
        if (inside && k < nsamples) {
            const uint2 c = VR.color16[p + k * plane];
            const __half2 rg = *reinterpret_cast<const __half2*>(&c.x), ba = *reinterpret_cast<const __half2*>(&c.y);
            col[k][0] = __low2float(rg);
            col[k][1] = __high2float(rg);
            col[k][2] = __low2float(ba);
            col[k][3] = __high2float(ba);
            dst_depth[k] = nsamples > 1 ? __uint_as_float((uint32_t)(VR.vis[p + k * plane] >> 32)) : VR.depth[p];
        }
    }
    const Sampler smp{&P, s_srgb};
    // a pass whose look-back gave up has records at unreliable slots: blend none of them
    const bool records_ok = !B.error_flags || !(*B.error_flags & kErrLookbackTimeout);
    const uint32_t n = records_ok ? min(B.header->records, B.record_capacity) : 0u;
    const int lane = tid & 31, warp = tid >> 5;
    for (uint32_t start = 0; start < n; start += kBlendBatch) {
        // ordered compaction of the records whose box meets this tile (4 per thread)
        uint32_t mask = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t r = start + 4 * tid + k;
            if (r < n) {
                const TriRecord& rec = B.records[r];
                const int bx0 = rec.p0 & 0xffff, by0 = rec.p0 >> 16, bx1 = rec.p1 & 0xffff, by1 = rec.p1 >> 16;
                if ((rec.view & kViewMask) == view && bx1 >= tx0 && bx0 <= tx0 + 15 && by1 >= ty0 && by0 <= ty0 + 15)
                    mask |= 1u << k;
            }
        }
        const uint32_t cnt = __popc(mask);
        uint32_t incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += v;
        }
        __syncthreads();
        if (lane == 31) s_count[warp] = incl;
        __syncthreads();
        uint32_t base = 0, total = 0;
        for (int w = 0; w < 8; ++w) {
            if (w < warp) base += s_count[w];
            total += s_count[w];
        }
        uint32_t pos = base + incl - cnt;
#pragma unroll
        for (int k = 0; k < 4; ++k)
            if (mask & (1u << k)) s_list[pos++] = start + 4 * tid + k;
        __syncthreads();
        if (inside) {
            for (uint32_t j = 0; j < total; ++j) {
                const TriRecord& rec = B.records[s_list[j]];
                const int bx0 = rec.p0 & 0xffff, by0 = rec.p0 >> 16, bx1 = rec.p1 & 0xffff, by1 = rec.p1 >> 16;
                if (px < bx0 || px > bx1 || py < by0 || py > by1) continue;
                const int32_t X[3] = {rec.X0, rec.X1, rec.X2}, Y[3] = {rec.Y0, rec.Y1, rec.Y2};
                uint32_t pass = 0;  // samples covered and in front of the opaque depth
                for (int k = 0; k < nsamples; ++k) {
                    const int32_t PX = px * 256 + (nsamples > 1 ? msaa_x(k) : 128);
                    const int32_t PY = py * 256 + (nsamples > 1 ? msaa_y(k) : 128);
                    bool in = true;
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        const int a = (i + 1) % 3, b = (i + 2) % 3;
                        const int32_t dx = X[b] - X[a], dy = Y[b] - Y[a];
                        const bool tl = dy < 0 || (dy == 0 && dx > 0);
                        const int64_t E = (int64_t)dx * (int64_t)(PY - Y[a]) - (int64_t)dy * (int64_t)(PX - X[a]);
                        in = in && (E > 0 || (E == 0 && tl));
                    }
                    if (!in) continue;
                    float z = fmaf(rec.dzdx, (float)(PX - rec.X0), fmaf(rec.dzdy, (float)(PY - rec.Y0), rec.z0));
                    if (!(z > 0.0f)) z = 0.0f;
                    if (z > 1.0f) z = 1.0f;
                    if (z >= dst_depth[k]) pass |= 1u << k;
                }
                if (!pass) continue;
                float s4[4];
                if (!shade_pixel(P, VR, *VR.scene, smp, rec.id - 1u, px, py, s4)) continue;
                const float a = s4[3];
#pragma unroll
                for (int k = 0; k < kMsaaSamples; ++k) {
                    if (!(pass & (1u << k))) continue;
#pragma unroll
                    for (int i = 0; i < 3; ++i) col[k][i] = half_round(s4[i] * a + col[k][i] * (1.0f - a));
                    col[k][3] = half_round(a);
                }
            }
        }
        __syncthreads();
    }
    // Debug-line overlay after the blended list (src/Engine/Graphics.cpp:5694-5738): the same
    // blend state and depth test, depth writes off; a covered sample in front of the opaque
    // depth takes the line's colour (SRC_ALPHA with alpha 1 keeps only the source).
    if (B.debug_count) {
        const DebugSeg* __restrict__ segs = B.debug + (size_t)view * B.debug_count;
        for (uint32_t start = 0; start < B.debug_count; start += kBlendBatch) {
            const uint32_t total = compact_batch(start, B.debug_count, tid, s_list, s_count, [&](uint32_t r) {
                const DebugSeg& sg = segs[r];
                const int bx0 = sg.p0 & 0xffff, by0 = sg.p0 >> 16, bx1 = sg.p1 & 0xffff, by1 = sg.p1 >> 16;
                return sg.live && bx1 >= tx0 && bx0 <= tx0 + 15 && by1 >= ty0 && by0 <= ty0 + 15;
            });
            if (inside) {
                for (uint32_t j = 0; j < total; ++j) {
                    const DebugSeg& sg = segs[s_list[j]];
                    const int bx0 = sg.p0 & 0xffff, by0 = sg.p0 >> 16, bx1 = sg.p1 & 0xffff, by1 = sg.p1 >> 16;
                    if (px < bx0 || px > bx1 || py < by0 || py > by1) continue;
                    uint32_t pass = 0;  // samples covered and in front of the opaque depth
                    for (int k = 0; k < nsamples; ++k) {
                        const int32_t PX = px * 256 + (nsamples > 1 ? msaa_x(k) : 128);
                        const int32_t PY = py * 256 + (nsamples > 1 ? msaa_y(k) : 128);
                        float z;
                        if (debug_covers(sg, PX, PY, z) && z >= dst_depth[k]) pass |= 1u << k;
                    }
                    if (!pass) continue;
#pragma unroll
                    for (int k = 0; k < kMsaaSamples; ++k) {
                        if (!(pass & (1u << k))) continue;
#pragma unroll
                        for (int i = 0; i < 3; ++i) col[k][i] = half_round(sg.rgb[i]);
                        col[k][3] = 1.0f;
                    }
                }
            }
            __syncthreads();
        }
    }
    if (!inside) return;
    float o[4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
        o[i] = nsamples > 1 ? resolve4(col[0][i], col[1][i], col[2][i], col[3][i]) : col[0][i];
    VR.color[p] = encode_srgb8(o[0]) | (encode_srgb8(o[1]) << 8) | (encode_srgb8(o[2]) << 16) | (encode_unorm8(o[3]) << 24);
}

void launch_blend(const BlendParams& p, cudaStream_t stream) {
    if (p.sh.shade_blocks == 0) return;
    k_blend<<<p.sh.shade_blocks, dim3(16, 16), 0, stream>>>(p);
    note_launch();
}

}  // namespace rz
