// Learned upsampler: a W x H G-buffer (colour, depth, albedo, normal) to a
// 2W x 2H RGBA8 sRGB frame, trained and run with this file's own kernels.
//
// Network: four 3x3 convolutions (zero padding) 16 -> 32 -> 32 -> 32 -> 12
// channels, ReLU after the first three; the 12 output channels are the 2x2
// sub-pixels (s = 2 i + j for full-resolution pixel (2x + j, 2y + i)) times RGB,
// added to the bilinear x2 upsampling of the input colour. Weights and
// activations are BF16, accumulation FP32.
//
// Every convolution is an implicit GEMM on the 5th-generation tensor cores
// (tcgen05.mma, kind::f16, M = 128, accumulators in tensor memory):
//   forward / input gradient:  D[pixel, cout] = sum over (tap, cin) of
//     X[pixel + offset(tap), cin] * W[cout, tap, cin]
//   One CTA owns a 128-pixel x 4-row output tile. It stages the input halo (6
//   rows x 130 pixels) in shared memory once, as one plane per group of 8
//   channels with each pixel's 8 channels in 16 bytes; a tap's A operand is the
//   same planes at a start address shifted by whole pixels (16 bytes), so no
//   im2col copy is made. The input gradient is the same kernel with the
//   weights transposed and the taps mirrored.
//   weight gradient: D[(tap, cin), cout] = sum over pixels of
//     X[pixel + offset(tap), cin] * dY[pixel, cout]
//   One persistent CTA per half SM walks 64-pixel x 4-row tiles; it stages X
//   transposed (8 pixels of one channel per 16 bytes) for the three horizontal
//   shifts, laid out so that the (tap, channel) rows of an M block sit at a
//   uniform stride, and accumulates D in tensor memory over all its tiles.
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// 8 x 16-byte core matrices; the descriptor's leading byte offset is the
// distance between core matrices along K and the stride byte offset the
// distance between 8-row groups along M (or N).
//
// Every wait on a copy or tensor-core completion barrier has a time limit
// (about a second; rz_upsampler_set_wait_limit can shorten it); a wait that runs
// out sets kErrMmaTimeout and skips the rest of the kernel's work. Before the CTA
// frees its tensor memory and returns, the thread that issued TMA copies waits
// (with the full limit again) for the copies it has in flight, and the thread
// that issued MMAs for its last commit.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "rz_internal.h"

namespace rz {
namespace up {

constexpr int kThreads = 128;      // weight-gradient and self-test kernels
constexpr int kConvEpilogueWarps = 16;  // convolution: one epilogue warp per (TMEM lane quadrant, tile row),
constexpr int kConvThreads = 32 * (kConvEpilogueWarps + 2);  // then a TMA warp and an MMA warp
constexpr int kTileW = 128;  // conv: MMA rows (M = 128), one row segment of output pixels
constexpr int kTileRows = 4; // conv: output rows per tile (8 measured 4% slower)
constexpr int kConvStages = 4; // conv: halo buffers in flight (TMA loads ahead of the MMAs)
// conv: pixels of one halo row = one TMA box of 256 8-byte elements (2,048 bytes, the
// largest box); a tile row yields kTileOut valid outputs, and MMA rows kTileOut and
// kTileOut + 1 (whose 3x3 window runs past the halo) are computed and dropped
constexpr int kHaloW = kTileW;
constexpr int kTileOut = kHaloW - 2;
constexpr int kWgKP = 64;    // weight gradient: pixels per tile row (K chunk)
constexpr int kWgRows = 4;   // weight gradient: rows per tile
constexpr long long kWaitCycles = 2000000000ll;  // about one second at 2 GHz
constexpr uint32_t kErrMmaTimeout = 1u << 0;

enum { kEpiRelu = 0, kEpiMask = 1, kEpiFinal = 2 };

// Parameter layout: per layer weights [cout][9][cin] then biases [cout].
__host__ __device__ constexpr int layer_cin(int l) { return l == 0 ? 16 : 32; }
__host__ __device__ constexpr int layer_cout(int l) { return l == 3 ? 16 : 32; }
__host__ __device__ constexpr int layer_wcount(int l) { return 9 * layer_cin(l) * layer_cout(l); }
__host__ __device__ constexpr int layer_woff(int l) {
    return l == 0 ? 0 : layer_woff(l - 1) + layer_wcount(l - 1) + layer_cout(l - 1);
}
__host__ __device__ constexpr int layer_boff(int l) { return layer_woff(l) + layer_wcount(l); }
constexpr int kParamCount = layer_boff(3) + layer_cout(3);
static_assert(kParamCount == (int)RZ_UPSAMPLER_PARAM_COUNT, "parameter count");
// BF16 operand images: forward for layers 0..3, input gradient for layers 1..3.
__host__ __device__ constexpr int fwd_img_off(int l) { return l == 0 ? 0 : fwd_img_off(l - 1) + layer_wcount(l - 1); }
__host__ __device__ constexpr int dgrad_img_off(int l) {
    return l == 1 ? fwd_img_off(3) + layer_wcount(3) : dgrad_img_off(l - 1) + layer_wcount(l - 1);
}
constexpr int kImgCount = dgrad_img_off(3) + layer_wcount(3);
constexpr int kOutChannels = 12;
constexpr int kFeatChannels = 16;

// ---- PTX helpers ------------------------------------------------------------

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory matrix descriptor, no swizzle.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;  // descriptor version 1 (tcgen05)
    return d;                 // base offset 0, absolute LBO mode, layout type 0 = no swizzle
}

// Instruction descriptor, kind::f16: D f32, A and B bf16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate));
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Waits for the barrier phase of `parity`; false if `limit` clock cycles ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, long long limit = kWaitCycles) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity)) {
        if (clock64() - t0 > limit) return false;
    }
    return true;
}

__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t cols) {  // one full warp
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(slot)), "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t cols) {  // one full warp
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols) : "memory");
}

// 16-byte asynchronous global -> shared copy; valid == false writes zeros (src must still be a mapped address).
__device__ __forceinline__ void cp_async16(void* dst, const void* src, bool valid) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(dst)), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int kPending>
__device__ __forceinline__ void cp_async_wait_group() {
    asm volatile("cp.async.wait_group %0;" ::"n"(kPending) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// 16 consecutive f32 columns of the warp's 32 lanes (one lane per thread).
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 32 consecutive f32 columns of the warp's 32 lanes.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Writes zeros to `cols` (a multiple of 16) columns of this warp's 32 TMEM lanes from
// taddr on, and waits until the stores have landed.
__device__ __forceinline__ void tmem_zero(uint32_t taddr, int cols) {
    const uint32_t z = 0u;
    for (int c = 0; c < cols; c += 16)
        asm volatile(
            "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
            "{%1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1, %1};" ::"r"(taddr + c), "r"(z)
            : "memory");
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}

__host__ __device__ constexpr uint32_t tmem_cols_for(int cols) {
    return cols <= 32 ? 32u : cols <= 64 ? 64u : cols <= 128 ? 128u : cols <= 256 ? 256u : 512u;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&h);
}
__device__ __forceinline__ float bf16_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t v) { return __uint_as_float(v & 0xFFFF0000u); }

// Activations are stored planar by groups of 8 channels: [C / 8][H][W][8] bf16,
// so a TMA box of one channel group over a row of pixels is one contiguous run.
__device__ __forceinline__ size_t act_index(int W, int H, int x, int y, int c) {
    return (((size_t)(c >> 3) * H + y) * W + x) * 8 + (c & 7);
}

// ---- features -----------------------------------------------------------------

// One pixel's 16 input channels from the G-buffer (see rz_upsampler_* in the header).
// byte / 255, correctly rounded: the product with the rounded reciprocal and one
// residual-correction step (Markstein's method), which gives the correctly rounded
// quotient for every byte value (checked exhaustively against IEEE division).
__device__ __forceinline__ float unorm8(uint32_t b) {
    const float x = (float)b, r = 1.0f / 255.0f;
    const float q = x * r;
    return __fmaf_rn(__fmaf_rn(-q, 255.0f, x), r, q);
}

// Sum of the bilinear x2 weights of a sample point's marked sources: own pixel
// 9/16, horizontal and vertical neighbour 3/16 each, diagonal 1/16.
__device__ __forceinline__ float matched_weight(uint32_t m4) {
    float ws = 0.0f;
    if (m4 & 1u) ws = ws + 0.5625f;
    if (m4 & 2u) ws = ws + 0.1875f;
    if (m4 & 4u) ws = ws + 0.1875f;
    if (m4 & 8u) ws = ws + 0.0625f;
    return ws;
}

__global__ void k_features(rz_gbuffer g, __nv_bfloat16* __restrict__ feat) {
    const int n = (int)(g.width * g.height);
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t c = __ldg(static_cast<const uint32_t*>(g.color_rgba8) + i);
    const uint32_t a = __ldg(static_cast<const uint32_t*>(g.albedo_rgba8) + i);
    const uint32_t nn = __ldg(static_cast<const uint32_t*>(g.normal_oct_f16x2) + i);
    const float d = __ldg(static_cast<const float*>(g.depth_f32) + i);
    const __half2 h = *reinterpret_cast<const __half2*>(&nn);
    const float2 oct = __half22float2(h);
    float f[16];
    f[0] = unorm8(c & 255u);
    f[1] = unorm8((c >> 8) & 255u);
    f[2] = unorm8((c >> 16) & 255u);
    f[3] = unorm8(a & 255u);
    f[4] = unorm8((a >> 8) & 255u);
    f[5] = unorm8((a >> 16) & 255u);
    f[6] = oct.x;
    f[7] = oct.y;
    f[8] = unorm8(a >> 24);
    f[9] = fminf(d * 16.0f, 4.0f);
#pragma unroll
    for (int k = 10; k < 16; ++k) f[k] = 0.0f;
    if (g.sources_u16) {  // per sample point: the bilinear weight of the sources that show its triangle
        const uint32_t m = __ldg(static_cast<const uint16_t*>(g.sources_u16) + i);
#pragma unroll
        for (int k = 0; k < 4; ++k) f[10 + k] = matched_weight(m >> (4 * k));
    }
    uint4* dst0 = reinterpret_cast<uint4*>(feat + (size_t)i * 8);
    uint4* dst1 = reinterpret_cast<uint4*>(feat + (size_t)(n + i) * 8);
    *dst0 = make_uint4(pack_bf16(f[0], f[1]), pack_bf16(f[2], f[3]), pack_bf16(f[4], f[5]), pack_bf16(f[6], f[7]));
    *dst1 = make_uint4(pack_bf16(f[8], f[9]), pack_bf16(f[10], f[11]), pack_bf16(f[12], f[13]), pack_bf16(f[14], f[15]));
}

// ---- convolution (forward and input gradient) ---------------------------------

struct ConvArgs {
    const __nv_bfloat16* in;        // planar [CIN / 8][H][W][8]
    const __nv_bfloat16* wimg;      // B operand image [3 dx][CIN / 8][3 dy][N][8]
    const float* bias;              // N (relu, final)
    int W, H;
    __nv_bfloat16* out;             // planar [N / 8][H][W][8] (relu, mask)
    const __nv_bfloat16* mask_src;  // planar like out: out = acc where mask_src > 0, else 0 (mask)
    const uint32_t* color_lr;       // H x W RGBA8: bilinear base (final)
    const uint16_t* sources;        // H x W sub-pixel sources of the base, or null: plain bilinear (final)
    uint32_t* out_rgba8;            // 2H x 2W, or null (final)
    const uint32_t* target;         // 2H x 2W RGBA8, or null (final, training)
    __nv_bfloat16* dy;              // planar [2][H][W][8]: gradient of the loss sum (final, training)
    double* loss;                   // loss sum accumulator (final, training)
    uint32_t* err;
    long long wait_cycles;          // bound of each pipeline wait
};

// Shared memory of the persistent convolution: the weights (B operand) once,
// then kConvStages halo buffers (A operand) that tiles take in turn. Each halo
// buffer is (kTileRows + 2) rows x (CIN / 8) channel planes x kHaloW pixels x 16
// bytes; a plane is padded by two pixels (read by the dropped MMA rows, never
// written) and to a multiple of 128 bytes.
template <int CIN, int N>
struct ConvSmem {
    static constexpr int G = CIN / 8;
    static constexpr uint32_t S_G = ((kHaloW + 2) * 16 + 127) / 128 * 128;  // between channel planes (K direction)
    static constexpr uint32_t S_R = G * S_G;                          // between halo rows
    static constexpr uint32_t A_BYTES = (kTileRows + 2) * S_R;
    static constexpr uint32_t TX_BYTES = (kTileRows + 2) * G * kHaloW * 16;  // what one tile's TMA loads write
    static constexpr uint32_t B_BYTES = 9 * CIN * N * 2;
    static constexpr uint32_t A_OFF0 = (B_BYTES + 1023) / 1024 * 1024;
    static constexpr uint32_t A_STRIDE = (A_BYTES + 1023) / 1024 * 1024;  // between halo buffers
    static constexpr uint32_t BAR_OFF = A_OFF0 + kConvStages * A_STRIDE;
    static constexpr uint32_t NBAR = 2 * kConvStages + 5;                // full, empty, tfull[2], tempty[2], weights
    static constexpr uint32_t BYTES = BAR_OFF + NBAR * 8 + 16;           // the barriers, the TMEM address
    static constexpr uint32_t ACC_COLS = (kTileRows + 4) * N;                 // one accumulator buffer
    static constexpr uint32_t TMEM_COLS = tmem_cols_for(2 * ACC_COLS);        // two of them
};
static_assert(ConvSmem<32, 32>::BYTES + 2048 <= 227 * 1024, "conv shared memory (with the static arrays)");
static_assert(2 * (kTileRows + 4) * 32 <= 512, "two accumulator buffers fit the 512 TMEM columns");
static_assert(kTileRows * 4 % kConvEpilogueWarps == 0, "epilogue warps split the tile rows evenly");
static_assert(2 * kHaloW <= 256, "a halo row is one TMA box (at most 256 elements)");
static_assert(ConvSmem<32, 32>::S_G % 128 == 0 && ConvSmem<16, 32>::S_R % 128 == 0, "TMA destinations 128-byte aligned");

template <int N, int EPI>
__device__ __forceinline__ void conv_epilogue(const ConvArgs& a, const float* acc, int x, int y, float& loss,
                                              const float* bias, int xl, const float (*srcw)[4]) {
    const bool inside = x < a.W && y < a.H;
    if (EPI == kEpiRelu) {
        if (!inside) return;
        uint32_t pk[N / 2];
#pragma unroll
        for (int c = 0; c < N / 2; ++c)
            pk[c] = pack_bf16(fmaxf(acc[2 * c] + bias[2 * c], 0.0f), fmaxf(acc[2 * c + 1] + bias[2 * c + 1], 0.0f));
#pragma unroll
        for (int q = 0; q < N / 8; ++q)
            *reinterpret_cast<uint4*>(a.out + act_index(a.W, a.H, x, y, 8 * q)) =
                make_uint4(pk[4 * q], pk[4 * q + 1], pk[4 * q + 2], pk[4 * q + 3]);
    } else if (EPI == kEpiMask) {
        if (!inside) return;
#pragma unroll
        for (int q = 0; q < N / 8; ++q) {
            const uint4 m = __ldg(reinterpret_cast<const uint4*>(a.mask_src + act_index(a.W, a.H, x, y, 8 * q)));
            const uint32_t mw[4] = {m.x, m.y, m.z, m.w};
            uint32_t o[4];
#pragma unroll
            for (int h = 0; h < 4; ++h) {
                const int c = 8 * q + 2 * h;
                o[h] = pack_bf16(bf16_lo(mw[h]) > 0.0f ? acc[c] : 0.0f, bf16_hi(mw[h]) > 0.0f ? acc[c + 1] : 0.0f);
            }
            *reinterpret_cast<uint4*>(a.out + act_index(a.W, a.H, x, y, 8 * q)) = make_uint4(o[0], o[1], o[2], o[3]);
        }
    } else {  // final: pixel shuffle + x2 base (+ loss gradient)
        const int W = a.W, H = a.H;
        // The 3x3 neighbourhood of low-resolution colours (edges clamped), as byte / 255.
        // The warp's lanes hold consecutive columns xl (the tile's dropped MMA rows
        // included, clamped), so each lane loads and converts its own column of the
        // three rows and takes its left and right neighbours' from the adjacent lanes;
        // lanes 0 and 31 load the column past the warp's edge. Every lane takes part
        // (the shuffles), then lanes outside the image return.
        const int lane = threadIdx.x & 31;
        const int xo = min(max(xl, 0), W - 1);
        const int xe = min(max(lane == 0 ? xl - 1 : xl + 1, 0), W - 1);
        const bool edge_lane = lane == 0 || lane == 31;
        float f[3][3][3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const int yy = min(max(y + r - 1, 0), H - 1);
            const uint32_t c = __ldg(a.color_lr + (size_t)yy * W + xo);
            const uint32_t ce = edge_lane ? __ldg(a.color_lr + (size_t)yy * W + xe) : 0u;
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float own = unorm8((c >> (8 * k)) & 255u);
                const float ext = edge_lane ? unorm8((ce >> (8 * k)) & 255u) : 0.0f;
                const float lv = __shfl_up_sync(0xFFFFFFFFu, own, 1), rv = __shfl_down_sync(0xFFFFFFFFu, own, 1);
                f[r][0][k] = lane == 0 ? ext : lv;
                f[r][1][k] = own;
                f[r][2][k] = lane == 31 ? ext : rv;
            }
        }
        if (!inside) return;
        float net[kOutChannels];
#pragma unroll
        for (int c = 0; c < kOutChannels; ++c) net[c] = acc[c] + bias[c];
        const uint32_t srcmask = a.sources ? (uint32_t)__ldg(a.sources + (size_t)y * W + x) : 0xFFFFu;
        float g[kOutChannels];
#pragma unroll
        for (int i = 0; i < 2; ++i) {
            const int rs = i == 0 ? 0 : 2;
            const size_t op = (size_t)(2 * y + i) * (2 * W) + 2 * x;
            uint2 t = make_uint2(0u, 0u);
            if (a.target) t = __ldg(reinterpret_cast<const uint2*>(a.target + op));
            uint32_t o[2];
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const int qs = j == 0 ? 0 : 2;
                const uint32_t tj = j == 0 ? t.x : t.y;
                uint32_t ov = 255u << 24;
                // the weights of this point's sources (own, horizontal, vertical, diagonal) for
                // its source mask: bilinear renormalised over the sources that show its triangle
                const uint32_t m4 = (srcmask >> (4 * (2 * i + j))) & 15u;
                const float w0 = srcw[m4][0], w1 = srcw[m4][1], w2 = srcw[m4][2], w3 = srcw[m4][3];
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    float base = w0 * f[1][1][k];
                    base = base + w1 * f[1][qs][k];
                    base = base + w2 * f[rs][1][k];
                    base = base + w3 * f[rs][qs][k];
                    const float v = base + net[(2 * i + j) * 3 + k];
                    const float qv = fminf(fmaxf(v, 0.0f), 1.0f);
                    ov |= (uint32_t)floorf(qv * 255.0f + 0.5f) << (8 * k);
                    if (a.target) {
                        const float d = v - unorm8((tj >> (8 * k)) & 255u);
                        g[(2 * i + j) * 3 + k] = 2.0f * d;
                        loss += d * d;
                    }
                }
                o[j] = ov;
            }
            if (a.out_rgba8) *reinterpret_cast<uint2*>(a.out_rgba8 + op) = make_uint2(o[0], o[1]);
        }
        if (a.target) {
            *reinterpret_cast<uint4*>(a.dy + act_index(W, H, x, y, 0)) =
                make_uint4(pack_bf16(g[0], g[1]), pack_bf16(g[2], g[3]), pack_bf16(g[4], g[5]), pack_bf16(g[6], g[7]));
            *reinterpret_cast<uint4*>(a.dy + act_index(W, H, x, y, 8)) =
                make_uint4(pack_bf16(g[8], g[9]), pack_bf16(g[10], g[11]), 0u, 0u);
        }
    }
}

// TMA load of one box {256 8-byte elements = kHaloW pixels x 8 channels, 1 row,
// 1 channel group} of a planar [C / 8][H][W][8] bf16 tensor (viewed as rows of
// 2 W 8-byte elements) into shared memory, completing on `bar` with its byte
// count. x is in 8-byte elements and even (16-byte aligned), possibly negative.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y, int g) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4, %5}], [%2];" ::
            "r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(x), "r"(y), "r"(g)
        : "memory");
}

// Untiled bulk copy of `bytes` (a multiple of 16, both addresses 16-byte aligned)
// from global to shared memory, completing on `bar` with its byte count.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
                     "r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// Persistent, warp-specialised convolution. CTA b takes tiles b, b + grid, ...
// (128 pixels x kTileRows rows each) through a ring of kConvStages halo buffers
// and two TMEM accumulators:
//   warp 16 (one thread) TMA-loads tile j's halo into halo buffer j % kConvStages
//                        once the MMAs of tile j - kConvStages have released it
//                        (barrier `empty`);
//   warp 17 (one thread) waits for the halo (`full`) and for the epilogue of
//                        tile j - 2 to have drained accumulator buffer j % 2
//                        (`tempty`), issues the tile's tcgen05.mma and commits to
//                        `empty` and `tfull`;
//   warps 0-15           wait for `tfull`, read the accumulator (warp w reads
//                        TMEM lane quadrant w % 4 of tile row w / 4), zero it,
//                        run the epilogue and arrive on `tempty`.
// One MMA takes one halo row i, one horizontal tap dx and 16 input channels, and
// N = 3 x Cout weight columns: the three vertical taps at once. Its three column
// blocks add halo row i's contributions to output rows i, i - 1 and i - 2, so the
// accumulator of output row o (-2 <= o <= kTileRows + 1) sits at column
// Cout x (kTileRows + 1 - o) and the blocks of consecutive rows are adjacent in
// the order an MMA writes them. Rows outside 0..kTileRows - 1 collect the halo
// rows' unused contributions and are never read; the others are zeroed by the
// epilogue (and once at the start), and every MMA accumulates. Each activation
// read from shared memory thus feeds 96 weight columns instead of 32.
// Every wait is bounded; a role whose wait runs out sets kErrMmaTimeout and
// stops, and the others then run out in turn.
template <int CIN, int N, int EPI>
__global__ void __launch_bounds__(kConvThreads, 1) k_conv(ConvArgs a, const __grid_constant__ CUtensorMap in_map) {
    using L = ConvSmem<CIN, N>;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sB = smem;
    constexpr int NS = kConvStages;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + L::BAR_OFF);  // [NS]
    uint64_t* empty = full + NS;                                       // [NS]
    uint64_t* tfull = full + 2 * NS;                                   // [2]
    uint64_t* tempty = tfull + 2;                                      // [2]
    uint64_t* wbar = tfull + 4;                                        // the weights have landed
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L::BAR_OFF + L::NBAR * 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int tiles_x = (a.W + kTileOut - 1) / kTileOut;
    const int ntiles = tiles_x * ((a.H + kTileRows - 1) / kTileRows);
    const int my_tiles = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;

    __shared__ float s_bias[N];
    __shared__ float s_srcw[16][4];  // final layer: the x2 base's source weights for each source mask
    if (warp == 0) tmem_alloc(tmem_slot, L::TMEM_COLS);
    if (tid == 0) {
        for (int b = 0; b < NS; ++b) {
            mbar_init(&full[b], 1);
            mbar_init(&empty[b], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], kConvEpilogueWarps);
        }
        mbar_init(wbar, 1);
    }
    if (tid < N) s_bias[tid] = EPI == kEpiMask ? 0.0f : a.bias[tid];
    if (EPI == kEpiFinal && tid < 64) {
        // mask m keeps the bilinear sources of its set bits, each weight times 1 / (their sum);
        // no bit set is plain bilinear (as is every bit set: the sum is 1)
        const uint32_t m = (uint32_t)tid >> 2, s = (uint32_t)tid & 3u;
        const float w = s == 0 ? 0.5625f : (s == 3 ? 0.0625f : 0.1875f);
        s_srcw[m][s] = m == 0u ? w : (((m >> s) & 1u) ? w * (1.0f / matched_weight(m)) : 0.0f);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    if (warp < kConvEpilogueWarps) {  // the read accumulator rows of both buffers start at zero
        const int quad = warp & 3, row0 = (warp >> 2) * (kTileRows * 4 / kConvEpilogueWarps);
        for (int b = 0; b < 2; ++b)
            for (int tt = 0; tt < kTileRows * 4 / kConvEpilogueWarps; ++tt)
                tmem_zero(tmem + ((uint32_t)(quad * 32) << 16) + b * L::ACC_COLS + (kTileRows + 1 - (row0 + tt)) * N, N);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    bool ok = true;
    float loss = 0.0f;

    if (warp == kConvEpilogueWarps && lane == 0) {
        // producer: the weights once (one bulk copy), then the TMA loads of each tile's halo
        mbar_expect_tx(wbar, L::B_BYTES);
        bulk_load(sB, a.wimg, L::B_BYTES, wbar);
        int issued = 0;
        for (int j = 0; j < my_tiles && ok; ++j) {
            const int buf = j % NS;
            if (j >= NS && !mbar_wait(&empty[buf], (uint32_t)((j - NS) / NS) & 1u, a.wait_cycles)) {
                ok = false;
                break;
            }
            const int tile = blockIdx.x + j * gridDim.x;
            const int x0 = (tile % tiles_x) * kTileOut, y0 = (tile / tiles_x) * kTileRows;
            unsigned char* A = smem + L::A_OFF0 + buf * L::A_STRIDE;
            mbar_expect_tx(&full[buf], L::TX_BYTES);
            for (int r = 0; r < kTileRows + 2; ++r)
#pragma unroll
                for (int g = 0; g < L::G; ++g)
                    tma_load_3d(A + r * L::S_R + g * L::S_G, &in_map, &full[buf], 2 * (x0 - 1), y0 - 1 + r, g);
            issued = j + 1;
        }
        // the copies still in flight (the last NS tiles issued, and the weights) land
        // before the CTA exits; a buffer's barrier cannot have moved past these phases
        for (int j = issued - NS > 0 ? issued - NS : 0; j < issued; ++j)
            if (!mbar_wait(&full[j % NS], (uint32_t)(j / NS) & 1u)) ok = false;
        if (!mbar_wait(wbar, 0)) ok = false;
    } else if (warp == kConvEpilogueWarps + 1 && lane == 0) {
        // MMA issue
        constexpr uint32_t idesc = idesc_bf16(128, 3 * N);
        constexpr uint32_t lbo_b = 3 * N * 16;  // between the weight image's 8-channel groups
        const uint64_t db0 = umma_desc(smem_u32(sB), lbo_b, 128);
        if (my_tiles > 0 && !mbar_wait(wbar, 0, a.wait_cycles)) ok = false;
        int committed = 0;
        for (int j = 0; j < my_tiles && ok; ++j) {
            const int buf = j % NS, acc = j & 1;
            if (!mbar_wait(&full[buf], (uint32_t)(j / NS) & 1u, a.wait_cycles) ||
                (j >= 2 && !mbar_wait(&tempty[acc], (uint32_t)((j - 2) >> 1) & 1u, a.wait_cycles))) {
                ok = false;
                break;
            }
            tc_fence_after();
            // descriptors differ only in their start address (the low 14 bits, in 16-byte units), so each
            // MMA's descriptors are the tile's base descriptors plus a compile-time offset
            const uint64_t da0 = umma_desc(smem_u32(smem + L::A_OFF0 + buf * L::A_STRIDE), L::S_G, 128);
            const uint32_t d0 = tmem + acc * L::ACC_COLS;
#pragma unroll
            for (int i = 0; i < kTileRows + 2; ++i) {
#pragma unroll
                for (int dx = 0; dx < 3; ++dx) {
#pragma unroll
                    for (int s = 0; s < CIN / 16; ++s) {
                        const uint32_t oa = (i * L::S_R + dx * 16 + 2 * s * L::S_G) >> 4;
                        const uint32_t ob = ((dx * L::G + 2 * s) * lbo_b) >> 4;
                        mma_bf16(d0 + (kTileRows + 1 - i) * N, da0 + oa, db0 + ob, idesc, 1u);
                    }
                }
            }
            mma_commit(&empty[buf]);
            mma_commit(&tfull[acc]);
            committed = j + 1;
        }
        // the MMAs issued complete before the CTA frees its tensor memory: the last
        // commit tracks every earlier one
        if (committed > 0 && !mbar_wait(&empty[(committed - 1) % NS], (uint32_t)((committed - 1) / NS) & 1u))
            ok = false;
    } else if (warp < kConvEpilogueWarps) {
        const int quad = warp & 3, row0 = (warp >> 2) * (kTileRows * 4 / kConvEpilogueWarps);
        // the biases live in registers: shared-memory reads would queue behind the MMAs' operand traffic
        float bias[N];
#pragma unroll
        for (int c = 0; c < N; ++c) bias[c] = s_bias[c];
        for (int j = 0; j < my_tiles; ++j) {
            const int buf = j & 1;
            // one decision per warp: the epilogue's TMEM loads and shuffles are warp-wide
            if (!__all_sync(0xFFFFFFFFu, mbar_wait(&tfull[buf], (uint32_t)(j >> 1) & 1u, a.wait_cycles))) {
                ok = false;
                break;
            }
            tc_fence_after();
            const int tile = blockIdx.x + j * gridDim.x;
            const int x0 = (tile % tiles_x) * kTileOut, y0 = (tile / tiles_x) * kTileRows;
            const int col = quad * 32 + lane;
            const int x = col < kTileOut ? x0 + col : a.W;  // the dropped MMA rows count as outside the image
#pragma unroll
            for (int tt = 0; tt < kTileRows * 4 / kConvEpilogueWarps; ++tt) {
                const int t = row0 + tt;
                float acc[N];
                const uint32_t ta = tmem + ((uint32_t)(quad * 32) << 16) + buf * L::ACC_COLS + (kTileRows + 1 - t) * N;
                if constexpr (N == 32) tmem_ld32(ta, acc);
                else tmem_ld16(ta, acc);
                tmem_zero(ta, N);
                conv_epilogue<N, EPI>(a, acc, x, y0 + t, loss, bias, x0 + col, s_srcw);
            }
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[buf]);
        }
    }
    if (!ok) atomicOr(a.err, kErrMmaTimeout);
    if (EPI == kEpiFinal && a.target && warp < kConvEpilogueWarps) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) loss += __shfl_xor_sync(0xFFFFFFFFu, loss, o);
        if (lane == 0 && loss != 0.0f) atomicAdd(a.loss, (double)loss);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tmem, L::TMEM_COLS);
}

// ---- weight gradient ------------------------------------------------------------

struct WgradArgs {
    const __nv_bfloat16* x;   // planar [CIN / 8][H][W][8]: the layer's input
    const __nv_bfloat16* dy;  // planar [N / 8][H][W][8]: gradient of the loss sum w.r.t. the pre-activation output
    float* dw;                // [N][9][CIN], accumulated
    float* db;                // [N], accumulated
    int W, H;
    uint32_t* err;
    long long wait_cycles;    // bound of each wait for the previous tile's MMAs
};

template <int CIN, int N>
struct WgSmem {
    static constexpr int G = CIN / 8;
    static constexpr int NB = (9 * CIN + 127) / 128;         // M blocks of 128 (tap, channel) rows
    static constexpr uint32_t S_CG = kWgKP * 16;              // between 8-channel groups (M direction)
    static constexpr uint32_t S_KX = G * S_CG;                // between horizontal shifts
    static constexpr uint32_t S_ROW = 3 * S_KX;               // between halo rows
    static constexpr uint32_t XT_USED = (kWgRows + 2) * S_ROW;
    static constexpr uint32_t XT_READ = (kWgRows - 1) * S_ROW + 16 * NB * S_CG;  // end of the furthest M block read
    static constexpr uint32_t XT_BYTES = XT_USED > XT_READ ? XT_USED : XT_READ;
    static constexpr uint32_t S_COG = kWgKP * 16;             // between 8-channel groups of dY (N direction)
    static constexpr uint32_t S_DYROW = (N / 8) * S_COG;
    static constexpr uint32_t DY_OFF = (XT_BYTES + 127) / 128 * 128;
    static constexpr uint32_t DY_BYTES = kWgRows * S_DYROW;
    static constexpr uint32_t BAR_OFF = (DY_OFF + DY_BYTES + 127) / 128 * 128;
    static constexpr uint32_t BYTES = BAR_OFF + 16;
    static constexpr uint32_t TMEM_COLS = tmem_cols_for(NB * N);
};

template <int CIN, int N>
__global__ void __launch_bounds__(kThreads) k_wgrad(WgradArgs a) {
    using L = WgSmem<CIN, N>;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char* sX = smem;
    unsigned char* sD = smem + L::DY_OFF;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + L::BAR_OFF);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + L::BAR_OFF + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) tmem_alloc(tmem_slot, L::TMEM_COLS);
    if (tid == 0) mbar_init(bar, 1);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const int tiles_x = (a.W + kWgKP - 1) / kWgKP, tiles_y = (a.H + kWgRows - 1) / kWgRows;
    const int ntiles = tiles_x * tiles_y;
    const int ci = tid % CIN, xgroups = kThreads / CIN;
    const int co = tid % N, dgroups = kThreads / N;
    float dbsum = 0.0f;
    bool ok = true;
    int iter = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++iter) {
        if (iter > 0) ok = ok && mbar_wait(bar, (uint32_t)(iter - 1) & 1u, a.wait_cycles);
        if (!__syncthreads_and(ok ? 1 : 0)) {
            ok = false;
            break;
        }
        const int x0 = (tile % tiles_x) * kWgKP, y0 = (tile / tiles_x) * kWgRows;
        // X transposed, three horizontal shifts: 16 bytes = 8 pixels of one channel
        for (int task = tid / CIN; task < (kWgRows + 2) * (kWgKP / 8); task += xgroups) {
            const int r = task / (kWgKP / 8), pxg = task % (kWgKP / 8);
            const int y = y0 - 1 + r;
            const int xs = x0 + 8 * pxg - 1;
            float v[10];
#pragma unroll
            for (int j = 0; j < 10; ++j) {
                const int x = xs + j;
                v[j] = (y >= 0 && y < a.H && x >= 0 && x < a.W)
                           ? __bfloat162float(a.x[act_index(a.W, a.H, x, y, ci)])
                           : 0.0f;
            }
#pragma unroll
            for (int kx = 0; kx < 3; ++kx) {
                const uint4 w = make_uint4(pack_bf16(v[kx], v[kx + 1]), pack_bf16(v[kx + 2], v[kx + 3]),
                                           pack_bf16(v[kx + 4], v[kx + 5]), pack_bf16(v[kx + 6], v[kx + 7]));
                *reinterpret_cast<uint4*>(sX + r * L::S_ROW + kx * L::S_KX + (ci / 8) * L::S_CG + pxg * 128 +
                                          (ci % 8) * 16) = w;
            }
        }
        // dY transposed: 16 bytes = 8 pixels of one output channel
        for (int task = tid / N; task < kWgRows * (kWgKP / 8); task += dgroups) {
            const int r = task / (kWgKP / 8), pxg = task % (kWgKP / 8);
            const int y = y0 + r;
            float v[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int x = x0 + 8 * pxg + j;
                v[j] = (y < a.H && x < a.W) ? __bfloat162float(a.dy[act_index(a.W, a.H, x, y, co)]) : 0.0f;
                dbsum += v[j];
            }
            *reinterpret_cast<uint4*>(sD + r * L::S_DYROW + (co / 8) * L::S_COG + pxg * 128 + (co % 8) * 16) =
                make_uint4(pack_bf16(v[0], v[1]), pack_bf16(v[2], v[3]), pack_bf16(v[4], v[5]), pack_bf16(v[6], v[7]));
        }
        fence_async_smem();
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
        if (tid == 0) {
            constexpr uint32_t idesc = idesc_bf16(128, N);
            const uint32_t xa = smem_u32(sX), da0 = smem_u32(sD);
            for (int r = 0; r < kWgRows; ++r) {
#pragma unroll
                for (int s = 0; s < kWgKP / 16; ++s) {
                    const uint64_t db = umma_desc(da0 + r * L::S_DYROW + s * 256, 128, L::S_COG);
                    const uint32_t accum = (iter > 0 || r > 0 || s > 0) ? 1u : 0u;
#pragma unroll
                    for (int b = 0; b < L::NB; ++b) {
                        const uint64_t dx = umma_desc(xa + r * L::S_ROW + 16 * b * L::S_CG + s * 256, 128, L::S_CG);
                        mma_bf16(tmem + b * N, dx, db, idesc, accum);
                    }
                }
            }
            mma_commit(bar);
        }
    }
    if (ok && iter > 0) ok = mbar_wait(bar, (uint32_t)(iter - 1) & 1u, a.wait_cycles);
    ok = __syncthreads_and(ok ? 1 : 0) != 0;
    // after a wait ran out, the MMAs of the last tile (committed by thread 0) still
    // complete before the tensor memory is freed
    if (!ok && tid == 0 && iter > 0) mbar_wait(bar, (uint32_t)(iter - 1) & 1u);
    tc_fence_after();
    if (ok && iter > 0) {
        for (int b = 0; b < L::NB; ++b) {
            float acc[N];
#pragma unroll
            for (int c = 0; c < N; c += 16) tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + b * N + c, acc + c);
            const int m = 128 * b + 32 * warp + lane;
            const int tap = m / CIN, c_in = m % CIN;
            if (tap < 9) {
#pragma unroll
                for (int c = 0; c < N; ++c)
                    if (acc[c] != 0.0f) atomicAdd(a.dw + ((size_t)c * 9 + tap) * CIN + c_in, acc[c]);
            }
        }
        if (dbsum != 0.0f) atomicAdd(a.db + co, dbsum);
    } else if (!ok && tid == 0) {
        atomicOr(a.err, kErrMmaTimeout);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, L::TMEM_COLS);
}

// ---- optimizer and operand images --------------------------------------------------

__global__ void k_adam(float* __restrict__ p, float* __restrict__ g, float* __restrict__ m, float* __restrict__ v, int n,
                       float lr, float b1, float b2, float eps, float scale, float bc1, float bc2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] * scale;
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    g[i] = 0.0f;
}

// BF16 operand images of every layer from the f32 parameters: the forward image
// of layer l at element ((k / 8) * cout + co) * 8 + k % 8 with k = tap * cin + ci,
// and (l >= 1) the input-gradient image: rows ci, k' = (8 - tap) * cout + co.
__global__ void k_pack(const float* __restrict__ p, __nv_bfloat16* __restrict__ img) {
    constexpr int kWoff[4] = {layer_woff(0), layer_woff(1), layer_woff(2), layer_woff(3)};
    constexpr int kFwd[4] = {fwd_img_off(0), fwd_img_off(1), fwd_img_off(2), fwd_img_off(3)};
    constexpr int kDgrad[4] = {0, dgrad_img_off(1), dgrad_img_off(2), dgrad_img_off(3)};
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParamCount) return;
    const int l = i >= kWoff[3] ? 3 : i >= kWoff[2] ? 2 : i >= kWoff[1] ? 1 : 0;
    const int local = i - kWoff[l];
    const int cin = l == 0 ? 16 : 32, cout = l == 3 ? 16 : 32;
    if (local >= 9 * cin * cout) return;  // biases
    const int c_in = local % cin, tap = (local / cin) % 9, co = local / (9 * cin);
    const __nv_bfloat16 w = __float2bfloat16_rn(p[i]);
    // image [dx][8-channel group][dy][n][8]: for one horizontal tap and group, the
    // 3 x N rows an MMA reads are the three vertical taps' weights for every output n
    const int dy = tap / 3, dx = tap % 3;
    img[kFwd[l] + (((dx * (cin / 8) + c_in / 8) * 3 + dy) * cout + co) * 8 + c_in % 8] = w;
    if (l >= 1) {  // input gradient: the mirrored tap, inputs and outputs swapped
        const int dy2 = (8 - tap) / 3, dx2 = (8 - tap) % 3;
        img[kDgrad[l] + (((dx2 * (cout / 8) + co / 8) * 3 + dy2) * cin + c_in) * 8 + co % 8] = w;
    }
}

// ---- self-test GEMM ------------------------------------------------------------------

// D (128 x n) = A (128 x k) * B (n x k)^T with the layouts the convolutions use.
// The operand regions are sized so that every address either descriptor field
// could reach stays inside them.
template <int N>
__global__ void __launch_bounds__(kThreads) k_selftest(const __nv_bfloat16* A, const __nv_bfloat16* B, float* D, int K,
                                                      uint32_t* err) {
    extern __shared__ __align__(1024) unsigned char smem[];
    constexpr uint32_t kA = 65536, kB = 16384;
    unsigned char* sA = smem;
    unsigned char* sB = smem + kA;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kA + kB);
    uint32_t* slot = reinterpret_cast<uint32_t*>(smem + kA + kB + 8);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (warp == 0) tmem_alloc(slot, 32);
    if (tid == 0) mbar_init(bar, 1);
    for (uint32_t i = tid; i < (kA + kB) / 16; i += kThreads) reinterpret_cast<uint4*>(smem)[i] = make_uint4(0u, 0u, 0u, 0u);
    __syncthreads();
    // A: core matrix (m / 8, k / 8) at (k / 8) * 2048 + (m / 8) * 128; B: (k / 8) * (N * 16) + (n / 8) * 128
    for (int i = tid; i < 128 * K; i += kThreads) {
        const int m = i / K, k = i % K;
        *reinterpret_cast<__nv_bfloat16*>(sA + (k / 8) * 2048 + m * 16 + (k % 8) * 2) = A[i];
    }
    for (int i = tid; i < N * K; i += kThreads) {
        const int n = i / K, k = i % K;
        *reinterpret_cast<__nv_bfloat16*>(sB + (k / 8) * (N * 16) + n * 16 + (k % 8) * 2) = B[i];
    }
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *slot;
    if (tid == 0) {
        const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
        for (int s = 0; s < K / 16; ++s)
            mma_bf16(tmem, umma_desc(a0 + s * 2 * 2048, 2048, 128), umma_desc(b0 + s * 2 * N * 16, N * 16, 128),
                     idesc_bf16(128, N), s > 0 ? 1u : 0u);
        mma_commit(bar);
    }
    const bool ok = __syncthreads_and(mbar_wait(bar, 0) ? 1 : 0) != 0;
    tc_fence_after();
    if (ok) {
        float acc[N];
#pragma unroll
        for (int c = 0; c < N; c += 16) tmem_ld16(tmem + ((uint32_t)(warp * 32) << 16) + c, acc + c);
        const int m = warp * 32 + lane;
#pragma unroll
        for (int c = 0; c < N; ++c) D[m * N + c] = acc[c];
    } else if (tid == 0) {
        atomicOr(err, kErrMmaTimeout);
        mbar_wait(bar, 0);  // the MMAs complete before the tensor memory is freed
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) tmem_dealloc(tmem, 32);
}

}  // namespace up
}  // namespace rz

using namespace rz::up;

struct rz_upsampler {
    int device = 0;
    int sms = 0;
    uint32_t max_w = 0, max_h = 0;
    float* d_params = nullptr;
    float* d_grads = nullptr;
    float* d_m = nullptr;
    float* d_v = nullptr;
    __nv_bfloat16* d_img = nullptr;
    __nv_bfloat16* d_feat = nullptr;
    __nv_bfloat16* d_act[3] = {nullptr, nullptr, nullptr};
    __nv_bfloat16* d_dy3 = nullptr;
    __nv_bfloat16* d_dyA = nullptr;
    __nv_bfloat16* d_dyB = nullptr;
    double* d_loss = nullptr;
    uint32_t* d_err = nullptr;
    uint64_t values = 0;
    int adam_t = 0;
    long long wait_cycles = kWaitCycles;  // bound of the pipeline waits (rz_upsampler_set_wait_limit)
};

namespace {

template <class T>
cudaError_t ualloc(T** p, size_t count) {
    return cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
}

void ufree_all(rz_upsampler* u) {
    cudaFree(u->d_params);
    cudaFree(u->d_grads);
    cudaFree(u->d_m);
    cudaFree(u->d_v);
    cudaFree(u->d_img);
    cudaFree(u->d_feat);
    for (auto* p : u->d_act) cudaFree(p);
    cudaFree(u->d_dy3);
    cudaFree(u->d_dyA);
    cudaFree(u->d_dyB);
    cudaFree(u->d_loss);
    cudaFree(u->d_err);
}

template <class K>
cudaError_t allow_smem(K kernel, uint32_t bytes) {
    return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
}

std::once_flag g_attr_once;
cudaError_t g_attr_status = cudaSuccess;

void set_attributes() {
    cudaError_t e = cudaSuccess;
    auto keep = [&](cudaError_t r) {
        if (e == cudaSuccess) e = r;
    };
    keep(allow_smem(k_conv<16, 32, kEpiRelu>, ConvSmem<16, 32>::BYTES));
    keep(allow_smem(k_conv<32, 32, kEpiRelu>, ConvSmem<32, 32>::BYTES));
    keep(allow_smem(k_conv<32, 16, kEpiFinal>, ConvSmem<32, 16>::BYTES));
    keep(allow_smem(k_conv<16, 32, kEpiMask>, ConvSmem<16, 32>::BYTES));
    keep(allow_smem(k_conv<32, 32, kEpiMask>, ConvSmem<32, 32>::BYTES));
    keep(allow_smem(k_wgrad<32, 16>, WgSmem<32, 16>::BYTES));
    keep(allow_smem(k_wgrad<32, 32>, WgSmem<32, 32>::BYTES));
    keep(allow_smem(k_wgrad<16, 32>, WgSmem<16, 32>::BYTES));
    keep(allow_smem(k_selftest<16>, 65536 + 16384 + 16));
    keep(allow_smem(k_selftest<32>, 65536 + 16384 + 16));
    g_attr_status = e;
}

cudaError_t ensure_attributes() {
    std::call_once(g_attr_once, set_attributes);
    return g_attr_status;
}

// cuTensorMapEncodeTiled, from the driver through the runtime (no link against libcuda).
PFN_cuTensorMapEncodeTiled_v12000 g_encode_tiled = nullptr;
std::once_flag g_encode_once;

void load_encode_tiled() {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q{};
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
        g_encode_tiled = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
}

// Tensor map of a planar [C / 8][H][W][8] bf16 tensor viewed as [C / 8][H][2 W]
// 8-byte elements (a pixel's 8 channels are two elements), with boxes of
// {2 kHaloW elements, 1 row, 1 group}: each box is one contiguous 2,048-byte
// run, so TMA moves whole rows rather than 16-byte pieces. Out-of-range
// elements read as zero.
bool encode_planar(CUtensorMap* map, const void* base, int C, int W, int H) {
    std::call_once(g_encode_once, load_encode_tiled);
    if (!g_encode_tiled) return false;
    const cuuint64_t dims[3] = {(cuuint64_t)W * 2, (cuuint64_t)H, (cuuint64_t)(C / 8)};
    const cuuint64_t strides[2] = {(cuuint64_t)W * 16, (cuuint64_t)W * H * 16};
    const cuuint32_t box[3] = {(cuuint32_t)(2 * kHaloW), 1, 1};
    const cuuint32_t elem[3] = {1, 1, 1};
    return g_encode_tiled(map, CU_TENSOR_MAP_DATA_TYPE_UINT64, 3, const_cast<void*>(base), dims, strides, box, elem,
                          CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int CIN, int N, int EPI>
bool launch_conv(const rz_upsampler* u, const ConvArgs& a, cudaStream_t s) {
    CUtensorMap map;
    if (!encode_planar(&map, a.in, CIN, a.W, a.H)) return false;
    const int tiles = ((a.W + kTileOut - 1) / kTileOut) * ((a.H + kTileRows - 1) / kTileRows);
    const int grid = std::min(tiles, std::max(u->sms, 1));
    k_conv<CIN, N, EPI><<<grid, kConvThreads, ConvSmem<CIN, N>::BYTES, s>>>(a, map);
    return true;
}

template <int CIN, int N>
void launch_wgrad(const rz_upsampler* u, const WgradArgs& a, cudaStream_t s) {
    const int tiles = ((a.W + kWgKP - 1) / kWgKP) * ((a.H + kWgRows - 1) / kWgRows);
    const int grid = std::min(tiles, 2 * std::max(u->sms, 1));
    k_wgrad<CIN, N><<<grid, kThreads, WgSmem<CIN, N>::BYTES, s>>>(a);
}

bool gbuffer_ok(const rz_upsampler* u, const rz_gbuffer* g) {
    return g && g->color_rgba8 && g->depth_f32 && g->albedo_rgba8 && g->normal_oct_f16x2 && g->width > 0 &&
           g->height > 0 && g->width <= u->max_w && g->height <= u->max_h;
}

ConvArgs conv_args(const rz_upsampler* u, int W, int H) {
    ConvArgs a{};
    a.W = W;
    a.H = H;
    a.err = u->d_err;
    a.wait_cycles = u->wait_cycles;
    return a;
}

// Forward pass; with `target` it also writes the loss gradient and sum. False if
// a tensor map could not be encoded.
bool forward(rz_upsampler* u, const rz_gbuffer* g, const void* target, void* out, cudaStream_t s) {
    const int W = (int)g->width, H = (int)g->height;
    const int n = W * H;
    k_features<<<(n + 255) / 256, 256, 0, s>>>(*g, u->d_feat);
    ConvArgs a = conv_args(u, W, H);
    a.in = u->d_feat;
    a.wimg = u->d_img + fwd_img_off(0);
    a.bias = u->d_params + layer_boff(0);
    a.out = u->d_act[0];
    if (!launch_conv<16, 32, kEpiRelu>(u, a, s)) return false;
    for (int l = 1; l <= 2; ++l) {
        a.in = u->d_act[l - 1];
        a.wimg = u->d_img + fwd_img_off(l);
        a.bias = u->d_params + layer_boff(l);
        a.out = u->d_act[l];
        if (!launch_conv<32, 32, kEpiRelu>(u, a, s)) return false;
    }
    ConvArgs f = conv_args(u, W, H);
    f.in = u->d_act[2];
    f.wimg = u->d_img + fwd_img_off(3);
    f.bias = u->d_params + layer_boff(3);
    f.color_lr = static_cast<const uint32_t*>(g->color_rgba8);
    f.sources = static_cast<const uint16_t*>(g->sources_u16);
    f.out_rgba8 = static_cast<uint32_t*>(out);
    f.target = static_cast<const uint32_t*>(target);
    f.dy = u->d_dy3;
    f.loss = u->d_loss;
    if (!launch_conv<32, 16, kEpiFinal>(u, f, s)) return false;
    return true;
}

}  // namespace

extern "C" {

int rz_upsampler_create(rz_upsampler** out, int device, uint32_t max_width, uint32_t max_height) {
    if (!out || max_width == 0 || max_height == 0 || max_width > 8192 || max_height > 8192) return RZ_INVALID_ARGUMENT;
    *out = nullptr;
    if (cudaSetDevice(device) != cudaSuccess) return RZ_ERROR;
    if (ensure_attributes() != cudaSuccess) return RZ_ERROR;
    rz_upsampler* u = new rz_upsampler();
    u->device = device;
    u->max_w = max_width;
    u->max_h = max_height;
    cudaDeviceGetAttribute(&u->sms, cudaDevAttrMultiProcessorCount, device);
    const size_t px = (size_t)max_width * max_height;
    bool ok = ualloc(&u->d_params, kParamCount) == cudaSuccess && ualloc(&u->d_grads, kParamCount) == cudaSuccess &&
              ualloc(&u->d_m, kParamCount) == cudaSuccess && ualloc(&u->d_v, kParamCount) == cudaSuccess &&
              ualloc(&u->d_img, kImgCount) == cudaSuccess && ualloc(&u->d_feat, px * kFeatChannels) == cudaSuccess &&
              ualloc(&u->d_act[0], px * 32) == cudaSuccess && ualloc(&u->d_act[1], px * 32) == cudaSuccess &&
              ualloc(&u->d_act[2], px * 32) == cudaSuccess && ualloc(&u->d_dy3, px * 16) == cudaSuccess &&
              ualloc(&u->d_dyA, px * 32) == cudaSuccess && ualloc(&u->d_dyB, px * 32) == cudaSuccess &&
              ualloc(&u->d_loss, 1) == cudaSuccess && ualloc(&u->d_err, 1) == cudaSuccess;
    if (ok) {
        ok = cudaMemset(u->d_params, 0, kParamCount * sizeof(float)) == cudaSuccess &&
             cudaMemset(u->d_grads, 0, kParamCount * sizeof(float)) == cudaSuccess &&
             cudaMemset(u->d_m, 0, kParamCount * sizeof(float)) == cudaSuccess &&
             cudaMemset(u->d_v, 0, kParamCount * sizeof(float)) == cudaSuccess &&
             cudaMemset(u->d_img, 0, kImgCount * sizeof(__nv_bfloat16)) == cudaSuccess &&
             cudaMemset(u->d_loss, 0, sizeof(double)) == cudaSuccess && cudaMemset(u->d_err, 0, 4) == cudaSuccess &&
             cudaDeviceSynchronize() == cudaSuccess;
    }
    if (!ok) {
        ufree_all(u);
        delete u;
        return RZ_ERROR;
    }
    *out = u;
    return RZ_OK;
}

void rz_upsampler_destroy(rz_upsampler* u) {
    if (!u) return;
    cudaSetDevice(u->device);
    cudaDeviceSynchronize();
    ufree_all(u);
    delete u;
}

int rz_upsampler_set_params(rz_upsampler* u, const float* params, uint32_t count, void* stream) {
    if (!u || !params || count != (uint32_t)kParamCount) return RZ_INVALID_ARGUMENT;
    cudaSetDevice(u->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaMemcpyAsync(u->d_params, params, kParamCount * sizeof(float), cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(u->d_m, 0, kParamCount * sizeof(float), s) != cudaSuccess ||
        cudaMemsetAsync(u->d_v, 0, kParamCount * sizeof(float), s) != cudaSuccess)
        return RZ_ERROR;
    u->adam_t = 0;
    k_pack<<<(kParamCount + 255) / 256, 256, 0, s>>>(u->d_params, u->d_img);
    if (cudaStreamSynchronize(s) != cudaSuccess) return RZ_ERROR;  // the host array may be freed after return
    return cudaGetLastError() == cudaSuccess ? RZ_OK : RZ_ERROR;
}

int rz_upsampler_get_params(rz_upsampler* u, float* params, uint32_t count, void* stream) {
    if (!u || !params || count != (uint32_t)kParamCount) return RZ_INVALID_ARGUMENT;
    cudaSetDevice(u->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaMemcpyAsync(params, u->d_params, kParamCount * sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return RZ_ERROR;
    return RZ_OK;
}

int rz_upsampler_infer(rz_upsampler* u, const rz_gbuffer* in, void* out_rgba8, void* stream) {
    if (!u || !gbuffer_ok(u, in) || !out_rgba8) return RZ_INVALID_ARGUMENT;
    cudaSetDevice(u->device);
    if (!forward(u, in, nullptr, out_rgba8, static_cast<cudaStream_t>(stream))) return RZ_ERROR;
    return cudaGetLastError() == cudaSuccess ? RZ_OK : RZ_ERROR;
}

int rz_upsampler_accumulate(rz_upsampler* u, const rz_gbuffer* in, const void* target_rgba8, void* out_rgba8,
                            void* stream) {
    if (!u || !gbuffer_ok(u, in) || !target_rgba8) return RZ_INVALID_ARGUMENT;
    cudaSetDevice(u->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int W = (int)in->width, H = (int)in->height;
    if (!forward(u, in, target_rgba8, out_rgba8, s)) return RZ_ERROR;
    WgradArgs w{};
    w.W = W;
    w.H = H;
    w.err = u->d_err;
    w.wait_cycles = u->wait_cycles;
    ConvArgs d = conv_args(u, W, H);
    // layer 3
    w.x = u->d_act[2];
    w.dy = u->d_dy3;
    w.dw = u->d_grads + layer_woff(3);
    w.db = u->d_grads + layer_boff(3);
    launch_wgrad<32, 16>(u, w, s);
    d.in = u->d_dy3;
    d.wimg = u->d_img + dgrad_img_off(3);
    d.mask_src = u->d_act[2];
    d.out = u->d_dyA;
    if (!launch_conv<16, 32, kEpiMask>(u, d, s)) return RZ_ERROR;
    // layer 2
    w.x = u->d_act[1];
    w.dy = u->d_dyA;
    w.dw = u->d_grads + layer_woff(2);
    w.db = u->d_grads + layer_boff(2);
    launch_wgrad<32, 32>(u, w, s);
    d.in = u->d_dyA;
    d.wimg = u->d_img + dgrad_img_off(2);
    d.mask_src = u->d_act[1];
    d.out = u->d_dyB;
    if (!launch_conv<32, 32, kEpiMask>(u, d, s)) return RZ_ERROR;
    // layer 1
    w.x = u->d_act[0];
    w.dy = u->d_dyB;
    w.dw = u->d_grads + layer_woff(1);
    w.db = u->d_grads + layer_boff(1);
    launch_wgrad<32, 32>(u, w, s);
    d.in = u->d_dyB;
    d.wimg = u->d_img + dgrad_img_off(1);
    d.mask_src = u->d_act[0];
    d.out = u->d_dyA;
    if (!launch_conv<32, 32, kEpiMask>(u, d, s)) return RZ_ERROR;
    // layer 0
    w.x = u->d_feat;
    w.dy = u->d_dyA;
    w.dw = u->d_grads + layer_woff(0);
    w.db = u->d_grads + layer_boff(0);
    launch_wgrad<16, 32>(u, w, s);
    u->values += (uint64_t)4 * W * H * 3;
    return cudaGetLastError() == cudaSuccess ? RZ_OK : RZ_ERROR;
}

int rz_upsampler_get_grads(rz_upsampler* u, float* grads, uint32_t count, double* loss_sum, uint64_t* values,
                           void* stream) {
    if (!u || (grads && count != (uint32_t)kParamCount)) return RZ_INVALID_ARGUMENT;
    cudaSetDevice(u->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (grads && cudaMemcpyAsync(grads, u->d_grads, kParamCount * sizeof(float), cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return RZ_ERROR;
    double l = 0.0;
    if (cudaMemcpyAsync(&l, u->d_loss, sizeof(double), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return RZ_ERROR;
    if (loss_sum) *loss_sum = l;
    if (values) *values = u->values;
    return RZ_OK;
}

int rz_upsampler_adam_step(rz_upsampler* u, float lr, float beta1, float beta2, float eps, float grad_scale,
                           void* stream) {
    if (!u || !(lr >= 0.0f) || !(beta1 >= 0.0f && beta1 < 1.0f) || !(beta2 >= 0.0f && beta2 < 1.0f) || !(eps > 0.0f))
        return RZ_INVALID_ARGUMENT;
    cudaSetDevice(u->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    u->adam_t += 1;
    const float bc1 = 1.0f - (float)std::pow((double)beta1, (double)u->adam_t);
    const float bc2 = 1.0f - (float)std::pow((double)beta2, (double)u->adam_t);
    k_adam<<<(kParamCount + 255) / 256, 256, 0, s>>>(u->d_params, u->d_grads, u->d_m, u->d_v, kParamCount, lr, beta1,
                                                      beta2, eps, grad_scale, bc1, bc2);
    k_pack<<<(kParamCount + 255) / 256, 256, 0, s>>>(u->d_params, u->d_img);
    if (cudaMemsetAsync(u->d_loss, 0, sizeof(double), s) != cudaSuccess) return RZ_ERROR;
    u->values = 0;
    return cudaGetLastError() == cudaSuccess ? RZ_OK : RZ_ERROR;
}

int rz_upsampler_set_wait_limit(rz_upsampler* u, uint64_t cycles) {
    if (!u) return RZ_INVALID_ARGUMENT;
    u->wait_cycles = (cycles == 0 || cycles > (uint64_t)kWaitCycles) ? kWaitCycles : (long long)cycles;
    return RZ_OK;
}

int rz_upsampler_status(rz_upsampler* u, uint32_t* flags, void* stream) {
    if (!u || !flags) return RZ_INVALID_ARGUMENT;
    cudaSetDevice(u->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (cudaMemcpyAsync(flags, u->d_err, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess)
        return RZ_ERROR;
    return RZ_OK;
}

int rz_upsampler_selftest_gemm(const void* a_bf16, const void* b_bf16, float* d_f32, uint32_t n, uint32_t k, void* stream) {
    if (!a_bf16 || !b_bf16 || !d_f32 || (n != 16 && n != 32) || k == 0 || k > 64 || k % 16 != 0) return RZ_INVALID_ARGUMENT;
    if (ensure_attributes() != cudaSuccess) return RZ_ERROR;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    uint32_t* err = nullptr;
    if (cudaMalloc(&err, 4) != cudaSuccess) return RZ_ERROR;
    cudaMemsetAsync(err, 0, 4, s);
    const auto* A = static_cast<const __nv_bfloat16*>(a_bf16);
    const auto* B = static_cast<const __nv_bfloat16*>(b_bf16);
    if (n == 16) k_selftest<16><<<1, kThreads, 65536 + 16384 + 16, s>>>(A, B, d_f32, (int)k, err);
    else k_selftest<32><<<1, kThreads, 65536 + 16384 + 16, s>>>(A, B, d_f32, (int)k, err);
    uint32_t flags = 0;
    const bool ok = cudaGetLastError() == cudaSuccess &&
                    cudaMemcpyAsync(&flags, err, 4, cudaMemcpyDeviceToHost, s) == cudaSuccess &&
                    cudaStreamSynchronize(s) == cudaSuccess;
    cudaFree(err);
    if (!ok) return RZ_ERROR;
    return flags ? RZ_TIMEOUT : RZ_OK;
}

}  // extern "C"
