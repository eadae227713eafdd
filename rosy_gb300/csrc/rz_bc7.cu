// BC7 texture decoding on the device.
//
// The reference's images are BC7 blocks from .dds files that it uploads as
// VK_FORMAT_BC7_SRGB_BLOCK / VK_FORMAT_BC7_UNORM_BLOCK images
// (src/Engine/Graphics.cpp:3605-3647, 3700-3830) and leaves to the texture unit.
// This renderer samples RGBA8 texels with its own filtering code, so a BC7
// texture is decoded once, on upload, into the RGBA8 texel pool: k_bc7_decode
// turns every level of a mip chain into RGBA8 in one launch.
//
// Format (BPTC: Khronos Data Format Specification, "BPTC Compressed Texture
// Image Formats"; Direct3D 11 "BC7 Format"): a 128-bit block holds 4x4 texels.
// The lowest set bit of the first byte is the mode (0-7; none = reserved mode,
// decoded to 0,0,0,0). The mode fixes the subset count, partition / rotation /
// index-selection fields, endpoint precision and P-bits, and index widths.
// Endpoints are stored channel-major (R of every endpoint, then G, B, A),
// widened to 8 bits by bit replication; texel t of subset s takes
// ((64 - w) * e0 + w * e1 + 32) >> 6 with w from the 2-, 3- or 4-bit weight
// table; anchor texels store their index with one bit fewer.
//
// Work: one thread per block, reading its 16 bytes with one vector load and
// writing four rows of 16 bytes; a warp covers 32 consecutive blocks of a
// block row, so its loads and stores are contiguous. Tables (partition maps,
// anchor masks, mode fields, weights) are a kernel parameter copied to shared
// memory. Bound: HBM, 16 bytes read + 64 written per block.
#include "rz_device.cuh"

namespace rz {

namespace {

constexpr int kBc7Threads = 256;
constexpr int kBc7MaxLevels = 16;

// Subset maps (2 bits per texel, texel 0 lowest) and anchor-texel masks:
// entries [0, 64) are the two-subset partitions, [64, 128) the three-subset ones.
struct Bc7Tables {
    uint32_t map[128];
    uint32_t anchors[128];
    uint32_t mode_lo[8];  // per mode: ns | pb << 4 | rb << 8 | isb << 12 | cb << 16 | ab << 20 | pbit kind << 24 | ib << 28
    uint32_t mode_hi[8];  // per mode: secondary index bits
    uint32_t weights[12]; // bytes: [0,4) 2-bit, [4,12) 3-bit, [16,32) 4-bit weights, 4 per word
};

struct Bc7Level {
    uint32_t block0;  // first block of the level in the chain
    uint32_t bw, bh;  // blocks per row, block rows
    uint32_t w, h;    // texels
    uint32_t texel0;  // first texel of the level in the output
    uint32_t vec;     // rows and the level start are 16-byte aligned: full blocks store as uint4
};

struct Bc7Job {
    const uint4* blocks;
    uint32_t* texels;
    uint32_t levels;
    uint32_t total_blocks;
    Bc7Level L[kBc7MaxLevels];
};

// The two-subset partitions as 16-bit masks (bit t set = texel t in subset 1).
constexpr uint16_t kTwoSubset[64] = {
    0xCCCC, 0x8888, 0xEEEE, 0xECC8, 0xC880, 0xFEEC, 0xFEC8, 0xEC80, 0xC800, 0xFFEC, 0xFE80, 0xE800, 0xFFE8,
    0xFF00, 0xFFF0, 0xF000, 0xF710, 0x008E, 0x7100, 0x08CE, 0x008C, 0x7310, 0x3100, 0x8CCE, 0x088C, 0x3110,
    0x6666, 0x366C, 0x17E8, 0x0FF0, 0x718E, 0x399C, 0xAAAA, 0xF0F0, 0x5A5A, 0x33CC, 0x3C3C, 0x55AA, 0x9696,
    0xA55A, 0x73CE, 0x13C8, 0x324C, 0x3BDC, 0x6996, 0xC33C, 0x9966, 0x0660, 0x0272, 0x04E4, 0x4E40, 0x2720,
    0xC936, 0x936C, 0x39C6, 0x639C, 0x9336, 0x9CC6, 0x817E, 0xE718, 0xCCF0, 0x0FCC, 0x7744, 0xEE22,
};

// The three-subset partitions, one string of 16 subset digits per partition.
constexpr const char* kThreeSubset[64] = {
    "0011001102212222", "0001001122112221", "0000200122112211", "0222002200110111", "0000000011221122",
    "0011001100220022", "0022002211111111", "0011001122112211", "0000000011112222", "0000111111112222",
    "0000111122222222", "0012001200120012", "0112011201120112", "0122012201220122", "0011011211221222",
    "0011200122002220", "0001001101121122", "0111001120012200", "0000112211221122", "0022002200221111",
    "0111011102220222", "0001000122212221", "0000001101220122", "0000110022102210", "0122012200110000",
    "0012001211222222", "0110122112210110", "0000011012211221", "0022110211020022", "0110011020022222",
    "0011012201220011", "0000200022112221", "0000000211221222", "0222002200120011", "0011001200220222",
    "0120012001200120", "0000111122220000", "0120120120120120", "0120201212010120", "0011220011220011",
    "0011112222000011", "0101010122222222", "0000000021212121", "0022112200221122", "0022001100220011",
    "0220122102201221", "0101222222220101", "0000212121212121", "0101010101012222", "0222011102220111",
    "0002111200021112", "0000211221122112", "0222011101110222", "0002111211120002", "0110011001102222",
    "0000000021122112", "0110011022222222", "0022001100110022", "0022112211220022", "0000000000002112",
    "0002000100020001", "0222122202221222", "0101222222222222", "0111201122012220",
};

// Anchor texels of subset 1 (two subsets) and of subsets 1 and 2 (three subsets).
constexpr uint8_t kAnchorTwo[64] = {
    15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 2,  8,  2,  2,  8,  8,  15, 2,  8,  2,  2,
    8,  8,  2,  2,  15, 15, 6,  8,  2,  8,  15, 15, 2,  8,  2,  2,  2,  15, 15, 6,  6,  2,  6,  8,  15, 15, 2,  2,
    15, 15, 15, 15, 15, 2,  2,  15,
};
constexpr uint8_t kAnchorThreeA[64] = {
    3,  3,  15, 15, 8,  3,  15, 15, 8,  8,  6,  6,  6,  5,  3,  3,  3,  3,  8,  15, 3,  3,  6,  10, 5,  8,  8,  6,
    8,  5,  15, 15, 8,  15, 3,  5,  6,  10, 8,  15, 15, 3,  15, 5,  15, 15, 15, 15, 3,  15, 5,  5,  5,  8,  5,  10,
    5,  10, 8,  13, 15, 12, 3,  3,
};
constexpr uint8_t kAnchorThreeB[64] = {
    15, 8,  8,  3,  15, 15, 3,  8,  15, 15, 15, 15, 15, 15, 15, 8,  15, 8,  15, 3,  15, 8,  15, 8,  3,  15, 6,  10,
    15, 15, 10, 8,  15, 3,  15, 10, 10, 8,  9,  10, 6,  15, 8,  15, 3,  6,  6,  8,  15, 3,  15, 15, 15, 15, 15, 15,
    15, 15, 15, 15, 3,  15, 15, 8,
};

// Mode fields: subsets, partition bits, rotation bits, index-selection bits,
// colour bits, alpha bits, P-bits (0 none, 1 one per endpoint, 2 one per
// subset), index bits, secondary index bits.
constexpr uint8_t kModeFields[8][9] = {
    {3, 4, 0, 0, 4, 0, 1, 3, 0}, {2, 6, 0, 0, 6, 0, 2, 3, 0}, {3, 6, 0, 0, 5, 0, 0, 2, 0}, {2, 6, 0, 0, 7, 0, 1, 2, 0},
    {1, 0, 2, 1, 5, 6, 0, 2, 3}, {1, 0, 2, 0, 7, 8, 0, 2, 2}, {1, 0, 0, 0, 7, 7, 1, 4, 0}, {2, 6, 0, 0, 5, 5, 1, 2, 0},
};

constexpr uint8_t kWeightBytes[48] = {
    0, 21, 43, 64, 0, 9, 18, 27, 37, 46, 55, 64, 0, 0, 0, 0,
    0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64,
};

Bc7Tables make_tables() {
    Bc7Tables t{};
    for (int p = 0; p < 64; ++p) {
        uint32_t m2 = 0, m3 = 0;
        for (int i = 0; i < 16; ++i) {
            m2 |= (uint32_t)((kTwoSubset[p] >> i) & 1) << (2 * i);
            m3 |= (uint32_t)(kThreeSubset[p][i] - '0') << (2 * i);
        }
        t.map[p] = m2;
        t.map[64 + p] = m3;
        t.anchors[p] = 1u | (1u << kAnchorTwo[p]);
        t.anchors[64 + p] = 1u | (1u << kAnchorThreeA[p]) | (1u << kAnchorThreeB[p]);
    }
    for (int m = 0; m < 8; ++m) {
        const uint8_t* f = kModeFields[m];
        t.mode_lo[m] = f[0] | f[1] << 4 | f[2] << 8 | f[3] << 12 | f[4] << 16 | f[5] << 20 | f[6] << 24 | (uint32_t)f[7] << 28;
        t.mode_hi[m] = f[8];
    }
    for (int i = 0; i < 12; ++i)
        t.weights[i] = kWeightBytes[4 * i] | kWeightBytes[4 * i + 1] << 8 | kWeightBytes[4 * i + 2] << 16 |
                       (uint32_t)kWeightBytes[4 * i + 3] << 24;
    return t;
}

const Bc7Tables& tables() {
    static const Bc7Tables t = make_tables();
    return t;
}

// Takes the next n (0..8) bits of the 128-bit block held in lo:hi.
__device__ __forceinline__ uint32_t take(uint64_t& lo, uint64_t& hi, uint32_t n) {
    const uint32_t v = (uint32_t)lo & ((1u << n) - 1u);
    if (n) {
        lo = (lo >> n) | (hi << (64 - n));
        hi >>= n;
    }
    return v;
}

// Widens the three colour bytes of a packed endpoint from n (5..8) bits to 8 by
// replicating their high bits; each byte holds a value below 2^n.
__device__ __forceinline__ uint32_t widen3(uint32_t e, uint32_t n) {
    if (n >= 8) return e;
    const uint32_t hi_mask = ((0xFFu << (8 - n)) & 0xFFu) * 0x010101u;
    const uint32_t lo_mask = ((1u << (8 - n)) - 1u) * 0x010101u;
    return ((e << (8 - n)) & hi_mask) | ((e >> (2 * n - 8)) & lo_mask);
}

__device__ __forceinline__ uint32_t widen1(uint32_t v, uint32_t n) { return n >= 8 ? v : (v << (8 - n)) | (v >> (2 * n - 8)); }

__device__ __forceinline__ uint32_t weight(const uint8_t* w, uint32_t bits, uint32_t idx) {
    return w[(bits == 2 ? 0 : bits == 3 ? 4 : 16) + idx];
}

// Decodes one block into 16 RGBA8 texels (row-major).
__device__ void bc7_block(uint4 q, const Bc7Tables& T, uint32_t px[16]) {
    const uint32_t m8 = q.x & 0xFFu;
    if (m8 == 0) {
#pragma unroll
        for (int t = 0; t < 16; ++t) px[t] = 0u;
        return;
    }
    const uint32_t mode = __ffs(m8) - 1;
    const uint32_t f = T.mode_lo[mode];
    const uint32_t ns = f & 15, pb = (f >> 4) & 15, rb = (f >> 8) & 15, isbits = (f >> 12) & 15;
    const uint32_t cb = (f >> 16) & 15, ab = (f >> 20) & 15, pkind = (f >> 24) & 15, ib = f >> 28;
    const uint32_t ib2 = T.mode_hi[mode];
    uint64_t lo = q.x | (uint64_t)q.y << 32, hi = q.z | (uint64_t)q.w << 32;
    take(lo, hi, mode + 1);
    const uint32_t part = take(lo, hi, pb);
    const uint32_t rot = take(lo, hi, rb);
    const uint32_t isb = take(lo, hi, isbits);
    // endpoint k = 2 * subset + end, channels packed R | G << 8 | B << 16 | A << 24
    uint32_t E[6] = {0u, 0u, 0u, 0u, 0u, 0u};
#pragma unroll
    for (int ch = 0; ch < 3; ++ch)
#pragma unroll
        for (int k = 0; k < 6; ++k)
            if (k < (int)(2 * ns)) E[k] |= take(lo, hi, cb) << (8 * ch);
    if (ab) {
#pragma unroll
        for (int k = 0; k < 6; ++k)
            if (k < (int)(2 * ns)) E[k] |= take(lo, hi, ab) << 24;
    }
    if (pkind == 1) {
#pragma unroll
        for (int k = 0; k < 6; ++k)
            if (k < (int)(2 * ns)) E[k] = (E[k] << 1) | (take(lo, hi, 1) * 0x01010101u);
    } else if (pkind == 2) {
#pragma unroll
        for (int s = 0; s < 3; ++s)
            if (s < (int)ns) {
                const uint32_t p = take(lo, hi, 1) * 0x01010101u;
                E[2 * s] = (E[2 * s] << 1) | p;
                E[2 * s + 1] = (E[2 * s + 1] << 1) | p;
            }
    }
    const uint32_t nc = cb + (pkind ? 1u : 0u), na = ab ? ab + (pkind ? 1u : 0u) : 0u;
#pragma unroll
    for (int k = 0; k < 6; ++k) {
        const uint32_t a = na ? widen1(E[k] >> 24, na) : 255u;
        E[k] = widen3(E[k] & 0x00FFFFFFu, nc) | a << 24;
    }
    const uint32_t table = ns == 3 ? 64u + part : part;
    const uint32_t map = ns == 1 ? 0u : T.map[table];
    const uint32_t amask = ns == 1 ? 1u : T.anchors[table];
    uint64_t i1 = 0, i2 = 0;
#pragma unroll
    for (int t = 0; t < 16; ++t) i1 |= (uint64_t)take(lo, hi, ib - ((amask >> t) & 1u)) << (4 * t);
    if (ib2) {
#pragma unroll
        for (int t = 0; t < 16; ++t) i2 |= (uint64_t)take(lo, hi, ib2 - (t == 0 ? 1u : 0u)) << (4 * t);
    }
    // colour and alpha index sets: one set for both, or (modes 4, 5) the index-selection bit picks
    const bool swap = ib2 && isb;
    const uint64_t ci = swap ? i2 : i1, ai = ib2 ? (isb ? i1 : i2) : i1;
    const uint32_t cbits = swap ? ib2 : ib, abits = ib2 ? (isb ? ib : ib2) : ib;
    const uint8_t* W = reinterpret_cast<const uint8_t*>(T.weights);
    const uint32_t sel = rot == 0 ? 0x3210u : rot == 1 ? 0x0213u : rot == 2 ? 0x1230u : 0x2310u;
#pragma unroll
    for (int t = 0; t < 16; ++t) {
        const uint32_t s = (map >> (2 * t)) & 3u;
        const uint32_t e0 = s == 0 ? E[0] : s == 1 ? E[2] : E[4];
        const uint32_t e1 = s == 0 ? E[1] : s == 1 ? E[3] : E[5];
        const uint32_t wc = weight(W, cbits, (uint32_t)(ci >> (4 * t)) & 15u);
        const uint32_t wa = weight(W, abits, (uint32_t)(ai >> (4 * t)) & 15u);
        // R and B in two 16-bit lanes: (64 - w) * 255 + w * 255 + 32 < 2^16, so the lanes never carry
        const uint32_t rb2 = (((64u - wc) * (e0 & 0x00FF00FFu) + wc * (e1 & 0x00FF00FFu) + 0x00200020u) >> 6) & 0x00FF00FFu;
        const uint32_t g = ((64u - wc) * ((e0 >> 8) & 0xFFu) + wc * ((e1 >> 8) & 0xFFu) + 32u) >> 6;
        const uint32_t a = ((64u - wa) * (e0 >> 24) + wa * (e1 >> 24) + 32u) >> 6;
        px[t] = __byte_perm(rb2 | g << 8 | a << 24, 0u, sel);
    }
}

__global__ void __launch_bounds__(kBc7Threads) k_bc7_decode(const Bc7Job job, const Bc7Tables tables) {
    __shared__ Bc7Tables T;
    __shared__ Bc7Level L[kBc7MaxLevels];
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(&tables);
        uint32_t* dst = reinterpret_cast<uint32_t*>(&T);
        for (uint32_t i = threadIdx.x; i < sizeof(Bc7Tables) / 4; i += blockDim.x) dst[i] = src[i];
        const uint32_t* ls = reinterpret_cast<const uint32_t*>(job.L);
        uint32_t* ld = reinterpret_cast<uint32_t*>(L);
        for (uint32_t i = threadIdx.x; i < sizeof(job.L) / 4; i += blockDim.x) ld[i] = ls[i];
    }
    __syncthreads();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < job.total_blocks; b += stride) {
        uint32_t l = 0;
        while (l + 1 < job.levels && b >= L[l + 1].block0) ++l;
        const Bc7Level& lv = L[l];
        const uint32_t local = b - lv.block0, bx = local % lv.bw, by = local / lv.bw;
        uint32_t px[16];
        bc7_block(__ldg(job.blocks + b), T, px);
        const uint32_t x0 = 4 * bx, y0 = 4 * by;
        uint32_t* out = job.texels + lv.texel0;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const uint32_t y = y0 + r;
            if (y >= lv.h) break;
            uint32_t* row = out + (size_t)y * lv.w + x0;
            if (lv.vec && x0 + 4 <= lv.w) {
                *reinterpret_cast<uint4*>(row) = make_uint4(px[4 * r], px[4 * r + 1], px[4 * r + 2], px[4 * r + 3]);
            } else {
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    if (x0 + c < lv.w) row[c] = px[4 * r + c];
            }
        }
    }
}

// Point sampling of a BC7 CUDA array at texel centres: the texture unit's own decoding.
__global__ void k_bc7_texture_unit(cudaTextureObject_t tex, uint32_t w, uint32_t h, uint32_t* out) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= w || y >= h) return;
    const float4 v = tex2D<float4>(tex, (float)x + 0.5f, (float)y + 0.5f);
    auto q = [](float c) { return (uint32_t)floorf(fminf(fmaxf(c, 0.0f), 1.0f) * 255.0f + 0.5f); };
    out[(size_t)y * w + x] = q(v.x) | q(v.y) << 8 | q(v.z) << 16 | q(v.w) << 24;
}

}  // namespace

uint64_t bc7_chain_bytes(uint32_t width, uint32_t height, uint32_t levels) {
    uint64_t n = 0;
    for (uint32_t l = 0; l < levels; ++l) {
        const uint32_t w = std::max(1u, width >> l), h = std::max(1u, height >> l);
        n += (uint64_t)((w + 3) / 4) * ((h + 3) / 4) * 16;
    }
    return n;
}

// Decodes a mip chain of BC7 blocks (device) into RGBA8 texels (device, levels
// concatenated level 0 first, `level_off` texels each) on `stream`.
cudaError_t bc7_decode_chain(const void* blocks, uint32_t width, uint32_t height, uint32_t levels,
                             const uint32_t* level_off, uint32_t* texels, cudaStream_t stream) {
    if (levels == 0 || levels > kBc7MaxLevels) return cudaErrorInvalidValue;
    Bc7Job job{};
    job.blocks = static_cast<const uint4*>(blocks);
    job.texels = texels;
    job.levels = levels;
    uint64_t total = 0;
    for (uint32_t l = 0; l < levels; ++l) {
        Bc7Level& lv = job.L[l];
        lv.w = std::max(1u, width >> l);
        lv.h = std::max(1u, height >> l);
        lv.bw = (lv.w + 3) / 4;
        lv.bh = (lv.h + 3) / 4;
        lv.block0 = (uint32_t)total;
        lv.texel0 = level_off[l];
        lv.vec = (lv.w % 4 == 0 && lv.texel0 % 4 == 0 && reinterpret_cast<uintptr_t>(texels) % 16 == 0) ? 1u : 0u;
        total += (uint64_t)lv.bw * lv.bh;
    }
    if (total >= 0xFFFFFFFFull) return cudaErrorInvalidValue;
    job.total_blocks = (uint32_t)total;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const uint64_t want = (total + kBc7Threads - 1) / kBc7Threads;
    const uint32_t grid = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)std::max(sms, 1) * 8));
    k_bc7_decode<<<grid, kBc7Threads, 0, stream>>>(job, tables());
    return cudaGetLastError();
}

}  // namespace rz

using namespace rz;

extern "C" int rz_bc7_decode(const void* blocks, uint32_t width, uint32_t height, void* rgba8, void* stream) {
    if (!blocks || !rgba8 || width == 0 || height == 0) return RZ_INVALID_ARGUMENT;
    const uint32_t off = 0;
    const cudaError_t e = bc7_decode_chain(blocks, width, height, 1, &off, static_cast<uint32_t*>(rgba8),
                                           static_cast<cudaStream_t>(stream));
    return e == cudaSuccess ? RZ_OK : e == cudaErrorInvalidValue ? RZ_INVALID_ARGUMENT : RZ_ERROR;
}

extern "C" int rz_bc7_decode_texture_unit(const void* blocks, uint32_t width, uint32_t height, void* rgba8) {
    if (!blocks || !rgba8 || width == 0 || height == 0 || width % 4 || height % 4) return RZ_INVALID_ARGUMENT;
    const cudaChannelFormatDesc desc = cudaCreateChannelDesc(8, 8, 8, 8, cudaChannelFormatKindUnsignedBlockCompressed7);
    cudaArray_t arr = nullptr;
    if (cudaMallocArray(&arr, &desc, width, height) != cudaSuccess) {
        cudaGetLastError();
        return RZ_ALLOCATION_FAILURE;
    }
    int rc = RZ_OK;
    cudaTextureObject_t tex = 0;
    // a block-compressed array is copied by rows of blocks: (width / 4) blocks of 16 bytes, height / 4 rows
    const size_t row = (size_t)(width / 4) * 16;
    if (cudaMemcpy2DToArray(arr, 0, 0, blocks, row, row, height / 4, cudaMemcpyDeviceToDevice) != cudaSuccess) {
        rc = RZ_COPY_FAILED;
    } else {
        cudaResourceDesc res{};
        res.resType = cudaResourceTypeArray;
        res.res.array.array = arr;
        cudaTextureDesc td{};
        td.addressMode[0] = td.addressMode[1] = cudaAddressModeClamp;
        td.filterMode = cudaFilterModePoint;
        td.readMode = cudaReadModeNormalizedFloat;
        td.normalizedCoords = 0;
        if (cudaCreateTextureObject(&tex, &res, &td, nullptr) != cudaSuccess) {
            rc = RZ_CREATE_FAILED;
        } else {
            k_bc7_texture_unit<<<dim3((width + 127) / 128, height), 128>>>(tex, width, height, static_cast<uint32_t*>(rgba8));
            if (cudaGetLastError() != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess) rc = RZ_ERROR;
        }
    }
    if (tex) cudaDestroyTextureObject(tex);
    cudaFreeArray(arr);
    cudaGetLastError();
    return rc;
}
