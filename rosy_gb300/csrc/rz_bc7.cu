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
// Work: one CTA per tile of 64 x 4 blocks (256 x 16 texels). Each thread reads
// one block (a 16-byte load); the tile's blocks are counting-sorted by mode in
// shared memory, so that a warp almost always decodes 32 blocks of one mode with
// the code specialised for that mode: every field sits at a compile-time bit
// position (a funnel shift and a mask), and the index streams are made uniform
// by inserting the anchors' missing high bits. Decoded texels are staged in
// shared memory and the tile leaves as 16 rows of 1 KB, coalesced. Tables
// (partition maps, anchors) are a kernel parameter copied to shared memory.
// Algorithmic traffic: 16 bytes read + 64 written per block (the HBM roofline);
// the decode arithmetic (integer ALU issue) bounds it before HBM does.
#include "rz_device.cuh"

namespace rz {

namespace {

constexpr int kBc7Threads = 256;   // one thread per block of a tile
constexpr int kTileBX = 64;        // a tile: 64 x 4 blocks = 256 x 16 texels
constexpr int kTileBY = 4;
constexpr int kStagePitch = 4 * kTileBX + 4;  // staged texel row (u32), padded against bank conflicts
constexpr int kBc7MaxLevels = 16;
static_assert(kTileBX * kTileBY == kBc7Threads, "one thread per block of a tile");

// Subset of every texel (2 bits per texel, texel 0 lowest) and the anchor texels
// other than texel 0: entries [0, 64) are the two-subset partitions (anchor
// index), [64, 128) the three-subset ones (lower anchor | higher anchor << 8).
struct Bc7Tables {
    uint32_t map[128];
    uint32_t anchors[128];
};

struct Bc7Level {
    uint32_t block0;   // first block of the level in the chain
    uint32_t bw, bh;   // blocks per row, block rows
    uint32_t w, h;     // texels
    uint32_t texel0;   // first texel of the level in the output
    uint32_t tile0;    // first tile of the level
    uint32_t tiles_x;  // tiles per row of tiles
    uint32_t vec;      // rows and the level start are 16-byte aligned: four texels store as one uint4
};

struct Bc7Job {
    const uint4* blocks;
    uint32_t* texels;
    uint32_t levels;
    uint32_t total_tiles;
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
        t.anchors[p] = kAnchorTwo[p];
        const uint32_t a = kAnchorThreeA[p], b = kAnchorThreeB[p];
        t.anchors[64 + p] = std::min(a, b) | std::max(a, b) << 8;
    }
    return t;
}

const Bc7Tables& tables() {
    static const Bc7Tables t = make_tables();
    return t;
}

__device__ __forceinline__ uint32_t word_of(const uint4& q, int i) {
    return i == 0 ? q.x : i == 1 ? q.y : i == 2 ? q.z : i == 3 ? q.w : 0u;
}

// Bits [pos, pos + n) of the block, n <= 32. The decoders call it with positions
// and widths known at compile time, where it is a funnel shift and a mask.
__device__ __forceinline__ uint32_t field(const uint4& q, int pos, int n) {
    const uint32_t v = __funnelshift_r(word_of(q, pos >> 5), word_of(q, (pos >> 5) + 1), pos & 31);
    return n >= 32 ? v : v & ((1u << n) - 1u);
}

__device__ __forceinline__ uint64_t field64(const uint4& q, int pos, int n) {  // n <= 64
    const uint64_t lo = field(q, pos, n < 32 ? n : 32);
    return n <= 32 ? lo : lo | (uint64_t)field(q, pos + 32, n - 32) << 32;
}

// x with a zero bit inserted at position p (the bits from p up move up one).
__device__ __forceinline__ uint64_t insert_zero(uint64_t x, uint32_t p) {
    const uint64_t low = x & ((1ull << p) - 1ull);
    return low | ((x ^ low) << 1);
}

// Interpolation weight (out of 64) of a 2-, 3- or 4-bit index: the format's
// tables {0, 21, 43, 64}, {0, 9, 18, 27, 37, 46, 55, 64} and {0, 4, 9, ..., 60, 64}
// are floor((64 i + c) / (2^IB - 1)) with c = 1, 3, 7; the division is a
// multiply by a rounded-up 2^16 / (2^IB - 1), exact for these small numerators
// (checked against every table entry).
template <int IB>
__device__ __forceinline__ uint32_t weight_of(uint32_t i) {
    constexpr uint32_t c = IB == 2 ? 1u : IB == 3 ? 3u : 7u;
    constexpr uint32_t m = IB == 2 ? 21846u : IB == 3 ? 9363u : 4370u;
    return ((64u * i + c) * m) >> 16;
}

// Widens the three colour bytes of a packed endpoint from N (5..8) bits to 8 by
// replicating their high bits; each byte holds a value below 2^N.
template <int N>
__device__ __forceinline__ uint32_t widen3(uint32_t e) {
    if constexpr (N >= 8) {
        return e;
    } else {
        constexpr uint32_t hi_mask = ((0xFFu << (8 - N)) & 0xFFu) * 0x010101u;
        constexpr uint32_t lo_mask = ((1u << (8 - N)) - 1u) * 0x010101u;
        return ((e << (8 - N)) & hi_mask) | ((e >> (2 * N - 8)) & lo_mask);
    }
}

template <int N>
__device__ __forceinline__ uint32_t widen1(uint32_t v) {
    if constexpr (N >= 8) return v;
    else return (v << (8 - N)) | (v >> (2 * N - 8));
}

// One block of mode M to its 4 x 4 RGBA8 texels, row r at out + r * pitch (16-byte
// aligned). The layout follows the mode: partition, rotation and index-selection
// fields after the mode bits, colour endpoints channel-major, alpha endpoints,
// P-bits, then the primary and (modes 4, 5) secondary index streams. Rows are a
// loop (the streams and the subset map shift down after each), the four texels
// of a row unrolled: the eight decoders stay small enough for the instruction cache.
template <int M>
__device__ __forceinline__ void decode_mode(const uint4& q, const Bc7Tables& T, uint32_t* out, int pitch) {
    constexpr int NS = kModeFields[M][0], PB = kModeFields[M][1], RB = kModeFields[M][2], ISB = kModeFields[M][3];
    constexpr int CB = kModeFields[M][4], AB = kModeFields[M][5], PK = kModeFields[M][6];
    constexpr int IB = kModeFields[M][7], IB2 = kModeFields[M][8];
    constexpr int P0 = M + 1, R0 = P0 + PB, S0 = R0 + RB, E0 = S0 + ISB;
    constexpr int A0 = E0 + 3 * 2 * NS * CB, B0 = A0 + 2 * NS * AB;
    constexpr int I0 = B0 + (PK == 1 ? 2 * NS : PK == 2 ? NS : 0);
    constexpr int L1 = 16 * IB - NS, L2 = IB2 ? 16 * IB2 - 1 : 0;
    static_assert(I0 + L1 + L2 == 128, "the mode's fields fill the block");
    constexpr int NC = CB + (PK ? 1 : 0), NA = AB ? AB + (PK ? 1 : 0) : 0;
    const uint32_t part = PB ? field(q, P0, PB) : 0u;
    const uint32_t rot = RB ? field(q, R0, RB) : 0u;
    const uint32_t isb = ISB ? field(q, S0, ISB) : 0u;
    // endpoint k = 2 * subset + end, channels packed R | G << 8 | B << 16 | A << 24
    uint32_t E[2 * NS];
#pragma unroll
    for (int k = 0; k < 2 * NS; ++k) {
        uint32_t e = 0;
#pragma unroll
        for (int ch = 0; ch < 3; ++ch) e |= field(q, E0 + (ch * 2 * NS + k) * CB, CB) << (8 * ch);
        if constexpr (AB != 0) e |= field(q, A0 + k * AB, AB) << 24;
        if constexpr (PK == 1) e = (e << 1) | field(q, B0 + k, 1) * 0x01010101u;  // bytes < 128: no carries
        if constexpr (PK == 2) e = (e << 1) | field(q, B0 + k / 2, 1) * 0x01010101u;
        uint32_t a = 255u;
        if constexpr (NA != 0) a = widen1<NA>(e >> 24);
        E[k] = widen3<NC>(e & 0x00FFFFFFu) | a << 24;
    }
    // index streams, made uniform (IB bits per texel) by inserting the anchors' missing high bits
    uint64_t s1 = insert_zero(field64(q, I0, L1), IB - 1);
    uint32_t map = 0;
    if constexpr (NS == 2) {
        map = T.map[part];
        s1 = insert_zero(s1, T.anchors[part] * IB + IB - 1);
    } else if constexpr (NS == 3) {
        map = T.map[64 + part];
        const uint32_t an = T.anchors[64 + part];
        s1 = insert_zero(s1, (an & 255u) * IB + IB - 1);
        s1 = insert_zero(s1, (an >> 8) * IB + IB - 1);
    }
    uint64_t s2 = 0;
    if constexpr (IB2 != 0) s2 = insert_zero(field64(q, I0 + L1, L2), IB2 - 1);
    const uint32_t sel = rot == 0 ? 0x3210u : rot == 1 ? 0x0213u : rot == 2 ? 0x1230u : 0x2310u;
#pragma unroll 1
    for (int r = 0; r < 4; ++r) {
        uint32_t v[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            uint32_t e0 = E[0], e1 = E[1];
            if constexpr (NS >= 2) {
                const uint32_t s = (map >> (2 * c)) & 3u;
                if constexpr (NS == 2) {
                    e0 = s ? E[2] : E[0];
                    e1 = s ? E[3] : E[1];
                } else {
                    e0 = s == 0 ? E[0] : s == 1 ? E[2] : E[4];
                    e1 = s == 0 ? E[1] : s == 1 ? E[3] : E[5];
                }
            }
            const uint32_t w1 = weight_of<IB>((uint32_t)(s1 >> (IB * c)) & ((1u << IB) - 1u));
            uint32_t wc = w1, wa = w1;
            if constexpr (IB2 != 0) {
                const uint32_t w2 = weight_of<IB2>((uint32_t)(s2 >> (IB2 * c)) & ((1u << IB2) - 1u));
                wc = isb ? w2 : w1;  // the index-selection bit (mode 4) gives the colour the secondary set
                wa = isb ? w1 : w2;
            }
            // R and B in two 16-bit lanes: (64 - w) * 255 + w * 255 + 32 < 2^16, so the lanes never carry
            const uint32_t rb = (((64u - wc) * (e0 & 0x00FF00FFu) + wc * (e1 & 0x00FF00FFu) + 0x00200020u) >> 6) & 0x00FF00FFu;
            const uint32_t g = ((64u - wc) * ((e0 >> 8) & 0xFFu) + wc * ((e1 >> 8) & 0xFFu) + 32u) >> 6;
            const uint32_t a = ((64u - wa) * (e0 >> 24) + wa * (e1 >> 24) + 32u) >> 6;
            const uint32_t t = rb | g << 8 | a << 24;
            v[c] = RB ? __byte_perm(t, 0u, sel) : t;
        }
        *reinterpret_cast<uint4*>(out + r * pitch) = make_uint4(v[0], v[1], v[2], v[3]);
        map >>= 8;
        s1 >>= 4 * IB;
        if constexpr (IB2 != 0) s2 >>= 4 * IB2;
    }
}

__device__ __forceinline__ void decode_block(const uint4& q, const Bc7Tables& T, uint32_t* out, int pitch) {
    const uint32_t m8 = q.x & 0xFFu;
    switch (m8 ? __ffs(m8) - 1 : 8) {
        case 0: decode_mode<0>(q, T, out, pitch); break;
        case 1: decode_mode<1>(q, T, out, pitch); break;
        case 2: decode_mode<2>(q, T, out, pitch); break;
        case 3: decode_mode<3>(q, T, out, pitch); break;
        case 4: decode_mode<4>(q, T, out, pitch); break;
        case 5: decode_mode<5>(q, T, out, pitch); break;
        case 6: decode_mode<6>(q, T, out, pitch); break;
        case 7: decode_mode<7>(q, T, out, pitch); break;
        default:  // the reserved mode
            for (int r = 0; r < 4; ++r) *reinterpret_cast<uint4*>(out + r * pitch) = make_uint4(0u, 0u, 0u, 0u);
    }
}

__global__ void __launch_bounds__(kBc7Threads) k_bc7_decode(const Bc7Job job, const Bc7Tables tables) {
    __shared__ Bc7Tables T;
    __shared__ Bc7Level L[kBc7MaxLevels];
    __shared__ uint4 s_blk[kBc7Threads];
    __shared__ uint16_t s_src[kBc7Threads];
    __shared__ uint32_t s_count[10], s_off[10];
    __shared__ __align__(16) uint32_t s_out[4 * kTileBY][kStagePitch];
    const int tid = threadIdx.x;
    {
        const uint32_t* src = reinterpret_cast<const uint32_t*>(&tables);
        uint32_t* dst = reinterpret_cast<uint32_t*>(&T);
        for (uint32_t i = tid; i < sizeof(Bc7Tables) / 4; i += blockDim.x) dst[i] = src[i];
        const uint32_t* ls = reinterpret_cast<const uint32_t*>(job.L);
        uint32_t* ld = reinterpret_cast<uint32_t*>(L);
        for (uint32_t i = tid; i < sizeof(job.L) / 4; i += blockDim.x) ld[i] = ls[i];
        if (tid < 10) s_count[tid] = 0;
    }
    __syncthreads();
    const uint32_t tile = blockIdx.x;
    uint32_t l = 0;
    while (l + 1 < job.levels && tile >= L[l + 1].tile0) ++l;
    const Bc7Level& lv = L[l];
    const uint32_t lt = tile - lv.tile0;
    const uint32_t tbx = (lt % lv.tiles_x) * kTileBX, tby = (lt / lv.tiles_x) * kTileBY;
    // this thread's block, and its mode (9: outside the level)
    uint4 q = make_uint4(0u, 0u, 0u, 0u);
    uint32_t mode = 9;
    {
        const uint32_t bx = tbx + tid % kTileBX, by = tby + tid / kTileBX;
        if (bx < lv.bw && by < lv.bh) {
            q = __ldg(job.blocks + lv.block0 + (size_t)by * lv.bw + bx);
            const uint32_t m8 = q.x & 0xFFu;
            mode = m8 ? __ffs(m8) - 1 : 8;
        }
    }
    // counting sort of the tile's blocks by mode
    const uint32_t rank = atomicAdd(&s_count[mode], 1u);
    __syncthreads();
    if (tid == 0) {
        uint32_t acc = 0;
        for (int m = 0; m < 10; ++m) {
            s_off[m] = acc;
            acc += s_count[m];
        }
    }
    __syncthreads();
    const uint32_t pos = s_off[mode] + rank;
    s_blk[pos] = q;
    s_src[pos] = (uint16_t)tid;
    __syncthreads();
    // decode the sorted blocks into the staged tile
    {
        const uint32_t src = s_src[tid];
        const uint32_t sbx = src % kTileBX, sby = src / kTileBX;
        if (tbx + sbx < lv.bw && tby + sby < lv.bh) decode_block(s_blk[tid], T, &s_out[4 * sby][4 * sbx], kStagePitch);
    }
    __syncthreads();
    // the tile's texel rows, four texels per thread, consecutive threads on consecutive texels
    for (int i = tid; i < 4 * kTileBY * kTileBX; i += kBc7Threads) {
        const int r = i / kTileBX, g = i % kTileBX;
        const uint32_t y = 4 * tby + r, x = 4 * (tbx + g);
        if (y >= lv.h || x >= lv.w) continue;
        uint32_t* dst = job.texels + lv.texel0 + (size_t)y * lv.w + x;
        const uint4 v = *reinterpret_cast<const uint4*>(&s_out[r][4 * g]);
        if (lv.vec && x + 4 <= lv.w) {
            *reinterpret_cast<uint4*>(dst) = v;
        } else {
            dst[0] = v.x;
            if (x + 1 < lv.w) dst[1] = v.y;
            if (x + 2 < lv.w) dst[2] = v.z;
            if (x + 3 < lv.w) dst[3] = v.w;
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
        n += (((uint64_t)w + 3) / 4) * (((uint64_t)h + 3) / 4) * 16;
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
    uint64_t blocks_total = 0, tiles = 0;
    for (uint32_t l = 0; l < levels; ++l) {
        Bc7Level& lv = job.L[l];
        lv.w = std::max(1u, width >> l);
        lv.h = std::max(1u, height >> l);
        lv.bw = (uint32_t)(((uint64_t)lv.w + 3) / 4);  // 64-bit: no wrap near 2^32
        lv.bh = (uint32_t)(((uint64_t)lv.h + 3) / 4);
        lv.block0 = (uint32_t)blocks_total;
        lv.texel0 = level_off[l];
        lv.vec = (lv.w % 4 == 0 && lv.texel0 % 4 == 0 && reinterpret_cast<uintptr_t>(texels) % 16 == 0) ? 1u : 0u;
        lv.tiles_x = (lv.bw + kTileBX - 1) / kTileBX;
        lv.tile0 = (uint32_t)tiles;
        blocks_total += (uint64_t)lv.bw * lv.bh;
        tiles += (uint64_t)lv.tiles_x * ((lv.bh + kTileBY - 1) / kTileBY);
    }
    if (blocks_total >= 0xFFFFFFFFull || tiles >= 0x7FFFFFFFull) return cudaErrorInvalidValue;
    job.total_tiles = (uint32_t)tiles;
    k_bc7_decode<<<(uint32_t)tiles, kBc7Threads, 0, stream>>>(job, tables());
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
