// ORACLE — test infrastructure only. Scalar restatement of BC7 block decoding
// (the BPTC format: Khronos Data Format Specification, "BPTC Compressed Texture
// Image Formats"; Microsoft's "BC7 Format" documentation for Direct3D 11), the
// format of every image the reference uploads (src/Engine/Graphics.cpp:3632-3647:
// VK_FORMAT_BC7_SRGB_BLOCK for colour, metallic-roughness and mixmap images,
// VK_FORMAT_BC7_UNORM_BLOCK for normal maps), whose decoding the reference leaves
// to the GPU's texture unit. Pinned against that decoder: tests/golden/bc7_hw.npz
// holds blocks of every mode and the texels the GB300 texture unit decoded them
// to (tests/golden/make_bc7_golden.py).
#include <stdint.h>
#include <string.h>

#include <algorithm>

#include "oracle.h"

namespace {

// Per mode: subsets, partition bits, rotation bits, index-selection bits, colour
// bits, alpha bits, per-endpoint P-bits, shared P-bits, index bits, secondary
// index bits (the mode table of the format).
struct Bc7Mode {
    int ns, pb, rb, isb, cb, ab, epb, spb, ib, ib2;
};
constexpr Bc7Mode kModes[8] = {
    {3, 4, 0, 0, 4, 0, 1, 0, 3, 0}, {2, 6, 0, 0, 6, 0, 0, 1, 3, 0}, {3, 6, 0, 0, 5, 0, 0, 0, 2, 0},
    {2, 6, 0, 0, 7, 0, 1, 0, 2, 0}, {1, 0, 2, 1, 5, 6, 0, 0, 2, 3}, {1, 0, 2, 0, 7, 8, 0, 0, 2, 2},
    {1, 0, 0, 0, 7, 7, 1, 0, 4, 0}, {2, 6, 0, 0, 5, 5, 1, 0, 2, 0},
};

// Two-subset partitions: bit i set = texel i (row-major in the 4x4 block) is in subset 1.
constexpr uint16_t kPartition2[64] = {
    0xCCCC, 0x8888, 0xEEEE, 0xECC8, 0xC880, 0xFEEC, 0xFEC8, 0xEC80, 0xC800, 0xFFEC, 0xFE80, 0xE800, 0xFFE8,
    0xFF00, 0xFFF0, 0xF000, 0xF710, 0x008E, 0x7100, 0x08CE, 0x008C, 0x7310, 0x3100, 0x8CCE, 0x088C, 0x3110,
    0x6666, 0x366C, 0x17E8, 0x0FF0, 0x718E, 0x399C, 0xAAAA, 0xF0F0, 0x5A5A, 0x33CC, 0x3C3C, 0x55AA, 0x9696,
    0xA55A, 0x73CE, 0x13C8, 0x324C, 0x3BDC, 0x6996, 0xC33C, 0x9966, 0x0660, 0x0272, 0x04E4, 0x4E40, 0x2720,
    0xC936, 0x936C, 0x39C6, 0x639C, 0x9336, 0x9CC6, 0x817E, 0xE718, 0xCCF0, 0x0FCC, 0x7744, 0xEE22,
};

// Three-subset partitions, one row of four subset numbers per line.
constexpr uint8_t kPartition3[64][16] = {
    {0, 0, 1, 1, 0, 0, 1, 1, 0, 2, 2, 1, 2, 2, 2, 2}, {0, 0, 0, 1, 0, 0, 1, 1, 2, 2, 1, 1, 2, 2, 2, 1},
    {0, 0, 0, 0, 2, 0, 0, 1, 2, 2, 1, 1, 2, 2, 1, 1}, {0, 2, 2, 2, 0, 0, 2, 2, 0, 0, 1, 1, 0, 1, 1, 1},
    {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 2, 2, 1, 1, 2, 2}, {0, 0, 1, 1, 0, 0, 1, 1, 0, 0, 2, 2, 0, 0, 2, 2},
    {0, 0, 2, 2, 0, 0, 2, 2, 1, 1, 1, 1, 1, 1, 1, 1}, {0, 0, 1, 1, 0, 0, 1, 1, 2, 2, 1, 1, 2, 2, 1, 1},
    {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2}, {0, 0, 0, 0, 1, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2},
    {0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2, 2, 2}, {0, 0, 1, 2, 0, 0, 1, 2, 0, 0, 1, 2, 0, 0, 1, 2},
    {0, 1, 1, 2, 0, 1, 1, 2, 0, 1, 1, 2, 0, 1, 1, 2}, {0, 1, 2, 2, 0, 1, 2, 2, 0, 1, 2, 2, 0, 1, 2, 2},
    {0, 0, 1, 1, 0, 1, 1, 2, 1, 1, 2, 2, 1, 2, 2, 2}, {0, 0, 1, 1, 2, 0, 0, 1, 2, 2, 0, 0, 2, 2, 2, 0},
    {0, 0, 0, 1, 0, 0, 1, 1, 0, 1, 1, 2, 1, 1, 2, 2}, {0, 1, 1, 1, 0, 0, 1, 1, 2, 0, 0, 1, 2, 2, 0, 0},
    {0, 0, 0, 0, 1, 1, 2, 2, 1, 1, 2, 2, 1, 1, 2, 2}, {0, 0, 2, 2, 0, 0, 2, 2, 0, 0, 2, 2, 1, 1, 1, 1},
    {0, 1, 1, 1, 0, 1, 1, 1, 0, 2, 2, 2, 0, 2, 2, 2}, {0, 0, 0, 1, 0, 0, 0, 1, 2, 2, 2, 1, 2, 2, 2, 1},
    {0, 0, 0, 0, 0, 0, 1, 1, 0, 1, 2, 2, 0, 1, 2, 2}, {0, 0, 0, 0, 1, 1, 0, 0, 2, 2, 1, 0, 2, 2, 1, 0},
    {0, 1, 2, 2, 0, 1, 2, 2, 0, 0, 1, 1, 0, 0, 0, 0}, {0, 0, 1, 2, 0, 0, 1, 2, 1, 1, 2, 2, 2, 2, 2, 2},
    {0, 1, 1, 0, 1, 2, 2, 1, 1, 2, 2, 1, 0, 1, 1, 0}, {0, 0, 0, 0, 0, 1, 1, 0, 1, 2, 2, 1, 1, 2, 2, 1},
    {0, 0, 2, 2, 1, 1, 0, 2, 1, 1, 0, 2, 0, 0, 2, 2}, {0, 1, 1, 0, 0, 1, 1, 0, 2, 0, 0, 2, 2, 2, 2, 2},
    {0, 0, 1, 1, 0, 1, 2, 2, 0, 1, 2, 2, 0, 0, 1, 1}, {0, 0, 0, 0, 2, 0, 0, 0, 2, 2, 1, 1, 2, 2, 2, 1},
    {0, 0, 0, 0, 0, 0, 0, 2, 1, 1, 2, 2, 1, 2, 2, 2}, {0, 2, 2, 2, 0, 0, 2, 2, 0, 0, 1, 2, 0, 0, 1, 1},
    {0, 0, 1, 1, 0, 0, 1, 2, 0, 0, 2, 2, 0, 2, 2, 2}, {0, 1, 2, 0, 0, 1, 2, 0, 0, 1, 2, 0, 0, 1, 2, 0},
    {0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 0, 0, 0, 0}, {0, 1, 2, 0, 1, 2, 0, 1, 2, 0, 1, 2, 0, 1, 2, 0},
    {0, 1, 2, 0, 2, 0, 1, 2, 1, 2, 0, 1, 0, 1, 2, 0}, {0, 0, 1, 1, 2, 2, 0, 0, 1, 1, 2, 2, 0, 0, 1, 1},
    {0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 0, 0, 0, 0, 1, 1}, {0, 1, 0, 1, 0, 1, 0, 1, 2, 2, 2, 2, 2, 2, 2, 2},
    {0, 0, 0, 0, 0, 0, 0, 0, 2, 1, 2, 1, 2, 1, 2, 1}, {0, 0, 2, 2, 1, 1, 2, 2, 0, 0, 2, 2, 1, 1, 2, 2},
    {0, 0, 2, 2, 0, 0, 1, 1, 0, 0, 2, 2, 0, 0, 1, 1}, {0, 2, 2, 0, 1, 2, 2, 1, 0, 2, 2, 0, 1, 2, 2, 1},
    {0, 1, 0, 1, 2, 2, 2, 2, 2, 2, 2, 2, 0, 1, 0, 1}, {0, 0, 0, 0, 2, 1, 2, 1, 2, 1, 2, 1, 2, 1, 2, 1},
    {0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 0, 1, 2, 2, 2, 2}, {0, 2, 2, 2, 0, 1, 1, 1, 0, 2, 2, 2, 0, 1, 1, 1},
    {0, 0, 0, 2, 1, 1, 1, 2, 0, 0, 0, 2, 1, 1, 1, 2}, {0, 0, 0, 0, 2, 1, 1, 2, 2, 1, 1, 2, 2, 1, 1, 2},
    {0, 2, 2, 2, 0, 1, 1, 1, 0, 1, 1, 1, 0, 2, 2, 2}, {0, 0, 0, 2, 1, 1, 1, 2, 1, 1, 1, 2, 0, 0, 0, 2},
    {0, 1, 1, 0, 0, 1, 1, 0, 0, 1, 1, 0, 2, 2, 2, 2}, {0, 0, 0, 0, 0, 0, 0, 0, 2, 1, 1, 2, 2, 1, 1, 2},
    {0, 1, 1, 0, 0, 1, 1, 0, 2, 2, 2, 2, 2, 2, 2, 2}, {0, 0, 2, 2, 0, 0, 1, 1, 0, 0, 1, 1, 0, 0, 2, 2},
    {0, 0, 2, 2, 1, 1, 2, 2, 1, 1, 2, 2, 0, 0, 2, 2}, {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 2, 1, 1, 2},
    {0, 0, 0, 2, 0, 0, 0, 1, 0, 0, 0, 2, 0, 0, 0, 1}, {0, 2, 2, 2, 1, 2, 2, 2, 0, 2, 2, 2, 1, 2, 2, 2},
    {0, 1, 0, 1, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2}, {0, 1, 1, 1, 2, 0, 1, 1, 2, 2, 0, 1, 2, 2, 2, 0},
};

// Anchor texels (their index has an implicit leading zero bit): subset 1 of the
// two-subset partitions, subsets 1 and 2 of the three-subset partitions. Texel 0
// anchors subset 0 always.
constexpr uint8_t kAnchor2[64] = {
    15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 15, 2,  8,  2,  2,  8,  8,  15, 2,  8,  2,  2,
    8,  8,  2,  2,  15, 15, 6,  8,  2,  8,  15, 15, 2,  8,  2,  2,  2,  15, 15, 6,  6,  2,  6,  8,  15, 15, 2,  2,
    15, 15, 15, 15, 15, 2,  2,  15,
};
constexpr uint8_t kAnchor3a[64] = {
    3,  3,  15, 15, 8,  3,  15, 15, 8,  8,  6,  6,  6,  5,  3,  3,  3,  3,  8,  15, 3,  3,  6,  10, 5,  8,  8,  6,
    8,  5,  15, 15, 8,  15, 3,  5,  6,  10, 8,  15, 15, 3,  15, 5,  15, 15, 15, 15, 3,  15, 5,  5,  5,  8,  5,  10,
    5,  10, 8,  13, 15, 12, 3,  3,
};
constexpr uint8_t kAnchor3b[64] = {
    15, 8,  8,  3,  15, 15, 3,  8,  15, 15, 15, 15, 15, 15, 15, 8,  15, 8,  15, 3,  15, 8,  15, 8,  3,  15, 6,  10,
    15, 15, 10, 8,  15, 3,  15, 10, 10, 8,  9,  10, 6,  15, 8,  15, 3,  6,  6,  8,  15, 3,  15, 15, 15, 15, 15, 15,
    15, 15, 15, 15, 3,  15, 15, 8,
};

// Interpolation weights (out of 64) for 2-, 3- and 4-bit indices.
constexpr int kWeights2[4] = {0, 21, 43, 64};
constexpr int kWeights3[8] = {0, 9, 18, 27, 37, 46, 55, 64};
constexpr int kWeights4[16] = {0, 4, 9, 13, 17, 21, 26, 30, 34, 38, 43, 47, 51, 55, 60, 64};

const int* weights_for(int bits) { return bits == 2 ? kWeights2 : bits == 3 ? kWeights3 : kWeights4; }

// The block's 128 bits, read least significant bit first.
struct BitReader {
    const uint8_t* b;
    int pos = 0;
    int read(int n) {
        int v = 0;
        for (int i = 0; i < n; ++i, ++pos) v |= ((b[pos >> 3] >> (pos & 7)) & 1) << i;
        return v;
    }
};

int subset_of(int ns, int partition, int texel) {
    if (ns == 1) return 0;
    if (ns == 2) return (kPartition2[partition] >> texel) & 1;
    return kPartition3[partition][texel];
}

bool is_anchor(int ns, int partition, int texel) {
    if (texel == 0) return true;
    if (ns == 2) return texel == kAnchor2[partition];
    if (ns == 3) return texel == kAnchor3a[partition] || texel == kAnchor3b[partition];
    return false;
}

// An n-bit endpoint value widened to 8 bits by replicating its high bits.
int expand(int v, int n) { return n >= 8 ? v : (v << (8 - n)) | (v >> (2 * n - 8)); }

}  // namespace

extern "C" void oracle_bc7_block(const uint8_t block[16], uint8_t out[64]) {
    int mode = 0;
    while (mode < 8 && !((block[0] >> mode) & 1)) ++mode;
    if (mode == 8) {  // reserved mode: every channel of every texel is zero
        memset(out, 0, 64);
        return;
    }
    const Bc7Mode& m = kModes[mode];
    BitReader br{block};
    br.read(mode + 1);
    const int partition = br.read(m.pb);
    const int rotation = br.read(m.rb);
    const int isb = br.read(m.isb);
    int ep[3][2][4] = {};  // [subset][endpoint][channel]
    for (int ch = 0; ch < 3; ++ch)
        for (int s = 0; s < m.ns; ++s)
            for (int e = 0; e < 2; ++e) ep[s][e][ch] = br.read(m.cb);
    if (m.ab)
        for (int s = 0; s < m.ns; ++s)
            for (int e = 0; e < 2; ++e) ep[s][e][3] = br.read(m.ab);
    int cbits = m.cb, abits = m.ab;
    if (m.epb) {
        for (int s = 0; s < m.ns; ++s)
            for (int e = 0; e < 2; ++e) {
                const int p = br.read(1);
                for (int ch = 0; ch < 4; ++ch) ep[s][e][ch] = (ep[s][e][ch] << 1) | p;
            }
        ++cbits;
        if (abits) ++abits;
    } else if (m.spb) {
        for (int s = 0; s < m.ns; ++s) {
            const int p = br.read(1);
            for (int e = 0; e < 2; ++e)
                for (int ch = 0; ch < 4; ++ch) ep[s][e][ch] = (ep[s][e][ch] << 1) | p;
        }
        ++cbits;
        if (abits) ++abits;
    }
    for (int s = 0; s < m.ns; ++s)
        for (int e = 0; e < 2; ++e) {
            for (int ch = 0; ch < 3; ++ch) ep[s][e][ch] = expand(ep[s][e][ch], cbits);
            ep[s][e][3] = abits ? expand(ep[s][e][3], abits) : 255;
        }
    int idx[16], idx2[16] = {};
    for (int i = 0; i < 16; ++i) idx[i] = br.read(m.ib - (is_anchor(m.ns, partition, i) ? 1 : 0));
    if (m.ib2)
        for (int i = 0; i < 16; ++i) idx2[i] = br.read(m.ib2 - (i == 0 ? 1 : 0));
    for (int i = 0; i < 16; ++i) {
        const int s = subset_of(m.ns, partition, i);
        int wc, wa;
        if (!m.ib2) {
            wc = wa = weights_for(m.ib)[idx[i]];
        } else if (!isb) {
            wc = weights_for(m.ib)[idx[i]];
            wa = weights_for(m.ib2)[idx2[i]];
        } else {
            wc = weights_for(m.ib2)[idx2[i]];
            wa = weights_for(m.ib)[idx[i]];
        }
        int px[4];
        for (int ch = 0; ch < 4; ++ch) {
            const int w = ch < 3 ? wc : wa;
            px[ch] = ((64 - w) * ep[s][0][ch] + w * ep[s][1][ch] + 32) >> 6;
        }
        if (rotation) std::swap(px[3], px[rotation - 1]);
        for (int ch = 0; ch < 4; ++ch) out[4 * i + ch] = (uint8_t)px[ch];
    }
}

extern "C" int oracle_bc7_decode(const uint8_t* blocks, uint32_t width, uint32_t height, uint8_t* rgba) {
    if (!blocks || !rgba || width == 0 || height == 0) return 3;
    const uint32_t bw = (uint32_t)(((uint64_t)width + 3) / 4), bh = (uint32_t)(((uint64_t)height + 3) / 4);
    uint8_t px[64];
    for (uint32_t by = 0; by < bh; ++by)
        for (uint32_t bx = 0; bx < bw; ++bx) {
            oracle_bc7_block(blocks + 16 * ((size_t)by * bw + bx), px);
            for (uint32_t ty = 0; ty < 4; ++ty)
                for (uint32_t tx = 0; tx < 4; ++tx) {
                    const uint32_t x = 4 * bx + tx, y = 4 * by + ty;
                    if (x < width && y < height) memcpy(rgba + 4 * ((size_t)y * width + x), px + 4 * (4 * ty + tx), 4);
                }
        }
    return 0;
}
