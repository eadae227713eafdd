// Reader for the .dds images of Rosy's assets: rz_dds_read / rz_dds_parse.
//
// The engine opens every asset image with dds::readFile (src/Engine/Graphics.cpp:
// 3605-3613; src/libs/dds.hpp:581-596), which reads the file and hands it to
// dds::readImage (dds.hpp:409-574), and uploads the mip spans it returns as a
// BC7 image (Graphics.cpp:3632-3647). This reader performs the same steps on
// the file layout (magic "DDS ", the 124-byte header, the 20-byte DX10 header
// when the pixel format's FourCC carries "DX10", then the levels' blocks) with
// the same results, plus one check the reference lacks: every level the header
// announces must lie inside the file (readImage builds spans past a short
// file's end). Only BC7 payloads are accepted, since the engine uploads every
// image as BC7.
#include <cstdio>
#include <cstring>
#include <vector>

#include "../../include/rosy_gb300.h"

struct rz_dds {
    std::vector<unsigned char> bytes;
    rz_dds_info info{};
};

namespace {

constexpr uint32_t kMagicDds = 0x20534444u;   // "DDS "
constexpr uint32_t kFourCcDx10 = 0x30315844u; // "DX10"
constexpr uint32_t kPfAlphaPixels = 0x1u;
constexpr uint32_t kPfFourCc = 0x4u;
constexpr uint64_t kHeaderEnd = 4 + 124;      // magic + header
constexpr uint64_t kDx10End = kHeaderEnd + 20;
constexpr uint32_t kDxgiBc7Typeless = 97, kDxgiBc7Srgb = 99;

uint32_t u32_at(const unsigned char* p, uint64_t off) {
    return (uint32_t)p[off] | (uint32_t)p[off + 1] << 8 | (uint32_t)p[off + 2] << 16 | (uint32_t)p[off + 3] << 24;
}

// Fills `info` from the file in `b`; data points into `b`.
int parse(const std::vector<unsigned char>& b, rz_dds_info& info) {
    const uint64_t size = b.size();
    if (size < kHeaderEnd) return RZ_READ_FAILED;                 // ReadResult::Failure
    const unsigned char* p = b.data();
    if (u32_at(p, 0) != kMagicDds) return RZ_READ_FAILED;         // ReadResult::Failure
    const uint32_t height = u32_at(p, 4 + 8), width = u32_at(p, 4 + 12), mip_count = u32_at(p, 4 + 24);
    const uint32_t pf_flags = u32_at(p, 4 + 72 + 4), four_cc = u32_at(p, 4 + 72 + 8);
    // a DX10 header follows when the flags carry FourCC and the FourCC carries
    // every bit of "DX10" (the reference's bit test, dds.hpp:426-427)
    if (!((pf_flags & kPfFourCc) == kPfFourCc && (four_cc & kFourCcDx10) == kFourCcDx10))
        return RZ_INVALID_ARGUMENT;  // legacy FourCC / bit-mask formats are never BC7: UnsupportedFormat
    if (size < kDx10End) return RZ_READ_FAILED;                   // ReadResult::InvalidSize
    const uint32_t dxgi = u32_at(p, kHeaderEnd), array_size = u32_at(p, kHeaderEnd + 12);
    if (dxgi < kDxgiBc7Typeless || dxgi > kDxgiBc7Srgb) return RZ_INVALID_ARGUMENT;  // not BC7
    if (array_size > 1) return RZ_INVALID_ARGUMENT;               // ReadResult::UnsupportedFormat
    if (array_size == 0 || width == 0 || height == 0) return RZ_READ_FAILED;  // no image to read
    const uint32_t levels = mip_count > 1 ? mip_count : 1;
    const uint64_t avail = size - kDx10End;
    uint64_t total = 0;
    uint32_t w = width, h = height;
    for (uint32_t l = 0; l < levels; ++l) {
        const uint64_t bw = ((uint64_t)w + 3) / 4, bh = ((uint64_t)h + 3) / 4;  // 64-bit: no wrap near 2^32
        total += (bw > 1 ? bw : 1) * (bh > 1 ? bh : 1) * 16;
        if (total > avail) return RZ_READ_FAILED;                 // a level past the end of the file
        w = w / 2 > 1 ? w / 2 : 1;
        h = h / 2 > 1 ? h / 2 : 1;
    }
    info.width = width;
    info.height = height;
    info.levels = levels;
    info.dxgi_format = dxgi;
    info.supports_alpha = (pf_flags & kPfAlphaPixels) ? 1u : 0u;
    info.reserved = 0;
    info.data_bytes = total;
    info.data = p + kDx10End;
    return RZ_OK;
}

int finish(std::vector<unsigned char>&& bytes, rz_dds** out) {
    rz_dds* d = new rz_dds();
    d->bytes = std::move(bytes);
    const int rc = parse(d->bytes, d->info);
    if (rc != RZ_OK) {
        delete d;
        return rc;
    }
    *out = d;
    return RZ_OK;
}

}  // namespace

extern "C" {

int rz_dds_read(const char* path, rz_dds** out) {
    if (!path || !out) return RZ_INVALID_ARGUMENT;
    *out = nullptr;
    FILE* f = std::fopen(path, "rb");
    if (!f) return RZ_OPEN_FAILED;
    std::vector<unsigned char> bytes;
    unsigned char chunk[1 << 16];
    size_t n;
    while ((n = std::fread(chunk, 1, sizeof(chunk), f)) > 0) bytes.insert(bytes.end(), chunk, chunk + n);
    const bool err = std::ferror(f) != 0;
    std::fclose(f);
    if (err) return RZ_READ_FAILED;
    return finish(std::move(bytes), out);
}

int rz_dds_parse(const void* bytes, uint64_t size, rz_dds** out) {
    if (!out || (size && !bytes)) return RZ_INVALID_ARGUMENT;
    *out = nullptr;
    const unsigned char* b = static_cast<const unsigned char*>(bytes);
    return finish(std::vector<unsigned char>(b, b + size), out);
}

void rz_dds_free(rz_dds* image) { delete image; }

int rz_dds_get_info(const rz_dds* image, rz_dds_info* out) {
    if (!image || !out) return RZ_INVALID_ARGUMENT;
    *out = image->info;
    return RZ_OK;
}

}  // extern "C"
