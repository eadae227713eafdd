// Device helpers shared by the raster and shading kernels. These implement the
// renderer's fp32 geometry contract; the translation units that include this
// file are compiled with -fmad=false so that every fused multiply-add is an
// explicit fmaf() and every other product and sum rounds on its own.
#pragma once

#include "rz_internal.h"

namespace rz {

// C = A * B for column-major 4x4 matrices; element (c, r) is the fma chain
// A[0][r]*B[c][0] -> +A[1][r]*B[c][1] -> +A[2][r]*B[c][2] -> +A[3][r]*B[c][3].
// (mul(sd.viewproj, worldMat) of src/shaders/basic.slang:116 and
//  mul(sd.shadowProjNear, worldMat) of src/shaders/shadow.slang:17.)
__device__ __forceinline__ void mat4_mul(const float* __restrict__ A, const float* __restrict__ B, float* __restrict__ C) {
#pragma unroll
    for (int c = 0; c < 4; ++c) {
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            float acc = A[0 * 4 + r] * B[c * 4 + 0];
            acc = fmaf(A[1 * 4 + r], B[c * 4 + 1], acc);
            acc = fmaf(A[2 * 4 + r], B[c * 4 + 2], acc);
            acc = fmaf(A[3 * 4 + r], B[c * 4 + 3], acc);
            C[c * 4 + r] = acc;
        }
    }
}

// clip = M * (x, y, z, 1): fma(M0r, x, M3r) -> fma(M1r, y, .) -> fma(M2r, z, .).
__device__ __forceinline__ float4 transform_point(const float* __restrict__ M, float x, float y, float z) {
    float4 o;
    o.x = fmaf(M[8], z, fmaf(M[4], y, fmaf(M[0], x, M[12])));
    o.y = fmaf(M[9], z, fmaf(M[5], y, fmaf(M[1], x, M[13])));
    o.z = fmaf(M[10], z, fmaf(M[6], y, fmaf(M[2], x, M[14])));
    o.w = fmaf(M[11], z, fmaf(M[7], y, fmaf(M[3], x, M[15])));
    return o;
}

// Index of the draw whose triangle range holds `tri` (draws sorted by tri_base).
__device__ __forceinline__ uint32_t find_draw(const DrawRec* __restrict__ draws, uint32_t n, uint32_t tri) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&draws[mid].tri_base) <= tri) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Thread `tid` of `stride` threads' share of zeroing n bytes at ptr: 16-byte
// stores on the 16-byte-aligned body, byte stores on the unaligned head and
// tail, so any start address and size is safe.
__device__ __forceinline__ void zero_share(void* ptr, size_t n, size_t tid, size_t stride) {
    unsigned char* base = static_cast<unsigned char*>(ptr);
    size_t head = (16 - ((size_t)base & 15)) & 15;
    if (head > n) head = n;
    if (tid < head) base[tid] = 0;
    const size_t n16 = (n - head) / 16;
    uint4* body = reinterpret_cast<uint4*>(base + head);
    for (size_t i = tid; i < n16; i += stride) body[i] = make_uint4(0u, 0u, 0u, 0u);
    const size_t done = head + n16 * 16;
    if (tid < n - done) base[done + tid] = 0;
}

// This thread's share of zeroing every range of L (all threads of the grid).
__device__ __forceinline__ void clear_share(const ClearList& L) {
    const size_t tid = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (int b = 0; b < L.count; ++b) zero_share(L.ptr[b], L.bytes[b], tid, stride);
}

}  // namespace rz
