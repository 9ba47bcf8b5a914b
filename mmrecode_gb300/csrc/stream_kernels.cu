// Marker candidates of a whole media stream (sm_103a).
//
// The reference CLI frames a file of concatenated JFIF images by running
// parse_jpeg on what remains after each image (crates/cli/src/main.rs:1555-1572);
// parse_jpeg ends each entropy-coded segment at the first 0xFF run followed by a
// code that is not 0x00 (stuffing) or RST0..7 (crates/codecs/mjpeg/src/parser.rs:
// 373-414). Those bytes are 99% of the file, so they are scanned here, once, for
// every position q whose byte is 0xFF and whose next byte is neither 0x00, 0xFF
// nor 0xD0..0xD7: the last 0xFF of each such run. The first candidate at or after
// an entropy-coded segment's start is where parse_jpeg stops it; the host walks
// the few header bytes of each image itself.
//
// A thread tests 16-byte groups with word-wide byte tests (a borrow test for any
// 0xFF, exact zero-byte masks where there is one), four loads in flight at a
// time; a group with a candidate (a few per image) appends its positions with an
// atomic. HBM-bound: the stream is read once.
#include <cuda_runtime.h>

#include <cstdint>

#include "stream.h"

namespace mmr {
namespace {

// Group g of the stream (16 bytes from 16 g), bytes past the end read as 0x00.
__device__ __forceinline__ uint4 load_group(const uint8_t *__restrict__ in, unsigned long long len, bool aligned,
                                            unsigned long long g) {
    const unsigned long long base = g * 16;
    if (aligned && base + 16 <= len) return __ldcs(reinterpret_cast<const uint4 *>(in) + g);
    uint32_t w[4] = {0, 0, 0, 0};
#pragma unroll
    for (int b = 0; b < 16; b++)
        if (base + b < len) w[b >> 2] |= (uint32_t)in[base + b] << (8 * (b & 3));
    return make_uint4(w[0], w[1], w[2], w[3]);
}

// Appends the candidates among the 16 bytes at `base` (v: those bytes).
__device__ __forceinline__ void scan_group(const uint8_t *__restrict__ in, unsigned long long len,
                                           unsigned long long base, uint4 v, unsigned long long *__restrict__ out,
                                           uint32_t cap, uint32_t *__restrict__ count) {
    if (!(any_ff(v.x) | any_ff(v.y) | any_ff(v.z) | any_ff(v.w))) return;
    // the byte after the group matters only when the group ends in 0xFF
    const uint32_t w[5] = {v.x, v.y, v.z, v.w, (v.w >> 24) == 0xffu && base + 16 < len ? (uint32_t)in[base + 16] : 0u};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const uint32_t ff = zero_bytes(~w[k]);
        if (!ff) continue;
        // little-endian: byte b of w[k] is stream byte base + 4k + b; its successor is
        // byte b + 1, or byte 0 of the next word. A successor 0x00 (stuffing), 0xFF
        // (fill) or 0xD0..0xD7 (RSTn) keeps the 0xFF from ending a scan.
        const uint32_t next = (w[k] >> 8) | (w[k + 1] << 24);
        const uint32_t excluded =
            zero_bytes(next) | zero_bytes(~next) | zero_bytes((next & 0xf8f8f8f8u) ^ 0xd0d0d0d0u);
        uint32_t hit = ff & ~excluded;
        while (hit) {
            const int bit = __ffs(hit) - 1;
            hit &= hit - 1;
            const unsigned long long q = base + 4 * k + (bit >> 3);
            if (q + 1 >= len) continue;  // no code byte follows
            const uint32_t slot = atomicAdd(count, 1u);
            if (slot < cap) out[slot] = q;
        }
    }
}

constexpr int kGroupsPerThread = 4;  // 16-byte loads in flight per thread and iteration

__global__ void __launch_bounds__(256) marker_candidates_kernel(const uint8_t *__restrict__ in,
                                                                unsigned long long len,
                                                                unsigned long long *__restrict__ out, uint32_t cap,
                                                                uint32_t *__restrict__ count) {
    const unsigned long long groups = (len + 15) / 16;
    const bool aligned = (reinterpret_cast<uintptr_t>(in) & 15) == 0;
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long g0 = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; g0 < groups;
         g0 += stride * kGroupsPerThread) {
        uint4 v[kGroupsPerThread];
#pragma unroll
        for (int k = 0; k < kGroupsPerThread; k++) v[k] = load_group(in, len, aligned, g0 + k * stride);
#pragma unroll
        for (int k = 0; k < kGroupsPerThread; k++) scan_group(in, len, (g0 + k * stride) * 16, v[k], out, cap, count);
    }
}

}  // namespace

void launch_marker_candidates(const uint8_t *in, uint64_t len, uint64_t *out, uint32_t cap, uint32_t *count,
                              int sm_count, cudaStream_t s) {
    const uint64_t groups = (len + 15) / 16;
    if (!groups) return;
    const uint64_t want = (groups + 256 * kGroupsPerThread - 1) / (256 * kGroupsPerThread);
    const uint64_t full = (uint64_t)(sm_count > 0 ? sm_count : 152) * 8;  // 8 CTAs of 256 per SM
    const unsigned grid = (unsigned)(want < full ? want : full);
    marker_candidates_kernel<<<grid, 256, 0, s>>>(in, len, reinterpret_cast<unsigned long long *>(out), cap, count);
}

}  // namespace mmr
