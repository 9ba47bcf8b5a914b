// Planar YCbCr -> interleaved RGB24 at 1:1 scale, integer BT.601, for sm_103a.
// Restates crates/cli/src/terminal_preview.rs:7159-7236 (nearest chroma sample
// at x*cw/W, y*ch/H) and :7308-7330 (fixed-point matrix, full or limited range).
//
// A CTA converts 4096 consecutive pixels of one frame (16 per thread), stages
// the 12 KiB of RGB in shared memory and writes it out with coalesced 16-byte
// stores. Chroma column indices advance incrementally (x*cw/W without a
// division per pixel; cw <= W), and rows are recomputed only when a thread's
// run of 16 pixels crosses into the next row.
#include <cuda_runtime.h>

#include "kernels.h"

namespace mmr {

namespace {

constexpr int kRgbThreads = 256;
constexpr int kRgbPix = 16;
constexpr uint32_t kCtaPixels = kRgbThreads * kRgbPix;

__device__ __forceinline__ uint32_t clamp255(int32_t v) { return (uint32_t)(v < 0 ? 0 : v > 255 ? 255 : v); }

// Nearest-sample row of a plane of height ph for output row y of h rows.
__device__ __forceinline__ uint32_t near_row(uint32_t y, uint32_t ph, uint32_t h) {
    return min(y * ph / h, ph - 1);
}

struct Cursor {
    uint32_t col, rem;  // x * pw / w and its remainder
};

__device__ __forceinline__ Cursor cursor_at(uint32_t x, uint32_t pw, uint32_t w) {
    Cursor c;
    c.col = x * pw / w;
    c.rem = x * pw - c.col * w;
    return c;
}

__device__ __forceinline__ void cursor_step(Cursor &c, uint32_t pw, uint32_t w) {
    c.rem += pw;
    if (c.rem >= w) {
        c.rem -= w;
        c.col++;
    }
}

__global__ void __launch_bounds__(kRgbThreads) rgb_kernel(RgbLaunch L) {
    __shared__ uint32_t s_job;
    __shared__ __align__(16) uint32_t s_out[kRgbThreads * kRgbPix * 3 / 4];
    if (threadIdx.x == 0) {
        uint32_t lo = 0, hi = L.n_jobs;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (L.cta_first[mid] <= blockIdx.x) lo = mid;
            else hi = mid;
        }
        s_job = lo;
    }
    __syncthreads();
    const uint32_t job = s_job;
    const RgbJob &J = L.jobs[job];
    if (!L.item_ok[J.item]) return;
    const uint32_t W = J.w, npix = J.w * J.h;
    const uint32_t base = (blockIdx.x - L.cta_first[job]) * kCtaPixels;
    const uint32_t p0 = base + threadIdx.x * kRgbPix;
    uint32_t words[12];
#pragma unroll
    for (int q = 0; q < 12; q++) words[q] = 0;
    if (p0 < npix) {
        uint32_t y = p0 / W, x = p0 - y * W;
        const uint8_t *P = J.planes;
        const uint8_t *Yrow = P + (uint64_t)near_row(y, J.lh, J.h) * J.lw;
        const uint8_t *Brow = P + J.cb_off + (uint64_t)near_row(y, J.cbh, J.h) * J.cbw;
        const uint8_t *Rrow = P + J.cr_off + (uint64_t)near_row(y, J.crh, J.h) * J.crw;
        Cursor cb = cursor_at(x, J.cbw, W), cr = cursor_at(x, J.crw, W);
        // 16 luma samples in one load when they are contiguous and aligned
        uint4 yv = make_uint4(0, 0, 0, 0);
        const bool yvec = J.lw == W && J.lh == J.h && x + kRgbPix <= W && ((((uintptr_t)(Yrow + x)) & 15) == 0);
        if (yvec) yv = *reinterpret_cast<const uint4 *>(Yrow + x);
        const uint32_t yw[4] = {yv.x, yv.y, yv.z, yv.w};
#pragma unroll
        for (int i = 0; i < kRgbPix; i++) {
            if (p0 + i < npix) {
                const int32_t Y = yvec ? (int32_t)((yw[i >> 2] >> (8 * (i & 3))) & 0xff) : (int32_t)Yrow[x];
                uint32_t r, g, b;
                if (J.gray) {
                    r = g = b = (uint32_t)Y;
                } else {
                    const int32_t u = (int32_t)Brow[min(cb.col, J.cbw - 1)] - 128;
                    const int32_t v = (int32_t)Rrow[min(cr.col, J.crw - 1)] - 128;
                    if (J.limited) {
                        const int32_t yl = Y - 16 < 0 ? 0 : Y - 16;
                        r = clamp255((298 * yl + 409 * v + 128) >> 8);
                        g = clamp255((298 * yl - 100 * u - 208 * v + 128) >> 8);
                        b = clamp255((298 * yl + 516 * u + 128) >> 8);
                    } else {
                        r = clamp255(Y + ((359 * v + 128) >> 8));
                        g = clamp255(Y - ((88 * u + 183 * v + 128) >> 8));
                        b = clamp255(Y + ((454 * u + 128) >> 8));
                    }
                }
                words[(3 * i) >> 2] |= r << (8 * ((3 * i) & 3));
                words[(3 * i + 1) >> 2] |= g << (8 * ((3 * i + 1) & 3));
                words[(3 * i + 2) >> 2] |= b << (8 * ((3 * i + 2) & 3));
                if (++x == W) {
                    x = 0;
                    y++;
                    if (y < J.h) {
                        Yrow = P + (uint64_t)near_row(y, J.lh, J.h) * J.lw;
                        Brow = P + J.cb_off + (uint64_t)near_row(y, J.cbh, J.h) * J.cbw;
                        Rrow = P + J.cr_off + (uint64_t)near_row(y, J.crh, J.h) * J.crw;
                    }
                    cb.col = cb.rem = cr.col = cr.rem = 0;
                } else {
                    cursor_step(cb, J.cbw, W);
                    cursor_step(cr, J.crw, W);
                }
            }
        }
    }
    // 48 bytes per thread: three 16-byte stores, conflict-free (thread stride 3 x 16 B)
    uint4 *so = reinterpret_cast<uint4 *>(s_out) + threadIdx.x * 3;
    so[0] = make_uint4(words[0], words[1], words[2], words[3]);
    so[1] = make_uint4(words[4], words[5], words[6], words[7]);
    so[2] = make_uint4(words[8], words[9], words[10], words[11]);
    __syncthreads();
    const uint32_t nbytes = min(npix - base, kCtaPixels) * 3;
    uint8_t *dst = J.out + (uint64_t)base * 3;
    const uint8_t *src = reinterpret_cast<const uint8_t *>(s_out);
    if ((((uintptr_t)dst) & 15) == 0) {
        for (uint32_t o = threadIdx.x * 16; o + 16 <= nbytes; o += kRgbThreads * 16)
            *reinterpret_cast<uint4 *>(dst + o) = *reinterpret_cast<const uint4 *>(src + o);
        for (uint32_t o = (nbytes & ~15u) + threadIdx.x; o < nbytes; o += kRgbThreads) dst[o] = src[o];
    } else {
        for (uint32_t o = threadIdx.x; o < nbytes; o += kRgbThreads) dst[o] = src[o];
    }
}

}  // namespace

uint32_t rgb_ctas(uint32_t w, uint32_t h) { return (uint32_t)(((uint64_t)w * h + kCtaPixels - 1) / kCtaPixels); }

void launch_rgb(const RgbLaunch &L, cudaStream_t s) {
    if (L.n_ctas == 0) return;
    rgb_kernel<<<L.n_ctas, kRgbThreads, 0, s>>>(L);
}

}  // namespace mmr
