// Planar YCbCr -> interleaved RGB24 at 1:1 scale, integer BT.601, for sm_103a.
// Restates crates/cli/src/terminal_preview.rs:7159-7236 (nearest chroma sample
// at x*cw/W, y*ch/H) and :7308-7330 (fixed-point matrix, full or limited range).
#include <cuda_runtime.h>

#include "kernels.h"

namespace mmr {

namespace {

__device__ __forceinline__ uint8_t clamp255(int32_t v) { return (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v); }

__global__ void rgb_kernel(RgbLaunch L) {
    uint64_t gp = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gp >= L.n_pixels) return;
    uint32_t lo = 0, hi = L.n_jobs;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (L.first[mid] <= gp) lo = mid;
        else hi = mid;
    }
    const RgbJob &J = L.jobs[lo];
    if (!L.item_ok[J.item]) return;
    uint64_t local = gp - L.first[lo];
    uint32_t y = (uint32_t)(local / J.w), x = (uint32_t)(local % J.w);
    uint8_t *o = J.out + local * 3;
    if (J.gray) {
        uint8_t v = J.planes[(uint64_t)y * J.lw + x];
        o[0] = v;
        o[1] = v;
        o[2] = v;
        return;
    }
    uint32_t ly = (uint32_t)min((uint64_t)y * J.lh / J.h, (uint64_t)J.lh - 1);
    uint32_t bx = (uint32_t)min((uint64_t)x * J.cbw / J.w, (uint64_t)J.cbw - 1);
    uint32_t by = (uint32_t)min((uint64_t)y * J.cbh / J.h, (uint64_t)J.cbh - 1);
    uint32_t rx = (uint32_t)min((uint64_t)x * J.crw / J.w, (uint64_t)J.crw - 1);
    uint32_t ry = (uint32_t)min((uint64_t)y * J.crh / J.h, (uint64_t)J.crh - 1);
    int32_t Y = J.planes[(uint64_t)ly * J.lw + x];
    int32_t cb = (int32_t)J.planes[J.cb_off + (uint64_t)by * J.cbw + bx] - 128;
    int32_t cr = (int32_t)J.planes[J.cr_off + (uint64_t)ry * J.crw + rx] - 128;
    int32_t r, g, b;
    if (J.limited) {
        int32_t yl = Y - 16 < 0 ? 0 : Y - 16;
        r = (298 * yl + 409 * cr + 128) >> 8;
        g = (298 * yl - 100 * cb - 208 * cr + 128) >> 8;
        b = (298 * yl + 516 * cb + 128) >> 8;
    } else {
        r = Y + ((359 * cr + 128) >> 8);
        g = Y - ((88 * cb + 183 * cr + 128) >> 8);
        b = Y + ((454 * cb + 128) >> 8);
    }
    o[0] = clamp255(r);
    o[1] = clamp255(g);
    o[2] = clamp255(b);
}

}  // namespace

void launch_rgb(const RgbLaunch &L, cudaStream_t s) {
    if (L.n_pixels == 0) return;
    uint64_t grid = (L.n_pixels + 255) / 256;
    rgb_kernel<<<(unsigned)grid, 256, 0, s>>>(L);
}

}  // namespace mmr
