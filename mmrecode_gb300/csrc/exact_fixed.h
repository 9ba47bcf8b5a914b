// Second decision stage of the exact transforms: a sample the fp32 evaluation
// cannot decide is evaluated exactly in 2^-40 fixed point by a whole warp, and
// only the samples that are still within the bound of a half-integer go to the
// binary64 reference order. GB300's binary64 pipe takes tens of cycles per warp
// instruction, so the reference order (a dependent chain of up to 64 terms, run
// by one lane) is kept for genuine near-ties only.
//
// A transform sample is linear in the block's coefficients: value = sum_i w_i
// c_i with w_i the exact real product of the reference's binary64 constants
//   MJPEG IDCT (transform.rs:86-109)     w = M[y][v] * M[x][u]            (+128 after)
//   DV 8-8     (dv decoder.rs:520-548)   w = (cu cv) cos_u(x) cos_v(y) / 4, cu cv for
//                                            u = v = 0 being fl(FRAC * FRAC) as there
//   DV 2-4-8   (dv decoder.rs:555-602)   w = +-(cv cos8_v(y)) (cu cos16_u(x)) / 4 on the
//                                            two coefficients of each butterfly pair
// The tables hold W_i = round(w_i * 2^40) with w_i computed in binary64 on the
// host (at most three roundings of 2^-53 relative, |w_i| <= 1/4), so
// |W_i / 2^40 - w_i| <= 2^-41 + 2^-53. The warp computes T = sum W_i c_i exactly
// (int64: |c_i| < 2^21 and C1 = sum |c_i| < 2^21 keep every partial sum below
// 2^61), hence |T / 2^40 - value| <= C1 (2^-41 + 2^-53). The reference's own
// binary64 evaluation differs from the exact value by at most 67 * 2^-53 times
// the sum of its |terms| (<= C1 / 4: three product roundings and at most 63
// additions per term for DV 8-8; fewer for the others; plus 2^-53 (|s| + 128)
// for the MJPEG +128.0). Both together stay below C1 * 2^-40 + 2^-40: if no
// half-integer lies within (C1 + 2) / 2^40 of T / 2^40, the reference rounds to
// the integer nearest T / 2^40 (and clamps alike).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>

#include "common.h"
#include "tables.h"

namespace mmr {

constexpr int kFixShift = 40;
constexpr int kFixEntries = 64 * 64;  // per transform: [sample y * 8 + x][coefficient v * 8 + u]
constexpr int32_t kFixMaxC1 = 1 << 21;

// ----------------------------------------------------------- host tables ---

inline long long fix_round(double w) { return llrint(w * 0x1p40); }

// MJPEG IDCT: w[(y*8+x)*64 + v*8+u] = M[y][v] * M[x][u].
inline void build_jpeg_fixed(long long *w) {
    static const double M[64] = MMR_IDCT_MATRIX_INIT;
    for (int y = 0; y < 8; y++)
        for (int x = 0; x < 8; x++)
            for (int v = 0; v < 8; v++)
                for (int u = 0; u < 8; u++) w[(y * 8 + x) * 64 + v * 8 + u] = fix_round(M[y * 8 + v] * M[x * 8 + u]);
}

// DV 8-8 (w88) and 2-4-8 (w248) from the libm cos table the transforms use.
inline void build_dv_fixed(long long *w88, long long *w248) {
    static const double cs[128] = {
#include "cos_table.inc"
    };
    const double frac = 0.7071067811865476;  // FRAC_1_SQRT_2
    const double kk00 = frac * frac;
    for (int y = 0; y < 8; y++)
        for (int x = 0; x < 8; x++) {
            long long *r88 = w88 + (y * 8 + x) * 64, *r248 = w248 + (y * 8 + x) * 64;
            for (int v = 0; v < 8; v++)
                for (int u = 0; u < 8; u++) {
                    const double k = (u == 0 && v == 0) ? kk00 : (u == 0 || v == 0) ? frac : 1.0;
                    r88[v * 8 + u] = fix_round(k * cs[(2 * x + 1) * u] * cs[(2 * y + 1) * v] / 4.0);
                }
            const int field = y & 1, yy = y >> 1;
            for (int i = 0; i < 64; i++) r248[i] = 0;
            for (int v = 0; v < 4; v++)
                for (int u = 0; u < 8; u++) {
                    const double wv = (v == 0 ? frac : 1.0) * cs[2 * (2 * yy + 1) * v];
                    const double wu = (u == 0 ? frac : 1.0) * cs[(2 * x + 1) * u];
                    const double w = wv * wu / 4.0;
                    // row 2v + field of the butterfly: c[v*16+u] + c[v*16+8+u] (even), - (odd)
                    r248[v * 16 + u] = fix_round(w);
                    r248[v * 16 + 8 + u] = fix_round(field ? -w : w);
                }
        }
}

// ------------------------------------------------------------ evaluation ---

#if defined(__CUDACC__)
// T = sum_i W_i c_i over the 64 coefficients of a block, every lane of the warp
// taking part (all 32 call it with the same wrow and c); the result in every lane.
__device__ __forceinline__ long long fixed_sum(const long long *__restrict__ wrow, const int32_t *c) {
    const int lane = threadIdx.x & 31;
    long long p = __ldg(wrow + lane) * (long long)c[lane] + __ldg(wrow + lane + 32) * (long long)c[lane + 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) p += __shfl_xor_sync(0xffffffffu, p, o);
    return p;
}
#endif

// The clamped sample of T / 2^40 + offset when no half-integer lies within
// (c1 + 2) / 2^40 of it, else -1 (decide in the reference order). Host and
// device: the CPU tests check it against the reference's rounding.
MMR_HD int fixed_round(long long t, int32_t c1, int offset) {
    const long long one = 1ll << kFixShift, half = one >> 1;
    const long long d = (t & (one - 1)) - half;  // T mod 2^40, centred on the half-integer
    if ((d < 0 ? -d : d) <= (long long)c1 + 2) return -1;
    const long long n = ((t + half) >> kFixShift) + offset;  // nearest integer
    return n < 0 ? 0 : n > 255 ? 255 : (int)n;
}

}  // namespace mmr
