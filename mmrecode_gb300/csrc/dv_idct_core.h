// The reference's DV25 inverse DCTs reproduced exactly
// (crates/codecs/dv/src/decoder.rs:520-548 inverse_88, 555-602 inverse_248).
//
// Both transforms are first evaluated in fp32 as separable sums (8 + 8 terms for
// 8-8; butterfly, 8 + 4 terms for 2-4-8), each factor cu * cos the fp32 product
// of the fp32 roundings (3u, u = 2^-24) and each pass an FMA chain. Against the
// exact real value of the reference's terms (its doubles: FRAC_1_SQRT_2, the cos
// table, the integer c) the fp32 sum is off by at most (3u + 8u) + (3u + 8u) = 22u B
// for 8-8 and 11u + 3u + 4u = 18u B for 2-4-8; the binary64 sequence by < 70 *
// 2^-53 B. B = sum |terms| <= C1 = sum |c| for 8-8 (|cos| <= 1, cu cv <= 1) and
// <= C1 / 2 per 2-4-8 field (a butterfly output is at most |c1| + |c2|); after the
// final / 4.0 or / 2.0, |value32 - value64| <= 5.5u C1 < delta = 2^-21 C1 + 2^-30
// (= 8u C1 + 2^-30, margin 1.45). If no half-integer lies within delta of value32
// both round (half away from zero) and clamp alike; the rest are recomputed in
// the reference order.
//
// Used by dv_idct_kernel (one thread per sample) and, with the same functions,
// by the block-level transform tests.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "rounding.h"

namespace mmr {
namespace {

__constant__ double c_cos16[128] = {
#include "cos_table.inc"
};

__constant__ float c_cos16f[128] = {
#include "cos_table.inc"
};

constexpr double kFrac = 0.7071067811865476;  // FRAC_1_SQRT_2

// The reference's binary64 8-8 direct sum for sample (y, x) (decoder.rs:520-548):
// terms ((((cu*cv)*c)*cos_u)*cos_v) accumulated in (v, u) order, then / 4.0. Zero
// coefficients are skipped: their term is +-0.0, which leaves any sum that is not
// -0.0 unchanged, and these sums are never -0.0.
__device__ __noinline__ double exact_88(const int32_t *c, int y, int x) {
    const double kk00 = __dmul_rn(kFrac, kFrac);
    double sum = 0.0;
    for (int v = 0; v < 8; v++) {
        for (int u = 0; u < 8; u++) {
            const int32_t cv = c[v * 8 + u];
            if (cv == 0) continue;
            const double k = (u == 0 && v == 0) ? kk00 : (u == 0 || v == 0) ? kFrac : 1.0;
            double t = __dmul_rn(k, (double)cv);
            t = __dmul_rn(t, c_cos16[(2 * x + 1) * u]);
            t = __dmul_rn(t, c_cos16[(2 * y + 1) * v]);
            sum = __dadd_rn(sum, t);
        }
    }
    return sum / 4.0;
}

// The reference's binary64 2-4-8 transform for sample (y, x) (decoder.rs:555-602):
// butterfly of row pairs, horizontal pass per row (/ 2.0), four-term field pass (/ 2.0).
__device__ __noinline__ double exact_248(const int32_t *c, int y, int x) {
    const int field = y & 1, yy = y >> 1;
    double sum = 0.0;
    for (int v = 0; v < 4; v++) {
        const int row = v * 2 + field, pair = row >> 1;
        double hs = 0.0;
        for (int u = 0; u < 8; u++) {
            const double first = (double)c[pair * 16 + u], second = (double)c[pair * 16 + 8 + u];
            const double b = (row & 1) ? __dsub_rn(first, second) : __dadd_rn(first, second);
            if (b != 0.0) hs = __dadd_rn(hs, __dmul_rn(__dmul_rn(u == 0 ? kFrac : 1.0, b), c_cos16[(2 * x + 1) * u]));
        }
        const double h = hs / 2.0;
        if (h != 0.0) sum = __dadd_rn(sum, __dmul_rn(__dmul_rn(v == 0 ? kFrac : 1.0, h), c_cos16[2 * (2 * yy + 1) * v]));
    }
    return sum / 2.0;
}

// Horizontal pass for output (row, x) of a block of int32 coefficients c
// (natural order): the 8-8 row sum, or for 2-4-8 the row sum over the
// butterfly of the row pair, halved.
__device__ __forceinline__ float dv_row_pass(const int32_t *c, bool mode248, int row, int x) {
    float h = 0.0f;
    if (mode248) {
        const int pair = row >> 1;
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const float first = (float)c[pair * 16 + u], second = (float)c[pair * 16 + 8 + u];
            const float b = (row & 1) ? first - second : first + second;  // exact: |c| < 2^23
            h = fmaf((u == 0 ? (float)kFrac : 1.0f) * c_cos16f[(2 * x + 1) * u], b, h);
        }
        h *= 0.5f;
    } else {
#pragma unroll
        for (int u = 0; u < 8; u++)
            h = fmaf((u == 0 ? (float)kFrac : 1.0f) * c_cos16f[(2 * x + 1) * u], (float)c[row * 8 + u], h);
    }
    return h;
}

// Vertical pass for sample (y, x) from the 64 row-pass outputs h: the 8-8 column
// sum / 4, or the 2-4-8 four-term field sum / 2.
__device__ __forceinline__ float dv_column_pass(const float *h, bool mode248, int y, int x) {
    if (mode248) {
        const int field = y & 1, yy = y >> 1;
        float s = 0.0f;
#pragma unroll
        for (int v = 0; v < 4; v++)
            s = fmaf((v == 0 ? (float)kFrac : 1.0f) * c_cos16f[2 * (2 * yy + 1) * v], h[(v * 2 + field) * 8 + x], s);
        return s * 0.5f;
    }
    float s = 0.0f;
#pragma unroll
    for (int v = 0; v < 8; v++)
        s = fmaf((v == 0 ? (float)kFrac : 1.0f) * c_cos16f[(2 * y + 1) * v], h[v * 8 + x], s);
    return s * 0.25f;
}

// The sample: the fp32 value's rounding when no half-integer lies within delta of
// it (c1 = sum |c| of the block), else the reference's binary64 value rounded
// half away from zero; clamped to 0..255.
__device__ __forceinline__ uint8_t dv_sample(float value, float c1, const int32_t *c, bool mode248, int y, int x) {
    const float near = 0.5f - (c1 * 0x1p-21f + 0x1p-30f);
    float r;
    const int32_t v = round_nearest(value, r);
    if (fabsf(value - r) < near && fabsf(value) < 0x1p22f) return (uint8_t)min(max(v, 0), 255);
    const double e = mode248 ? exact_248(c, y, x) : exact_88(c, y, x);
    return (uint8_t)fmin(fmax(round(e), 0.0), 255.0);
}

}  // namespace
}  // namespace mmr
