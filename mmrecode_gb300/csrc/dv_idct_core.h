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
// Used by dv_idct_kernel (eight threads per block, the row-parallel form at the
// end of this file) and, with the same functions, by the block-level transform
// tests.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "exact_fixed.h"
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

// The fp32 value's sample when it is certain: no half-integer within delta of
// the value (c1 = sum |c| of the block), or the value so far beyond 255.5 or
// below -0.5 that the reference clamps it whatever its rounding (the comparison
// constants leave room for the fp32 rounding of 256 + delta). -1: undecided.
__device__ __forceinline__ int dv_decide32(float value, float c1) {
    const float delta = c1 * 0x1p-21f + 0x1p-30f;
    float r;
    const int32_t v = round_nearest(value, r);
    if (fabsf(value - r) < 0.5f - delta && fabsf(value) < 0x1p22f) return min(max(v, 0), 255);
    if (value > 256.0f + delta) return 255;
    if (value < -1.0f - delta) return 0;
    return -1;
}

// The reference order for sample (y, x), rounded and clamped.
__device__ __forceinline__ uint8_t dv_exact_sample(const int32_t *c, bool mode248, int y, int x) {
    const double e = mode248 ? exact_248(c, y, x) : exact_88(c, y, x);
    return (uint8_t)fmin(fmax(round(e), 0.0), 255.0);
}

// The sample of every position of a block whose only nonzero coefficient is the
// DC: all 64 are equal (cos16[0] = cos8[0] = 1.0, and only the u = v = 0 terms
// are nonzero), so the reference-order value of position (0, 0) is computed once
// per block. These blocks are common in smooth content, and with an odd DC level
// their exact value is a half-integer: every sample would go to the binary64
// pass one by one.
__device__ __forceinline__ uint8_t dv_flat_sample(const int32_t *c, bool mode248) {
    return dv_exact_sample(c, mode248, 0, 0);
}

// ---------------------------------------------------------------------------
// Row-parallel form: eight threads per block, thread r producing output row r.
// The factors are fp32 products of the fp32 roundings, W[u][x] = (u ? 1 : FRAC)
// * cos16f[(2x+1)u] (transposed: a thread reads the eight x of one u as two
// 16-byte loads) and V4[yy][v] = (v ? 1 : FRAC) * cos16f[2(2yy+1)v]. Pass 1 is an
// FMA chain over u per output, pass 2 one over v, the 2-4-8 butterfly and the
// halvings exact: the evaluation the bound above describes.

// Fills the tables (64 + 16 floats) cooperatively; callers synchronise before use.
__device__ __forceinline__ void dv_fill_tables(float *wt, float *v4) {
    for (int i = threadIdx.x; i < 80; i += blockDim.x) {
        if (i < 64) {
            const int u = i >> 3, x = i & 7;
            wt[i] = (u == 0 ? (float)kFrac : 1.0f) * c_cos16f[(2 * x + 1) * u];
        } else {
            const int yy = (i - 64) >> 2, v = (i - 64) & 3;
            v4[i - 64] = (v == 0 ? (float)kFrac : 1.0f) * c_cos16f[2 * (2 * yy + 1) * v];
        }
    }
}

// Pass 1 for row r: h[r][0..7] into hrow (16-byte aligned). c: the block's 64
// coefficients (natural order).
__device__ __forceinline__ void dv_row_pass8(const int32_t *c, const float *wt, bool mode248, int r, float *hrow) {
    float b[8];
    if (mode248) {
        const int pair = r >> 1;
#pragma unroll
        for (int u = 0; u < 8; u++) {
            const float first = (float)c[pair * 16 + u], second = (float)c[pair * 16 + 8 + u];
            b[u] = (r & 1) ? first - second : first + second;  // exact: |c| < 2^23
        }
    } else {
#pragma unroll
        for (int u = 0; u < 8; u++) b[u] = (float)c[r * 8 + u];
    }
    float h[8];
#pragma unroll
    for (int x = 0; x < 8; x++) h[x] = 0.0f;
#pragma unroll
    for (int u = 0; u < 8; u++) {
        const float4 w0 = reinterpret_cast<const float4 *>(wt + u * 8)[0];
        const float4 w1 = reinterpret_cast<const float4 *>(wt + u * 8)[1];
        const float w[8] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w};
#pragma unroll
        for (int x = 0; x < 8; x++) h[x] = fmaf(w[x], b[u], h[x]);
    }
    if (mode248) {
#pragma unroll
        for (int x = 0; x < 8; x++) h[x] *= 0.5f;
    }
    reinterpret_cast<float4 *>(hrow)[0] = make_float4(h[0], h[1], h[2], h[3]);
    reinterpret_cast<float4 *>(hrow)[1] = make_float4(h[4], h[5], h[6], h[7]);
}

// Pass 2 for output row y: value[0..7] from the block's 64 pass-1 outputs h
// (row-major, 16-byte aligned rows).
__device__ __forceinline__ void dv_column_pass8(const float *h, const float *wt, const float *v4, bool mode248, int y,
                                                float *value) {
    float s[8];
#pragma unroll
    for (int x = 0; x < 8; x++) s[x] = 0.0f;
    if (mode248) {
        const int field = y & 1, yy = y >> 1;
#pragma unroll
        for (int v = 0; v < 4; v++) {
            const float wv = v4[yy * 4 + v];
            const float4 h0 = reinterpret_cast<const float4 *>(h + (v * 2 + field) * 8)[0];
            const float4 h1 = reinterpret_cast<const float4 *>(h + (v * 2 + field) * 8)[1];
            const float hv[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
#pragma unroll
            for (int x = 0; x < 8; x++) s[x] = fmaf(wv, hv[x], s[x]);
        }
#pragma unroll
        for (int x = 0; x < 8; x++) value[x] = s[x] * 0.5f;
    } else {
#pragma unroll
        for (int v = 0; v < 8; v++) {
            const float wv = wt[v * 8 + y];  // V[y][v] = W[v][y]
            const float4 h0 = reinterpret_cast<const float4 *>(h + v * 8)[0];
            const float4 h1 = reinterpret_cast<const float4 *>(h + v * 8)[1];
            const float hv[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
#pragma unroll
            for (int x = 0; x < 8; x++) s[x] = fmaf(wv, hv[x], s[x]);
        }
#pragma unroll
        for (int x = 0; x < 8; x++) value[x] = s[x] * 0.25f;
    }
}

// The samples of row y that the fp32 evaluation decides, packed little-endian
// (x = 0 in the low byte) into *row; returns the undecided ones as bits (x).
// For a flat block (no nonzero AC coefficient) lane `flat_src` of the warp
// computes the one reference-order value and broadcasts it (all eight lanes of
// the block's group call this together).
__device__ __forceinline__ uint32_t dv_row_fp32(const int32_t *c, const float *h, const float *wt, const float *v4,
                                                bool mode248, int y, float c1, bool flat, int flat_src,
                                                unsigned group_mask, unsigned long long *row) {
    if (flat) {
        uint32_t v = 0;
        if ((int)(threadIdx.x & 31) == flat_src) v = dv_flat_sample(c, mode248);
        v = __shfl_sync(group_mask, v, flat_src);
        *row = 0x0101010101010101ull * v;
        return 0;
    }
    float value[8];
    dv_column_pass8(h, wt, v4, mode248, y, value);
    unsigned long long out = 0;
    uint32_t und = 0;
#pragma unroll
    for (int x = 0; x < 8; x++) {
        const int d = dv_decide32(value[x], c1);
        if (d < 0) und |= 1u << x;
        else out |= (unsigned long long)d << (8 * x);
    }
    *row = out;
    return und;
}

// Settles the undecided samples of every lane of the warp (all 32 lanes call
// this; und = 0 for lanes with none): one sample at a time the whole warp forms
// its exact fixed-point value (exact_fixed.h), and the owner lane takes it, or
// the reference order when that value is too close to a half-integer.
// c: the lane's block coefficients (shared), c1i = sum |c| exactly, fix: the
// 8-8 table followed by the 2-4-8 table.
__device__ __forceinline__ void dv_resolve_row(uint32_t und, unsigned long long &row, const int32_t *c,
                                               bool mode248, int y, int32_t c1i, const long long *fix) {
    const int lane = threadIdx.x & 31;
    uint32_t m;
    while ((m = __ballot_sync(0xffffffffu, und != 0)) != 0) {
        const int src = __ffs(m) - 1;
        const uint32_t sund = __shfl_sync(0xffffffffu, und, src);
        const int x = __ffs(sund) - 1;
        const int sy = __shfl_sync(0xffffffffu, y, src);
        const int smode = __shfl_sync(0xffffffffu, mode248 ? 1 : 0, src);
        const int32_t sc1 = __shfl_sync(0xffffffffu, c1i, src);
        const int32_t *sc = reinterpret_cast<const int32_t *>(
            __shfl_sync(0xffffffffu, (unsigned long long)reinterpret_cast<uintptr_t>(c), src));
        int smp = -1;
        if (sc1 < kFixMaxC1) smp = fixed_round(fixed_sum(fix + smode * kFixEntries + (sy * 8 + x) * 64, sc), sc1, 0);
        if (lane == src) {
            if (smp < 0) smp = dv_exact_sample(c, mode248, y, x);
            row |= (unsigned long long)smp << (8 * x);
            und &= und - 1;
        }
    }
}

}  // namespace
}  // namespace mmr
