// The reference's 8x8 inverse DCT reproduced exactly (crates/codecs/mjpeg/src/transform.rs:86-109).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "exact_fixed.h"
#include "kernels.h"
#include "rounding.h"
#include "tables.h"

namespace mmr {

// transform.rs:86-109 computes, in binary64 and in this order,
//   t[v][x] = sum_u M[x][u] * c[v][u]            (from 0.0, u = 0..7)
//   s[y][x] = sum_v M[y][v] * t[v][x]            (from 0.0, v = 0..7)
//   sample  = clamp(round_half_away(s + 128.0), 0, 255)
// GB300 issues binary64 at a small fraction of its fp32 rate, so every sample
// is first computed in fp32 and kept only when it provably rounds like the
// binary64 value:
//   S  = sum_v sum_u M[y][v] M[x][u] c[v][u]   (exact real value, double M)
//   B  = sum_v sum_u |M[y][v]| |M[x][u]| |c[v][u]|  <=  Mmax^2 * C1,
//        C1 = sum |c|, Mmax = max |M| = 0.49039264 (Mmax^2 < 0.2405)
//   fp32 path (idct_block; M and c rounded to fp32, u = 2^-24): each pass output
//        is fl(E +- O) with E, O chains of four FMAs, so it carries at most 5
//        roundings over its sum of |terms| (Higham ch. 3: gamma_5), plus u each
//        for rounding M and c to fp32:
//          pass 1   |t32 - t| <= 7u A,   A = sum_u |M[x][u]| |c[v][u]|
//          pass 2   |s32 - S| <= 5u B + u B + 7u B = 13u B   (+ O(u^2) B)
//   binary64 reference: |s64 - S| <= 16 * 2^-53 * B, and its +128.0 rounds
//        by at most 2^-53 |s + 128|.
// With delta = 2^-22 * C1 + 2^-40 |s32| + 2^-30 (2^-22 * C1 = 4u C1 >=
// 13u * 0.2405 C1 = 3.13u C1, margin 1.28 over the bound; |s32| <= C1 / 4 turns
// the middle term into 2^-42 C1), if no half-integer lies within delta of s32
// (+128 shifts by an integer) both values round to the same integer, and so
// clamp to the same sample.
// Every other sample is recomputed in the exact reference order. Zero
// coefficients are skipped in the exact path: a zero term adds +-0.0, which
// leaves any sum that is not -0.0 unchanged, and these sums are never -0.0.

namespace {

__constant__ double c_idct[64] = MMR_IDCT_MATRIX_INIT;
__constant__ float c_idct32[64] = MMR_IDCT_MATRIX_INIT;

// Pass 1 of the reference order for one row: t[v][x] = sum_u M[x][u] c[v][u].
__device__ __forceinline__ double exact_row(const int32_t *crow, int x) {
    double acc = 0.0;
#pragma unroll
    for (int u = 0; u < 8; u++) {
        const int32_t cv = crow[u];
        if (cv) acc = __dadd_rn(acc, __dmul_rn(c_idct[x * 8 + u], (double)cv));
    }
    return acc;
}

// Pass 2, +128, round half away from zero, clamp.
__device__ __forceinline__ uint8_t exact_finish(const double *t, int y) {
    double acc = 0.0;
#pragma unroll
    for (int v = 0; v < 8; v++)
        if (t[v] != 0.0) acc = __dadd_rn(acc, __dmul_rn(c_idct[y * 8 + v], t[v]));
    const double px = round(__dadd_rn(acc, 128.0));
    return (uint8_t)fmin(fmax(px, 0.0), 255.0);
}

__device__ __forceinline__ uint8_t exact_sample(const int32_t *c, int stride, int y, int x) {
    double t[8];
#pragma unroll
    for (int v = 0; v < 8; v++) t[v] = exact_row(c + v * stride, x);
    return exact_finish(t, y);
}

// Settles the samples in `mask` of one block whose exact dequantised coefficients
// are in c (shared memory; all 32 lanes of the warp call this together). First
// the warp forms each sample's exact fixed-point value (exact_fixed.h, offset
// +128); the samples still too close to a half-integer take the reference
// order: once for the whole block when it has no nonzero AC coefficient (every
// M[x][0] is the same literal, so all 64 reference samples are equal: DC-only
// blocks whose value is a half-integer leave all 64 undecided), else one sample
// per lane in parallel. put(y, x, sample) may run on any lane.
template <class Put>
__device__ __forceinline__ void settle_samples(const long long *fixw, const int32_t *c, unsigned long long mask,
                                               Put put) {
    const int lane = threadIdx.x & 31;
    long long c1 = llabs((long long)c[lane]) + llabs((long long)c[lane + 32]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c1 += __shfl_xor_sync(0xffffffffu, c1, o);
    const bool flat = __ballot_sync(0xffffffffu, (lane != 0 && c[lane] != 0) || c[lane + 32] != 0) == 0;
    unsigned long long left = 0;  // samples for the reference order
    for (unsigned long long m = mask; m; m &= m - 1) {
        const int b = __ffsll((long long)m) - 1, y = b >> 3, x = b & 7;
        int smp = -1;
        if (c1 < kFixMaxC1) smp = fixed_round(fixed_sum(fixw + (y * 8 + x) * 64, c), (int32_t)c1, 128);
        if (smp >= 0) {
            if (lane == 0) put(y, x, (uint8_t)smp);
        } else {
            left |= 1ull << b;
        }
    }
    if (!left) return;
    if (flat) {
        uint8_t v = 0;
        if (lane == 0) v = exact_sample(c, 8, 0, 0);
        v = (uint8_t)__shfl_sync(0xffffffffu, (uint32_t)v, 0);
        for (unsigned long long m = left; m; m &= m - 1) {
            const int b = __ffsll((long long)m) - 1;
            if (((b ^ lane) & 31) == 0) put(b >> 3, b & 7, v);  // lanes b and b - 32 share the stores
        }
        return;
    }
    while (left) {  // lane i takes the i-th remaining sample
        unsigned long long m = left;
        for (int i = 0; i < lane && m; i++) m &= m - 1;
        if (m) {
            const int b = __ffsll((long long)m) - 1;
            put(b >> 3, b & 7, exact_sample(c, 8, b >> 3, b & 7));
        }
        for (int i = 0; i < 32 && left; i++) left &= left - 1;
    }
}

// The 64 levels of block g: in the speculative decode's scratch arena when the
// block map points there, else in the coefficient arena (any map value past the
// arena, the reset value included, means in place).
__device__ __forceinline__ const int16_t *block_levels(const JpegLaunch &L, uint64_t g) {
    if (L.blk_map) {
        const uint32_t v = L.blk_map[g];
        if (v < L.scratch_blocks) return L.scratch + (uint64_t)v * 64;
    }
    return L.coef + g * 64;
}

// Dequantises block g (its levels at `levels`) into fp32 rows q and q+4 of `blk` (the product of an
// int16 level and an 8-bit quantiser is exact in fp32; the DC is the decoder's
// dequantised int32, rounded to fp32 like every c in the bound). Returns the
// sum of |c| over the two rows.
__device__ __forceinline__ float stage_rows(const int16_t *levels, const int32_t *dc, uint64_t g, uint32_t q,
                                            const float *Qf, float *blk) {
    const int4 *src = reinterpret_cast<const int4 *>(levels);
    float l1 = 0.0f;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const int row = q + 4 * h;
        const int4 v = src[row];
        const int16_t *lv = reinterpret_cast<const int16_t *>(&v);
        const float4 qa = reinterpret_cast<const float4 *>(Qf + row * 8)[0];
        const float4 qb = reinterpret_cast<const float4 *>(Qf + row * 8)[1];
        const float qv[8] = {qa.x, qa.y, qa.z, qa.w, qb.x, qb.y, qb.z, qb.w};
        float f[8];
#pragma unroll
        for (int j = 0; j < 8; j++) f[j] = (float)lv[j] * qv[j];
        if (row == 0) f[0] = (float)dc[g];
#pragma unroll
        for (int j = 0; j < 8; j++) l1 += fabsf(f[j]);
        reinterpret_cast<float4 *>(blk + row * 8)[0] = make_float4(f[0], f[1], f[2], f[3]);
        reinterpret_cast<float4 *>(blk + row * 8)[1] = make_float4(f[4], f[5], f[6], f[7]);
    }
    return l1;
}

// Sample of an fp32 transform value. Rounding it provably equals rounding the
// binary64 value when no half-integer lies within delta of acc, i.e. when acc
// is closer than 0.5 - delta to its nearest integer (with delta >= 0.5 nothing
// is certain); the exact pass settles the rest, ties included, so the rounding
// mode's ties-to-even never decides a sample. Clamping after an agreed rounding
// agrees.
//
// round_nearest (rounding.h) avoids conversion instructions and is exact for
// |acc| < 2^22. Larger values need no check of their own: |s| <= C1/4 and
// |acc - s| <= delta give C1 > 2^24 for |acc| >= 2^22, so near < 0 and the
// rounding is unsure already. A value that far beyond the clamp limits
// (s + 128 > 255.5 or < -0.5 whatever the rounding; 129 and -130 leave room for
// the fp32 rounding of the bounds) is decided by the clamp. Returns the
// unclamped integer sample (+128), or one far outside 0..255 for a clamped one.
__device__ __forceinline__ int32_t round_sample(float acc, float near, bool &unsure) {
    float r;
    const int32_t v = round_nearest(acc, r) + 128;
    unsure = !(fabsf(acc - r) < near);
    if (unsure) {
        const float delta = 0.5f - near;
        if (acc > 129.0f + delta) {
            unsure = false;
            return 1 << 20;
        }
        if (acc < -130.0f - delta) {
            unsure = false;
            return -(1 << 20);
        }
    }
    return v;
}

// Two samples saturated to 0..255 in one instruction: a in byte 0, b in byte 1.
__device__ __forceinline__ uint32_t sat_pair_u8(int32_t a, int32_t b) {
    uint32_t d;
    asm("cvt.pack.sat.u8.s32.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(b), "r"(a), "r"(0));
    return d;
}

// Transform of one staged block by its four threads; thread q produces output
// columns q and 7 - q into out[row * stride + col]. Both passes use the even/odd
// split of the basis: M[7-x][u] = (-1)^u M[x][u] holds for the fp32 roundings of
// the reference's literals (the literals themselves differ from exact symmetry by
// < 2e-15, far inside the fp32 rounding), so
//   s[x] = E + O, s[7-x] = E - O,  E = sum_{u even} M[x][u] c[u], O = sum_{u odd}.
// Per output this is 4 FMAs per half and one add: each pass's error is <= 5u of
// the sum of |terms|, plus u for each rounded M and c, <= 13u B after both
// passes (the bound above). |s| <= Mmax^2 C1 < C1/4, so the relative term
// 2^-40 |s| of the bound is folded into 2^-42 C1.
// Returns the samples left to the exact pass as bits (row * 8 + column).
__device__ __forceinline__ unsigned long long idct_block(const float *blk, uint32_t q, float c1, uint8_t *out,
                                                         int stride) {
    float mq[8];
#pragma unroll
    for (int u = 0; u < 8; u++) mq[u] = c_idct32[q * 8 + u];
    float ta[8], tb[8];
#pragma unroll
    for (int v = 0; v < 8; v++) {
        const float4 c0 = reinterpret_cast<const float4 *>(blk + v * 8)[0];
        const float4 c1v = reinterpret_cast<const float4 *>(blk + v * 8)[1];
        float e = c0.x * mq[0];
        e = fmaf(mq[2], c0.z, e);
        e = fmaf(mq[4], c1v.x, e);
        e = fmaf(mq[6], c1v.z, e);
        float o = c0.y * mq[1];
        o = fmaf(mq[3], c0.w, o);
        o = fmaf(mq[5], c1v.y, o);
        o = fmaf(mq[7], c1v.w, o);
        ta[v] = e + o;
        tb[v] = e - o;
    }
    // delta = 2^-22 C1 >= 13u Mmax^2 C1 (margin 1.28), see the bound above
    const float near = 0.5f - (c1 * (0x1p-22f + 0x1p-42f) + 0x1p-30f);
    uint32_t bits = 0;  // bit 2*row (column q), 2*row+1 (column 7-q)
#pragma unroll
    for (int y = 0; y < 4; y++) {
#pragma unroll
        for (int side = 0; side < 2; side++) {
            const float *t = side ? tb : ta;
            float e = t[0] * c_idct32[y * 8 + 0];
            e = fmaf(c_idct32[y * 8 + 2], t[2], e);
            e = fmaf(c_idct32[y * 8 + 4], t[4], e);
            e = fmaf(c_idct32[y * 8 + 6], t[6], e);
            float o = t[1] * c_idct32[y * 8 + 1];
            o = fmaf(c_idct32[y * 8 + 3], t[3], o);
            o = fmaf(c_idct32[y * 8 + 5], t[5], o);
            o = fmaf(c_idct32[y * 8 + 7], t[7], o);
            const uint32_t col = side ? 7 - q : q;
            bool u0, u1;
            const uint32_t pair = sat_pair_u8(round_sample(e + o, near, u0), round_sample(e - o, near, u1));
            out[y * stride + col] = (uint8_t)pair;
            out[(7 - y) * stride + col] = (uint8_t)(pair >> 8);
            bits |= (u0 ? 1u : 0u) << (2 * y + side);
            bits |= (u1 ? 1u : 0u) << (2 * (7 - y) + side);
        }
    }
    unsigned long long mask = 0;
    if (bits) {
#pragma unroll
        for (int row = 0; row < 8; row++) {
            if (bits & (1u << (2 * row))) mask |= 1ull << (row * 8 + q);
            if (bits & (2u << (2 * row))) mask |= 1ull << (row * 8 + 7 - q);
        }
    }
    return mask;
}

}  // namespace

}  // namespace mmr
