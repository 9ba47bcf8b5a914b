// The reference's forward DCT and quantisation reproduced exactly
// (crates/codecs/mjpeg/src/transform.rs:111-134 forward_dct_quantize): an fp32
// evaluation with a per-coefficient error bound, and the binary64 reference
// order for quotients within that bound of a half-integer. Used by fdct_kernel
// (8 threads per block) and, with the same functions, by the block-level
// transform tests.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "tables.h"

namespace mmr {
namespace {

__constant__ float c_m32[64] = MMR_IDCT_MATRIX_INIT;   // IDCT_MATRIX[x][u] at x * 8 + u, rounded to fp32
__constant__ double c_m64[64] = MMR_IDCT_MATRIX_INIT;  // the reference's binary64 values

// The quantised coefficient (v, u) of a block exactly as forward_dct_quantize
// (transform.rs:111-134) computes it: binary64, every product and sum rounded
// separately, rows accumulated over x, then the column over y, both from 0.0,
// the quotient rounded half away from zero.
__device__ __noinline__ int exact_coefficient(const uint8_t *s, int u, int v, int q) {
    double value = 0.0;
    for (int y = 0; y < 8; y++) {
        double t = 0.0;
        for (int x = 0; x < 8; x++) t = __dadd_rn(t, __dmul_rn(c_m64[x * 8 + u], (double)s[y * 8 + x] - 128.0));
        value = __dadd_rn(value, __dmul_rn(c_m64[y * 8 + v], t));
    }
    return (int)round(__ddiv_rn(value, (double)q));
}

// Error bound of the fp32 path, per coefficient. With S = sample - 128 and the
// coefficient's magnitude sum B = sum_y |M[y][v]| sum_x |M[x][u]| |S[y][x]|, each
// pass is an 8-term FMA chain (8 roundings of at most 2^-24 of a partial sum
// bounded by its magnitude sum) on fp32 matrix entries (2^-24 relative each),
// against the reference's binary64 chains (2^-53 per operation):
// |V32 - V64| <= (8 + 9 + 1) * 2^-24 * B + 2^-46 * B < 1.08e-6 * B. The fp32
// quotient is V32 times the rounded reciprocal of q (two roundings of 2^-24 each:
// within 1.2e-7 |q32| of V32 / q) and the binary64 one is within 2^-53 |V64 / q|, so
// |q32 - q64| < 1.08e-6 * B / q + 1.2e-7 * |q32| + 1e-12. The guard below takes
// 1.5e-6, 3.6e-7 and 1e-9 for these (B itself computed in fp32 to within 2^-20
// relative, B / q as B times the reciprocal): a fp32 quotient farther than that from
// the nearest half-integer rounds to the reference's integer; the rest are
// recomputed in binary64. (B <= 1025, so the guard never exceeds 2e-3.)
__device__ __forceinline__ float tie_guard(float b, float rq, float quot_abs) {
    return 1.5e-6f * b * rq + 3.6e-7f * quot_abs + 1e-9f;
}
// Row pass output (r, u): t = sum_x M[x][u] S[r][x] over the row's centred
// samples srow[x] = sample - 128, and its magnitude sum sum_x |M[x][u]| |S[r][x]|.
__device__ __forceinline__ void fdct_row_pass(const float *srow, int u, float &acc, float &mag) {
    float a = 0.0f, m = 0.0f;
#pragma unroll
    for (int x = 0; x < 8; x++) {
        a = fmaf(c_m32[x * 8 + u], srow[x], a);
        m = fmaf(fabsf(c_m32[x * 8 + u]), fabsf(srow[x]), m);
    }
    acc = a;
    mag = m;
}

// Quantised coefficient (v, u) from the row-pass outputs rows[y * stride + u]
// and their magnitude sums mags[..] (raw: the block's 64 samples, q the
// quantiser, rq its fp32 reciprocal). exact reports whether the binary64
// reference order decided it. Unclamped.
__device__ __forceinline__ int fdct_quantise(const float *rows, const float *mags, int stride, const uint8_t *raw,
                                            int u, int v, int q, float rq, bool &exact) {
    float acc = 0.0f, mag = 0.0f;
#pragma unroll
    for (int y = 0; y < 8; y++) {
        acc = fmaf(c_m32[y * 8 + v], rows[y * stride + u], acc);
        mag = fmaf(fabsf(c_m32[y * 8 + v]), mags[y * stride + u], mag);
    }
    const float quot = acc * rq;
    const float a = fabsf(quot);
    exact = fabsf(a - floorf(a) - 0.5f) < tie_guard(mag * (1.0f + 1.0f / 1048576.0f), rq, a);
    return exact ? exact_coefficient(raw, u, v, q) : (int)rintf(quot);
}

}  // namespace
}  // namespace mmr
