// Round-to-nearest of an fp32 value without conversion instructions (FRND,
// F2I issue on a slow shared pipe; this is two adds and an integer subtract).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace mmr {

// For |x| < 2^22, x + 1.5 * 2^23 lies in [2^23, 2^24), where the fp32 spacing is
// 1, so the round-to-nearest-even add leaves the nearest integer n of x in the
// low mantissa bits (bits = 0x4B400000 + n), and subtracting 1.5 * 2^23 again
// gives n exactly as a float in r. Callers check |x| < 2^22 before trusting it.
__device__ __forceinline__ int32_t round_nearest(float x, float &r) {
    const float t = __fadd_rn(x, 0x1.8p23f);
    r = __fsub_rn(t, 0x1.8p23f);
    return (int32_t)(__float_as_uint(t) - 0x4B400000u);
}

}  // namespace mmr
