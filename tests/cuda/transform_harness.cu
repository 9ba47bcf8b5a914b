// Block-level harness for the library's exact transforms (test infrastructure).
//
// Runs arbitrary coefficient or sample blocks through the same device functions
// the decode and encode kernels use -- idct_core.h (MJPEG inverse DCT: fp32
// even/odd transform, decision bound, binary64 reference order), dv_idct_core.h
// (DV 8-8 and 2-4-8) and fdct_core.h (forward DCT + quantisation) -- with the
// kernels' thread mapping (4 threads per MJPEG block, one per DV sample, 8 per
// FDCT block), so the tests can compare millions of random and adversarial
// blocks with the oracle's per-block functions. Built by the tests with nvcc;
// not part of the library.
#include <cuda_runtime.h>
#include <stdint.h>

#include "dv_idct_core.h"
#include "fdct_core.h"
#include "idct_core.h"

namespace mmr {
namespace {

constexpr int kJBlocks = 32;  // MJPEG blocks per CTA (4 threads each)
constexpr int kJStride = 68;

__global__ void __launch_bounds__(kJBlocks * 4) jpeg_idct_blocks(const int32_t *c, uint64_t n, const long long *fixw,
                                                                  uint8_t *out, unsigned long long *exact) {
    __shared__ __align__(16) float s_f[kJBlocks * kJStride];
    __shared__ __align__(16) uint8_t s_o[kJBlocks * 64];
    const int lb = threadIdx.x >> 2, q = threadIdx.x & 3;
    const uint64_t b = (uint64_t)blockIdx.x * kJBlocks + lb;
    const bool valid = b < n;
    float *blk = s_f + lb * kJStride;
    float l1 = 0.0f;
    if (valid) {
#pragma unroll
        for (int h = 0; h < 2; h++) {
            const int row = q + 4 * h;
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const float f = (float)c[b * 64 + row * 8 + j];
                l1 += fabsf(f);
                blk[row * 8 + j] = f;
            }
        }
    }
#pragma unroll
    for (int o = 1; o < 4; o <<= 1) l1 += __shfl_xor_sync(0xffffffffu, l1, o);
    __syncwarp();
    unsigned long long mask = valid ? idct_block(blk, q, l1, s_o + lb * 64, 8) : 0ull;
#pragma unroll
    for (int o = 1; o < 4; o <<= 1) mask |= __shfl_xor_sync(0xffffffffu, mask, o);
    __syncwarp();
    // a warp settles the undecided samples of its eight blocks one block at a time,
    // as the decode kernels do (settle_samples)
    __shared__ int32_t s_cx[kJBlocks / 8][64];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t n_exact = 0;
    for (int k = 0; k < 8; k++) {
        const unsigned long long bm = __shfl_sync(0xffffffffu, mask, k * 4);
        if (!bm) continue;
        const int blb = w * 8 + k;
        const uint64_t bb = (uint64_t)blockIdx.x * kJBlocks + blb;
        s_cx[w][lane] = (int32_t)c[bb * 64 + lane];
        s_cx[w][lane + 32] = (int32_t)c[bb * 64 + lane + 32];
        __syncwarp();
        settle_samples(fixw, s_cx[w], bm, [&](int y, int x, uint8_t v) { s_o[blb * 64 + y * 8 + x] = v; });
        __syncwarp();
        n_exact += __popcll(bm);
    }
    if (!valid) return;
    for (int row = 0; row < 8; row++)
        for (int side = 0; side < 2; side++) {
            const int col = side ? 7 - q : q;
            out[b * 64 + row * 8 + col] = s_o[lb * 64 + row * 8 + col];
        }
    if (lane == 0 && n_exact) atomicAdd(exact, (unsigned long long)n_exact);
}

// DV: the decode kernel's row-parallel form (dv_idct_kernel), eight threads per
// block, output in natural order.
__global__ void __launch_bounds__(256) dv_idct_blocks(const int32_t *coef, const uint8_t *modes, uint64_t n,
                                                      const long long *fix, uint8_t *out) {
    __shared__ __align__(16) int32_t s_c[32][64];
    __shared__ __align__(16) float s_h[32][64];
    __shared__ __align__(16) float s_wt[64];
    __shared__ __align__(16) float s_v4[16];
    dv_fill_tables(s_wt, s_v4);
    __syncthreads();
    const int lane = threadIdx.x & 31, lb = threadIdx.x >> 3, r = threadIdx.x & 7;
    const unsigned group_mask = 0xffu << (lane & 24);
    const uint64_t b = (uint64_t)blockIdx.x * 32 + lb;
    const bool valid = b < n;
    const bool mode = valid && modes[b] != 0;
    int32_t *c = s_c[lb];
    float a = 0.0f;
    int32_t ai = 0;
    bool ac = false;
#pragma unroll
    for (int u = 0; u < 8; u++) {
        const int32_t v = valid ? coef[b * 64 + r * 8 + u] : 0;
        c[r * 8 + u] = v;
        a += fabsf((float)v);
        ai += abs(v);
        ac |= (r | u) != 0 && v != 0;
    }
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        ai += __shfl_xor_sync(0xffffffffu, ai, o);
    }
    const bool flat = (__ballot_sync(0xffffffffu, ac) & group_mask) == 0;
    __syncwarp();
    if (valid && !flat) dv_row_pass8(c, s_wt, mode, r, s_h[lb] + r * 8);
    __syncwarp();
    unsigned long long row = 0;
    uint32_t und = 0;
    if (valid) und = dv_row_fp32(c, s_h[lb], s_wt, s_v4, mode, r, a, flat, lane & 24, group_mask, &row);
    dv_resolve_row(und, row, c, mode, r, ai, fix);
    if (!valid) return;
#pragma unroll
    for (int x = 0; x < 8; x++) out[b * 64 + r * 8 + x] = (uint8_t)(row >> (8 * x));
}

constexpr int kFBlocks = 32;  // FDCT blocks per CTA (8 threads each)

__global__ void __launch_bounds__(kFBlocks * 8) fdct_blocks(const uint8_t *samples, const uint8_t *qt,
                                                             const float *rq, uint64_t n, int32_t *out,
                                                             unsigned long long *exact) {
    __shared__ float s_in[kFBlocks][8][9];
    __shared__ float s_row[kFBlocks][8][9];
    __shared__ float s_mag[kFBlocks][8][9];
    __shared__ uint8_t s_raw[kFBlocks][64];
    const int lb = threadIdx.x >> 3, r = threadIdx.x & 7;
    const uint64_t b = (uint64_t)blockIdx.x * kFBlocks + lb;
    const bool valid = b < n;
    if (valid) {
#pragma unroll
        for (int x = 0; x < 8; x++) {
            const uint8_t p = samples[b * 64 + r * 8 + x];
            s_raw[lb][r * 8 + x] = p;
            s_in[lb][r][x] = (float)p - 128.0f;
        }
    }
    __syncthreads();
    if (valid) {
#pragma unroll
        for (int u = 0; u < 8; u++) fdct_row_pass(s_in[lb][r], u, s_row[lb][r][u], s_mag[lb][r][u]);
    }
    __syncthreads();
    if (!valid) return;
    const int u = r;
    uint32_t n_exact = 0;
    for (int v = 0; v < 8; v++) {
        bool ex;
        out[b * 64 + v * 8 + u] = fdct_quantise(&s_row[lb][0][0], &s_mag[lb][0][0], 9, s_raw[lb], u, v,
                                                qt[b * 64 + v * 8 + u], rq[b * 64 + v * 8 + u], ex);
        n_exact += ex;
    }
    if (n_exact) atomicAdd(exact, (unsigned long long)n_exact);
}

template <class T>
cudaError_t upload(T **d, const T *h, size_t count) {
    cudaError_t e = cudaMalloc((void **)d, count * sizeof(T) + 16);
    if (e != cudaSuccess) return e;
    return cudaMemcpy(*d, h, count * sizeof(T), cudaMemcpyHostToDevice);
}

}  // namespace
}  // namespace mmr

using namespace mmr;

// Each entry runs n blocks (host arrays in, host arrays out) and returns a CUDA
// error code (0 = success); *exact receives how many samples or coefficients the
// binary64 reference order decided.
extern "C" int harness_jpeg_idct(const int32_t *c, uint64_t n, uint8_t *out, unsigned long long *exact) {
    int32_t *dc = nullptr;
    uint8_t *dout = nullptr;
    unsigned long long *dex = nullptr;
    long long *dfix = nullptr;
    static long long fix[kFixEntries];
    build_jpeg_fixed(fix);
    cudaError_t e = upload(&dc, c, n * 64);
    if (e == cudaSuccess) e = upload(&dfix, fix, (size_t)kFixEntries);
    if (e == cudaSuccess) e = cudaMalloc((void **)&dout, n * 64);
    if (e == cudaSuccess) e = cudaMalloc((void **)&dex, 8);
    if (e == cudaSuccess) e = cudaMemset(dex, 0, 8);
    if (e == cudaSuccess && n) {
        jpeg_idct_blocks<<<(unsigned)((n + kJBlocks - 1) / kJBlocks), kJBlocks * 4>>>(dc, n, dfix, dout, dex);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, n * 64, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(exact, dex, 8, cudaMemcpyDeviceToHost);
    cudaFree(dc);
    cudaFree(dfix);
    cudaFree(dout);
    cudaFree(dex);
    return (int)e;
}

extern "C" int harness_dv_idct(const int32_t *c, const uint8_t *modes, uint64_t n, uint8_t *out) {
    int32_t *dc = nullptr;
    uint8_t *dm = nullptr, *dout = nullptr;
    long long *dfix = nullptr;
    static long long fix[2 * kFixEntries];
    build_dv_fixed(fix, fix + kFixEntries);
    cudaError_t e = upload(&dc, c, n * 64);
    if (e == cudaSuccess) e = upload(&dm, modes, n);
    if (e == cudaSuccess) e = upload(&dfix, fix, 2 * (size_t)kFixEntries);
    if (e == cudaSuccess) e = cudaMalloc((void **)&dout, n * 64);
    if (e == cudaSuccess && n) {
        dv_idct_blocks<<<(unsigned)((n + 31) / 32), 256>>>(dc, dm, n, dfix, dout);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, n * 64, cudaMemcpyDeviceToHost);
    cudaFree(dc);
    cudaFree(dm);
    cudaFree(dfix);
    cudaFree(dout);
    return (int)e;
}

extern "C" int harness_fdct(const uint8_t *samples, const uint8_t *qt, const float *rq, uint64_t n, int32_t *out,
                            unsigned long long *exact) {
    uint8_t *ds = nullptr, *dq = nullptr;
    float *dr = nullptr;
    int32_t *dout = nullptr;
    unsigned long long *dex = nullptr;
    cudaError_t e = upload(&ds, samples, n * 64);
    if (e == cudaSuccess) e = upload(&dq, qt, n * 64);
    if (e == cudaSuccess) e = upload(&dr, rq, n * 64);
    if (e == cudaSuccess) e = cudaMalloc((void **)&dout, n * 64 * sizeof(int32_t));
    if (e == cudaSuccess) e = cudaMalloc((void **)&dex, 8);
    if (e == cudaSuccess) e = cudaMemset(dex, 0, 8);
    if (e == cudaSuccess && n) {
        fdct_blocks<<<(unsigned)((n + kFBlocks - 1) / kFBlocks), kFBlocks * 8>>>(ds, dq, dr, n, dout, dex);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, n * 64 * sizeof(int32_t), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(exact, dex, 8, cudaMemcpyDeviceToHost);
    cudaFree(ds);
    cudaFree(dq);
    cudaFree(dr);
    cudaFree(dout);
    cudaFree(dex);
    return (int)e;
}
