// Fused dequantisation + IDCT + chroma upsampling + YCbCr -> RGB24 for MJPEG
// frames with RGB output (sm_103a).
//
// For the common layouts (three components, luma sampled hmax x vmax with
// (hmax, vmax) in {(1,1), (2,1), (2,2)}, chroma 1x1) the reference's nearest
// chroma sample of pixel (x, y) (crates/cli/src/terminal_preview.rs:7159-7236,
// x * cw / W with cw = ceil(W / hmax)) is x / hmax: for x < W,
// x * ceil(W/2) / W = x/2 + x / (2W) rounds down to floor(x / 2). So every pixel
// of an MCU takes its chroma from the same MCU, and one CTA turns a strip of MCUs
// straight from coefficients into RGB: no planar samples go through HBM.
//
// A CTA: NM consecutive MCUs of one MCU row, four threads per block. Samples the
// fp32 transform cannot decide (idct_core.h) are settled inside the CTA, a warp
// per block: the exact fixed-point value, or the reference's binary64 order for
// genuine near-ties (settle_samples), before the colour conversion reads them.
#include <cuda_runtime.h>

#include "idct_core.h"
#include "kernels.h"

namespace mmr {
namespace {

constexpr int kFStride = 68;  // floats per staged block (16-byte rows, conflict-free over 8 blocks)

// Four channel values saturated to 0..255 and packed, b0 in the low byte
// (cvt.pack.sat: d = c << 16 | sat(a) << 8 | sat(b)).
__device__ __forceinline__ uint32_t pack4_sat_u8(int32_t b0, int32_t b1, int32_t b2, int32_t b3) {
    uint32_t hi, d;
    asm("cvt.pack.sat.u8.s32.b32 %0, %1, %2, %3;" : "=r"(hi) : "r"(b3), "r"(b2), "r"(0));
    asm("cvt.pack.sat.u8.s32.b32 %0, %1, %2, %3;" : "=r"(d) : "r"(b1), "r"(b0), "r"(hi));
    return d;
}

template <int HM, int VM, int NM>
struct FusedShape {
    static constexpr int BPM = HM * VM + 2;  // blocks per MCU
    static constexpr int NB = NM * BPM;      // blocks per CTA
    static constexpr int THREADS = NB * 4;
    static constexpr int YW = NM * HM * 8;   // luma tile width (samples)
    static constexpr int YH = VM * 8;
    static constexpr int CW = NM * 8;        // chroma tile width
    static constexpr int RW = YW * 3;        // RGB bytes per tile row
};

// MCUs per CTA of each launch slot (layout variant * 2 + wide): a narrow and a
// wide strip per layout, picked per frame class by the autotuner (wide by default)
__host__ __device__ constexpr int fused_slot_nm(int slot) {
    return slot == 0 ? 8 : slot == 1 ? 16 : slot == 2 || slot == 4 ? 4 : 8;
}

template <int HM, int VM, int NM>
struct FusedSmem {
    using Sh = FusedShape<HM, VM, NM>;
    __align__(16) float f[Sh::NB * kFStride];
    __align__(16) uint8_t y[Sh::YH * Sh::YW];
    __align__(16) uint8_t c[2][8 * Sh::CW];
    __align__(16) uint8_t rgb[Sh::YH * Sh::RW];
    __align__(16) float q[3][64];
    unsigned long long mask[Sh::NB];  // samples left to the exact pass, per block
    unsigned long long blk[Sh::NB];
    int32_t cx[Sh::THREADS / 32][64];  // per warp: exact coefficients of the block it settles
    uint32_t n;
};

// Converts MCUs mx0 .. mx0+NM-1 of MCU row my of job J to RGB; undecided samples
// are settled first, a warp per block (settle_samples).
template <int HM, int VM, int NM>
__device__ __forceinline__ void fused_tile(const JpegLaunch &L, const FusedLaunch &FL, uint32_t job, uint32_t my,
                                           uint32_t mx0, FusedSmem<HM, VM, NM> &S) {
    using Sh = FusedShape<HM, VM, NM>;
    const FusedJob J = FL.jobs[job];
    const JFrame &F = L.frames[J.frame];
    const JComp *comps = L.comps + F.comp_off;
    if (threadIdx.x == 0) S.n = 0;
    for (uint32_t i = threadIdx.x; i < 3 * 64; i += blockDim.x)
        S.q[i >> 6][i & 63] = (float)L.quant[F.quant_off + comps[i >> 6].q * 64 + (i & 63)];
    const uint32_t nm = min((uint32_t)NM, F.mcu_cols - mx0);
    const uint32_t lb = threadIdx.x >> 2, q = threadIdx.x & 3;
    const uint32_t m = lb / Sh::BPM, i = lb % Sh::BPM;
    const bool valid = lb < (uint32_t)Sh::NB && m < nm;
    const uint32_t comp = i < HM * VM ? 0 : i - HM * VM + 1;
    uint64_t g = 0;
    if (valid) {
        const JComp &C = comps[comp];
        const uint32_t mx = mx0 + m;
        if (comp == 0) g = F.blk_off + C.blk_base + (uint64_t)(my * VM + i / HM) * C.bw + mx * HM + i % HM;
        else g = F.blk_off + C.blk_base + (uint64_t)my * C.bw + mx;
        if (q == 0) S.blk[lb] = g;
    }
    __syncthreads();  // q, n
    float *blk = S.f + lb * kFStride;
    float l1 = valid ? stage_rows(block_levels(L, g), L.dc, g, q, S.q[comp], blk) : 0.0f;
#pragma unroll
    for (int o = 1; o < 4; o <<= 1) l1 += __shfl_xor_sync(0xffffffffu, l1, o);
    __syncwarp();
    unsigned long long mask = 0;
    if (valid) {
        uint8_t *out;
        int stride;
        if (comp == 0) {
            out = S.y + (i / HM) * 8 * Sh::YW + (m * HM + i % HM) * 8;
            stride = Sh::YW;
        } else {
            out = S.c[comp - 1] + m * 8;
            stride = Sh::CW;
        }
        mask = idct_block(blk, q, l1, out, stride);
    }
#pragma unroll
    for (int o = 1; o < 4; o <<= 1) mask |= __shfl_xor_sync(0xffffffffu, mask, o);
    if (q == 0 && lb < (uint32_t)Sh::NB) {
        S.mask[lb] = mask;
        if (mask) atomicAdd(&S.n, (uint32_t)__popcll(mask));
    }
    __syncthreads();
    const uint32_t n_exact = S.n;
    if (threadIdx.x == 0 && n_exact) atomicAdd(L.fix_count + 1, n_exact);
    if (n_exact) {  // a warp per block with undecided samples (settle_samples)
        const uint32_t w = threadIdx.x >> 5, nw = blockDim.x >> 5, lane = threadIdx.x & 31;
        int32_t *cx = S.cx[w];
        for (uint32_t b = w; b < (uint32_t)Sh::NB; b += nw) {
            const unsigned long long bits = S.mask[b];
            if (!bits) continue;
            const uint32_t bm = b / Sh::BPM, bi = b % Sh::BPM;
            const uint32_t bc = bi < HM * VM ? 0 : bi - HM * VM + 1;
            const uint64_t bg = S.blk[b];
            const uint16_t *Q = L.quant + F.quant_off + comps[bc].q * 64;
            const int16_t *lv = block_levels(L, bg);
            cx[lane] = lane == 0 ? L.dc[bg] : (int32_t)lv[lane] * (int32_t)Q[lane];
            cx[lane + 32] = (int32_t)lv[lane + 32] * (int32_t)Q[lane + 32];
            __syncwarp();
            settle_samples(L.fixw, cx, bits, [&](int y, int x, uint8_t smp) {
                if (bc == 0) S.y[((bi / HM) * 8 + y) * Sh::YW + (bm * HM + bi % HM) * 8 + x] = smp;
                else S.c[bc - 1][y * Sh::CW + bm * 8 + x] = smp;
            });
            __syncwarp();
        }
    }
    __syncthreads();
    // colour conversion (terminal_preview.rs:7308-7330, full range). When every row
    // starts 16-byte aligned (width a multiple of 16, aligned output; x0 is a
    // multiple of 64 pixels) a thread converts 16 pixels from one 16-byte luma
    // load and stores them as three 16-byte vectors, consecutive threads writing
    // consecutive 48-byte runs. Otherwise four pixels per thread: one 32-bit luma
    // load, three 32-bit words of RGB, stored straight from registers when rows
    // start 4-aligned, else through a shared-memory tile and a byte-exact copy.
    // Pixels past the visible width are computed from padding and never stored.
    const uint32_t x0 = mx0 * HM * 8, y0 = my * VM * 8;
    const uint32_t vis_w = min((uint32_t)(nm * HM * 8), J.width - x0);
    const uint32_t vis_h = min((uint32_t)Sh::YH, J.height - y0);
    if ((((reinterpret_cast<uintptr_t>(J.out) | J.width | vis_w) & 15) == 0)) {  // uniform over the CTA
        for (uint32_t p = threadIdx.x; p < vis_h * (Sh::YW / 16); p += blockDim.x) {
            const uint32_t ly = p / (Sh::YW / 16), lx = (p - ly * (Sh::YW / 16)) * 16;
            if (lx >= vis_w) continue;
            const uint4 yv = *reinterpret_cast<const uint4 *>(S.y + ly * Sh::YW + lx);
            const uint8_t *cbr = S.c[0] + (ly / VM) * Sh::CW + lx / HM;
            const uint8_t *crr = S.c[1] + (ly / VM) * Sh::CW + lx / HM;
            uint32_t cb[4], cr[4];  // the 16 / HM chroma bytes of the 16 pixels
            if (HM == 2) {
                const uint2 a = *reinterpret_cast<const uint2 *>(cbr), b = *reinterpret_cast<const uint2 *>(crr);
                cb[0] = a.x, cb[1] = a.y, cr[0] = b.x, cr[1] = b.y;
                cb[2] = cb[3] = cr[2] = cr[3] = 0;
            } else {
                const uint4 a = *reinterpret_cast<const uint4 *>(cbr), b = *reinterpret_cast<const uint4 *>(crr);
                cb[0] = a.x, cb[1] = a.y, cb[2] = a.z, cb[3] = a.w;
                cr[0] = b.x, cr[1] = b.y, cr[2] = b.z, cr[3] = b.w;
            }
            const uint32_t ys[4] = {yv.x, yv.y, yv.z, yv.w};
            uint32_t word[12];
#pragma unroll
            for (int g = 0; g < 4; g++) {
                int32_t ch[12];
#pragma unroll
                for (int k = 0; k < 4; k++) {
                    const int px = 4 * g + k, ci = px / HM;
                    const int32_t Y = (int32_t)((ys[g] >> (8 * k)) & 0xff);
                    const int32_t u = (int32_t)((cb[ci >> 2] >> (8 * (ci & 3))) & 0xff) - 128;
                    const int32_t w = (int32_t)((cr[ci >> 2] >> (8 * (ci & 3))) & 0xff) - 128;
                    ch[3 * k + 0] = Y + ((359 * w + 128) >> 8);
                    ch[3 * k + 1] = Y - ((88 * u + 183 * w + 128) >> 8);
                    ch[3 * k + 2] = Y + ((454 * u + 128) >> 8);
                }
#pragma unroll
                for (int j = 0; j < 3; j++)
                    word[3 * g + j] = pack4_sat_u8(ch[4 * j], ch[4 * j + 1], ch[4 * j + 2], ch[4 * j + 3]);
            }
            uint4 *o = reinterpret_cast<uint4 *>(J.out + ((uint64_t)(y0 + ly) * J.width + x0 + lx) * 3);
            o[0] = make_uint4(word[0], word[1], word[2], word[3]);
            o[1] = make_uint4(word[4], word[5], word[6], word[7]);
            o[2] = make_uint4(word[8], word[9], word[10], word[11]);
        }
        return;
    }
    const bool direct = ((reinterpret_cast<uintptr_t>(J.out) | J.width) & 3) == 0;
    for (uint32_t p = threadIdx.x; p < vis_h * (Sh::YW / 4); p += blockDim.x) {
        const uint32_t ly = p / (Sh::YW / 4), lx = (p - ly * (Sh::YW / 4)) * 4;
        if (lx >= vis_w) continue;
        const uint32_t yq = *reinterpret_cast<const uint32_t *>(S.y + ly * Sh::YW + lx);
        const uint8_t *cbr = S.c[0] + (ly / VM) * Sh::CW + lx / HM;
        const uint8_t *crr = S.c[1] + (ly / VM) * Sh::CW + lx / HM;
        int32_t ch[12];
#pragma unroll
        for (int k = 0; k < 4; k++) {
            const int32_t Y = (int32_t)((yq >> (8 * k)) & 0xff);
            const int32_t u = (int32_t)cbr[k / HM] - 128, w = (int32_t)crr[k / HM] - 128;
            ch[3 * k + 0] = Y + ((359 * w + 128) >> 8);
            ch[3 * k + 1] = Y - ((88 * u + 183 * w + 128) >> 8);
            ch[3 * k + 2] = Y + ((454 * u + 128) >> 8);
        }
        uint32_t word[3];
#pragma unroll
        for (int j = 0; j < 3; j++) word[j] = pack4_sat_u8(ch[4 * j], ch[4 * j + 1], ch[4 * j + 2], ch[4 * j + 3]);
        uint32_t *o = direct ? reinterpret_cast<uint32_t *>(J.out + ((uint64_t)(y0 + ly) * J.width + x0 + lx) * 3)
                             : reinterpret_cast<uint32_t *>(S.rgb + ly * Sh::RW + lx * 3);
        o[0] = word[0];
        o[1] = word[1];
        o[2] = word[2];
    }
    if (direct) return;  // uniform over the CTA
    __syncthreads();
    // rows out: 16-byte stores when the row is aligned, bytes otherwise
    const uint32_t row_bytes = vis_w * 3;
    const uint32_t chunks = (row_bytes + 15) / 16;
    for (uint32_t c = threadIdx.x; c < vis_h * chunks; c += blockDim.x) {
        const uint32_t ly = c / chunks, ch = c - ly * chunks;
        uint8_t *dst = J.out + ((uint64_t)(y0 + ly) * J.width + x0) * 3;
        const uint8_t *src = S.rgb + ly * Sh::RW;
        const uint32_t b0 = ch * 16, b1 = min(b0 + 16, row_bytes);
        // (a tile row of 8 RGB pixels is 24 bytes: the source needs the check too)
        if (b1 - b0 == 16 && ((((uintptr_t)(dst + b0)) | ((uintptr_t)(src + b0))) & 15) == 0) {
            *reinterpret_cast<uint4 *>(dst + b0) = *reinterpret_cast<const uint4 *>(src + b0);
        } else {
            for (uint32_t k = b0; k < b1; k++) dst[k] = src[k];
        }
    }
}

// Main pass: a CTA per strip of MCUs.
template <int HM, int VM, int NM>
__global__ void __launch_bounds__(FusedShape<HM, VM, NM>::THREADS) idct_rgb_kernel(JpegLaunch L, FusedLaunch FL) {
    __shared__ __align__(16) FusedSmem<HM, VM, NM> S;
    __shared__ uint32_t s_job;
    if (threadIdx.x == 0) {
        uint32_t lo = 0, hi = FL.n_jobs;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (FL.cta_first[mid] <= blockIdx.x) lo = mid;
            else hi = mid;
        }
        s_job = lo;
    }
    __syncthreads();
    const uint32_t job = s_job;
    const FusedJob &J = FL.jobs[job];
    if (!L.item_ok[L.frames[J.frame].item]) return;
    const uint32_t strip = blockIdx.x - FL.cta_first[job];
    fused_tile<HM, VM, NM>(L, FL, job, strip / J.strips_x, (strip % J.strips_x) * NM, S);
}

}  // namespace

int fused_variant(uint32_t hmax, uint32_t vmax) {
    if (hmax == 1 && vmax == 1) return 0;
    if (hmax == 2 && vmax == 1) return 1;
    if (hmax == 2 && vmax == 2) return 2;
    return -1;
}

int fused_slot(int variant, bool wide) { return variant < 0 ? -1 : 2 * variant + (wide ? 1 : 0); }

uint32_t fused_slot_mcus(int slot) { return (uint32_t)fused_slot_nm(slot); }

uint32_t fused_strips_x(int slot, uint32_t mcu_cols) {
    const uint32_t nm = fused_slot_mcus(slot);
    return (mcu_cols + nm - 1) / nm;
}

template <int HM, int VM, int NM>
static void launch_variant(const JpegLaunch &L, const FusedLaunch &FL, cudaStream_t s) {
    if (!FL.n_ctas) return;
    idct_rgb_kernel<HM, VM, NM><<<FL.n_ctas, FusedShape<HM, VM, NM>::THREADS, 0, s>>>(L, FL);
}

int fused_launches(const FusedLaunch &FL) { return FL.n_ctas ? 1 : 0; }

void launch_jpeg_idct_rgb(const JpegLaunch &L, const FusedLaunch *FL, cudaStream_t s) {
    launch_variant<1, 1, fused_slot_nm(0)>(L, FL[0], s);
    launch_variant<1, 1, fused_slot_nm(1)>(L, FL[1], s);
    launch_variant<2, 1, fused_slot_nm(2)>(L, FL[2], s);
    launch_variant<2, 1, fused_slot_nm(3)>(L, FL[3], s);
    launch_variant<2, 2, fused_slot_nm(4)>(L, FL[4], s);
    launch_variant<2, 2, fused_slot_nm(5)>(L, FL[5], s);
}

}  // namespace mmr
