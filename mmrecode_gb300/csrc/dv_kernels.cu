// DV25 decode kernels for sm_103a.
//
//   dif_check  one thread per 80-byte DIF block: identifier vs canonical layout
//              (crates/codecs/dv/src/dif.rs:181-253).
//   segment    one thread per video segment (5 macroblocks, 30 blocks):
//              DC/mode/class fields, VLC decode and the three-level spill of
//              unused bits -- block region, macroblock pool, segment pool
//              (dv/src/decoder.rs:152-317); writes dequantised coefficients.
//   resolve    first failing segment per frame (sequential semantics).
//   idct       one thread per sample: fp32 separable 8-8 / 2-4-8 transform with
//              a proven error bound; samples within it of a rounding boundary
//              get the reference's binary64 sum in its exact operation order
//              (decoder.rs:520-602); then placement (decoder.rs:395-505).
#include <cuda_runtime.h>

#include "dv_idct_core.h"
#include "kernels.h"
#include "rounding.h"
#include "tables.h"

namespace mmr {

__constant__ int c_dv_zz88[64] = MMR_ZIGZAG_INIT;
__constant__ int c_dv_zz248[64] = MMR_DV_ZIGZAG_248_INIT;
__constant__ uint8_t c_dv_shifts[88] = MMR_DV_QUANT_SHIFTS_INIT;
__constant__ int c_dv_qoff[4] = MMR_DV_QUANT_OFFSET_INIT;
__constant__ int32_t c_dv_w88[64] = MMR_DV_IWEIGHT_88_INIT;
__constant__ int32_t c_dv_w248[64] = MMR_DV_IWEIGHT_248_INIT;

namespace {

__device__ __forceinline__ uint32_t upper_index32(const uint32_t *first, uint32_t n, uint32_t x) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (first[mid] <= x) lo = mid;
        else hi = mid;
    }
    return lo;
}

// dif.rs:235-253 expected_id
__device__ __forceinline__ void expected_id(uint32_t pos, uint32_t *section, uint32_t *number) {
    if (pos == 0) {
        *section = 0;
        *number = 0;
    } else if (pos <= 2) {
        *section = 1;
        *number = pos - 1;
    } else if (pos <= 5) {
        *section = 2;
        *number = pos - 3;
    } else {
        uint32_t av = pos - 6;
        if (av % 16 == 0) {
            *section = 3;
            *number = av / 16;
        } else {
            *section = 4;
            *number = (av - av / 16 - 1) & 0xff;
        }
    }
}

__global__ void dif_check_kernel(DvLaunch L) {
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= L.n_dif) return;
    uint32_t f = upper_index32(L.dif_first, L.n_frames, g);
    uint32_t local = g - L.dif_first[f];
    const uint8_t *b = L.frames[f].in + (size_t)local * 80;
    uint32_t es, en;
    expected_id(local % 150, &es, &en);
    bool bad = (uint32_t)(b[0] >> 5) != es || (uint32_t)(b[1] >> 4) != local / 150 || (uint32_t)b[2] != en;
    L.flags[g] = bad ? 1 : 0;
}

// ---- bit buffers (MSB-first, 32-bit words) ----

__device__ __forceinline__ uint32_t get32(const uint32_t *w, uint32_t bit) {
    uint32_t i = bit >> 5, r = bit & 31;
    uint32_t hi = w[i] << r;
    return r ? hi | (w[i + 1] >> (32 - r)) : hi;
}

// Appends bits [start, start+n) of src to dst (which holds dn bits, zero beyond).
__device__ __forceinline__ void append_bits(uint32_t *dst, uint32_t &dn, const uint32_t *src, uint32_t start,
                                            uint32_t n) {
    while (n) {
        uint32_t k = n < 32 ? n : 32;
        uint32_t v = get32(src, start) >> (32 - k);  // k bits, right-aligned
        uint32_t i = dn >> 5, r = dn & 31;
        // place v's k bits at bit offset r of word i
        uint64_t sh = (uint64_t)v << (64 - r - k);
        dst[i] |= (uint32_t)(sh >> 32);
        if (r + k > 32) dst[i + 1] |= (uint32_t)sh;
        dn += k;
        start += k;
        n -= k;
    }
}

struct DvBlock {
    uint8_t position;
    uint8_t complete;
    uint8_t mode;     // 1 = 2-4-8
    uint8_t cls;
    uint16_t pval;    // partial bits (< 16), right-aligned
    uint8_t plen;
    uint8_t pad;
};

// consume_ac (decoder.rs:245-284) on the virtual stream (partial bits ++ buf[pos, end)).
// On completion *pos is left after the EOB; otherwise the remaining bits become the
// block's partial and *pos == end.
__device__ void consume_ac(DvBlock &b, const uint32_t *buf, uint32_t &pos, uint32_t end, int16_t *coef,
                           uint32_t qno, const uint32_t *__restrict__ vlc, bool &bad_vlc) {
    if (b.complete) return;
    uint32_t pval = b.pval;
    int plen = b.plen;
    b.plen = 0;
    b.pval = 0;
    for (;;) {
        uint32_t avail = (uint32_t)plen + (end - pos);
        // next 16 bits of (partial ++ input), zero-padded
        uint32_t w16;
        if (plen) {
            uint32_t rest = get32(buf, pos) >> 16;  // 16 bits from pos (beyond end: don't care, masked below)
            w16 = ((pval << (16 - plen)) | (rest >> plen)) & 0xffffu;
        } else {
            w16 = get32(buf, pos) >> 16;
        }
        if (avail < 16) w16 &= 0xffffu << (16 - avail);
        uint32_t e = vlc[w16 >> (16 - kDvVlcL1Bits)];
        if (e & 0x80000000u) e = vlc[(e & 0xffffu) + (w16 & ((1u << (16 - kDvVlcL1Bits)) - 1))];
        uint32_t len = e & 31;
        if (len != 0 && len <= avail) {
            // consume len bits: all partial bits first (a partial never holds a whole code)
            if ((int)len <= plen) {
                plen -= (int)len;
                pval &= (1u << plen) - 1;
            } else {
                pos += len - (uint32_t)plen;
                plen = 0;
                pval = 0;
            }
            uint32_t run = (e >> 5) & 127;
            int32_t level = (int32_t)((e >> 12) & 511) - 256;
            uint32_t p = b.position + run + 1;
            if (p >= 64) {
                b.position = 64;
                b.complete = 1;
                return;
            }
            b.position = (uint8_t)p;
            if (level != 0) {
                // inverse_factor_for_encoding (decoder.rs:290-310)
                uint32_t q = qno + (uint32_t)c_dv_qoff[b.cls];
                uint32_t area = p <= 5 ? 0 : p <= 20 ? 1 : p <= 42 ? 2 : 3;
                int32_t weight = b.mode ? c_dv_w248[p] : c_dv_w88[p];
                int32_t factor = weight << (c_dv_shifts[q * 4 + area] + 1 + (b.cls == 3));
                int32_t lv = (level * factor + 8192) >> 14;
                coef[b.mode ? c_dv_zz248[p] : c_dv_zz88[p]] = (int16_t)lv;
            }
        } else if (avail < 16) {
            // save as partial: remaining partial bits then the rest of the input
            uint32_t v = pval;
            int n = plen;
            uint32_t in_n = end - pos;
            if (in_n) {
                v = (v << in_n) | (get32(buf, pos) >> (32 - in_n));
                n += (int)in_n;
            }
            b.pval = (uint16_t)v;
            b.plen = (uint8_t)n;
            pos = end;
            return;
        } else {
            bad_vlc = true;  // unreachable: the DV VLC code is complete (Kraft sum 1)
            pos = end;
            return;
        }
    }
}

constexpr int kSegThreads = 64;

__global__ void __launch_bounds__(kSegThreads) segment_kernel(DvLaunch L) {
    uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= L.n_segments) return;
    uint32_t f = upper_index32(L.seg_first, L.n_frames, g);
    const DvFrame &F = L.frames[f];
    uint32_t local = g - L.seg_first[f];
    uint32_t sequence = local / 27, slot = local % 27;
    uint16_t kind = kDiagNone;

    uint32_t dif[5];
    for (int m = 0; m < 5; m++) {
        uint32_t vn = slot * 5 + m;
        dif[m] = sequence * 150 + 7 + (vn / 15) * 16 + vn % 15;
        if (kind == kDiagNone && L.flags[F.dif_first + dif[m]]) kind = kDvDamagedId;
    }
    if (kind == kDiagNone) {
        // payload words of the 5 macroblocks (bytes 4..80 of each DIF block)
        uint32_t pay[5 * 19 + 1];
        for (int m = 0; m < 5; m++) {
            const uint8_t *src = F.in + (size_t)dif[m] * 80 + 4;
            for (int i = 0; i < 19; i++)
                pay[m * 19 + i] = ((uint32_t)src[4 * i] << 24) | ((uint32_t)src[4 * i + 1] << 16) |
                                  ((uint32_t)src[4 * i + 2] << 8) | (uint32_t)src[4 * i + 3];
        }
        pay[95] = 0;
        uint32_t segpool[5 * 19 + 2];
        for (int i = 0; i < 97; i++) segpool[i] = 0;
        uint32_t segn = 0;
        DvBlock blk[30];
        int16_t *coef = L.coef + (F.blk_off + (uint64_t)local * 30) * 64;
        bool bad_vlc = false;
        const uint32_t kRegion[6] = {0, 112, 224, 336, 448, 528};
        const uint32_t kBits[6] = {112, 112, 112, 112, 80, 80};
        for (int m = 0; m < 5; m++) {
            // decode_macroblock (decoder.rs:193-223)
            uint32_t qno = F.in[(size_t)dif[m] * 80 + 3] & 0x0f;
            const uint32_t *w = pay + m * 19;
            uint32_t mbpool[20];
            for (int i = 0; i < 20; i++) mbpool[i] = 0;
            uint32_t mbn = 0;
            for (int j = 0; j < 6; j++) {
                DvBlock &b = blk[m * 6 + j];
                uint32_t r0 = kRegion[j];
                uint32_t head = get32(w, r0) >> 20;  // 12 bits: dc(9) mode(1) class(2)
                int32_t dc = (int32_t)(head >> 3);
                if (dc & 0x100) dc -= 512;
                b.position = 0;
                b.complete = 0;
                b.mode = (head >> 2) & 1;
                b.cls = head & 3;
                b.pval = 0;
                b.plen = 0;
                int16_t *bc = coef + (m * 6 + j) * 64;
                bc[0] = (int16_t)(dc * 4 + 1024);
                uint32_t pos = r0 + 12, end = r0 + kBits[j];
                consume_ac(b, w, pos, end, bc, qno, L.vlc, bad_vlc);
                if (b.complete) append_bits(mbpool, mbn, w, pos, end - pos);
            }
            // consume_pool over the macroblock (decoder.rs:235-243)
            uint32_t pos = 0;
            for (int j = 0; j < 6; j++) {
                DvBlock &b = blk[m * 6 + j];
                if (!b.complete && pos < mbn)
                    consume_ac(b, mbpool, pos, mbn, coef + (m * 6 + j) * 64, qno, L.vlc, bad_vlc);
            }
            if (pos < mbn) append_bits(segpool, segn, mbpool, pos, mbn - pos);
        }
        // consume_pool_for_macroblocks (decoder.rs:225-233)
        uint32_t pos = 0;
        for (int j = 0; j < 30; j++) {
            DvBlock &b = blk[j];
            if (!b.complete && pos < segn) {
                uint32_t qno = F.in[(size_t)dif[j / 6] * 80 + 3] & 0x0f;
                consume_ac(b, segpool, pos, segn, coef + j * 64, qno, L.vlc, bad_vlc);
            }
        }
        if (bad_vlc) kind = kDvBadVlc;
        else
            for (int j = 0; j < 30; j++)
                if (!blk[j].complete) {
                    kind = kDvIncomplete;
                    break;
                }
        uint8_t *modes = L.modes + F.blk_off + (uint64_t)local * 30;
        for (int j = 0; j < 30; j++) modes[j] = blk[j].mode;
    }
    L.seg_err[g] = (uint8_t)kind;
    if (kind != kDiagNone) {
        atomicMin(&L.states[f].bad_segment, local);
        atomicAdd(&L.states[f].failed, 1u);
    }
}

__global__ void dv_resolve_kernel(DvLaunch L) {
    uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= L.n_frames) return;
    DvState *st = &L.states[f];
    uint32_t bad = st->bad_segment;
    if (bad != 0xffffffffu) {
        uint16_t kind = L.seg_err[L.frames[f].seg_first + bad];
        st->diag = make_diag(kind, 0, bad % 27, bad / 27);
        if (!L.frames[f].conceal) L.item_ok[L.frames[f].item] = 0;
    }
}

// decoder.rs:395-422 macroblock_coordinates (in 8-sample units)
__device__ __forceinline__ void mb_coords(bool pal, uint32_t seqs, uint32_t sequence, uint32_t slot, uint32_t m,
                                          uint32_t *mbx, uint32_t *mby) {
    const uint32_t OFF[5] = {2, 6, 8, 0, 4};
    const uint32_t SHUF3[5] = {18, 9, 27, 0, 36};
    const uint32_t LSTART[5] = {9, 4, 13, 0, 18};
    if (pal) {
        // SERPENT1[slot] = 0,1,2,2,1,0 repeating
        uint32_t s6 = slot % 6;
        uint32_t serp1 = s6 < 3 ? s6 : 5 - s6;
        uint32_t x = SHUF3[m] + slot / 3;
        uint32_t y = serp1 + ((sequence + OFF[m]) % seqs) * 3;
        *mbx = x * 2;
        *mby = y * 2;
    } else {
        uint32_t row = (sequence + OFF[m]) % seqs;
        uint32_t k = slot + ((m == 1 || m == 2) ? 3 : 0);
        uint32_t x = LSTART[m] + k / 6;
        // SERPENT2[k] = 0..5,5..0 repeating
        uint32_t k12 = k % 12;
        uint32_t serp2 = k12 < 6 ? k12 : 11 - k12;
        uint32_t y = serp2 + row * 6;
        if (x > 21) y = y * 2 - row * 6;
        *mbx = x * 4;
        *mby = y;
    }
}

constexpr int kIdctBlocks = 32;                  // blocks per CTA
constexpr int kIdctThreads = kIdctBlocks * 8;    // eight threads (rows) per block

// Stores the eight bytes of `row` at dst (any alignment).
__device__ __forceinline__ void store_row8(uint8_t *dst, unsigned long long row) {
    const uintptr_t a = reinterpret_cast<uintptr_t>(dst);
    if ((a & 7) == 0) {
        *reinterpret_cast<uint2 *>(dst) = make_uint2((uint32_t)row, (uint32_t)(row >> 32));
    } else if ((a & 3) == 0) {
        reinterpret_cast<uint32_t *>(dst)[0] = (uint32_t)row;
        reinterpret_cast<uint32_t *>(dst)[1] = (uint32_t)(row >> 32);
    } else {
#pragma unroll
        for (int x = 0; x < 8; x++) dst[x] = (uint8_t)(row >> (8 * x));
    }
}

__device__ __forceinline__ void store_row4(uint8_t *dst, uint32_t row) {
    if ((reinterpret_cast<uintptr_t>(dst) & 3) == 0) {
        *reinterpret_cast<uint32_t *>(dst) = row;
    } else {
#pragma unroll
        for (int x = 0; x < 4; x++) dst[x] = (uint8_t)(row >> (8 * x));
    }
}

// Eight threads per block, thread r producing row r: the fp32 row and column
// passes with the exact fallback (dv_idct_core.h), then placement
// (decoder.rs:432-505) with 8-byte row stores. A warp holds four blocks of one
// frame (frames start at multiples of 4 blocks: 8100 and 9720 blocks per frame),
// so one search per warp finds it; the eight threads of a block synchronise
// through their warp only.
__global__ void __launch_bounds__(kIdctThreads) dv_idct_kernel(DvLaunch L) {
    __shared__ __align__(16) int32_t s_c[kIdctBlocks][64];
    __shared__ __align__(16) float s_h[kIdctBlocks][64];
    __shared__ __align__(16) float s_wt[64];
    __shared__ __align__(16) float s_v4[16];
    dv_fill_tables(s_wt, s_v4);
    __syncthreads();
    const int lane = threadIdx.x & 31, lb = threadIdx.x >> 3, r = threadIdx.x & 7;
    const unsigned group_mask = 0xffu << (lane & 24);
    const uint64_t gb = (uint64_t)blockIdx.x * kIdctBlocks + lb;
    bool valid = gb < L.n_blocks;
    uint32_t f = 0;
    if (lane == 0 && valid) {
        uint32_t lo = 0, hi = L.n_frames;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (L.frames[mid].blk_off <= gb) lo = mid;
            else hi = mid;
        }
        f = lo;
    }
    f = __shfl_sync(0xffffffffu, f, 0);
    const DvFrame *F = &L.frames[f];
    bool failed = false, mode = false;
    uint32_t local_blk = 0;
    int4 lv = make_int4(0, 0, 0, 0);
    if (valid) {
        local_blk = (uint32_t)(gb - F->blk_off);
        valid = L.item_ok[F->item] != 0;
        if (valid) {
            failed = L.seg_err[F->seg_first + local_blk / 30] != 0;
            mode = L.modes[gb] != 0;
            if (!failed) lv = reinterpret_cast<const int4 *>(L.coef + gb * 64)[r];  // row r: 8 int16
        }
    }
    int32_t *c = s_c[lb];
    {
        const int16_t *q = reinterpret_cast<const int16_t *>(&lv);
        int32_t row[8];
#pragma unroll
        for (int u = 0; u < 8; u++) row[u] = q[u];
        reinterpret_cast<int4 *>(c + r * 8)[0] = make_int4(row[0], row[1], row[2], row[3]);
        reinterpret_cast<int4 *>(c + r * 8)[1] = make_int4(row[4], row[5], row[6], row[7]);
    }
    // C1 of the block (fp32 for the first decision, exact for the second) and
    // whether any AC coefficient is nonzero, over its eight threads
    float a = 0.0f;
    int32_t ai = 0;
    bool ac = false;
    {
        const int16_t *q = reinterpret_cast<const int16_t *>(&lv);
#pragma unroll
        for (int u = 0; u < 8; u++) {
            a += fabsf((float)q[u]);
            ai += abs((int32_t)q[u]);
            ac |= (r | u) != 0 && q[u] != 0;
        }
    }
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) {
        a += __shfl_xor_sync(0xffffffffu, a, o);
        ai += __shfl_xor_sync(0xffffffffu, ai, o);
    }
    const bool flat = (__ballot_sync(0xffffffffu, ac) & group_mask) == 0;
    const bool active = valid && !failed;
    __syncwarp();
    if (active && !flat) dv_row_pass8(c, s_wt, mode, r, s_h[lb] + r * 8);
    __syncwarp();
    unsigned long long row = 0;
    uint32_t und = 0;
    if (active) und = dv_row_fp32(c, s_h[lb], s_wt, s_v4, mode, r, a, flat, lane & 24, group_mask, &row);
    dv_resolve_row(und, row, c, mode, r, ai, L.fixw);  // every lane of the warp takes part
    if (!valid) return;
    // placement (decoder.rs:432-505)
    const uint32_t seg = local_blk / 30, j = local_blk % 30;
    const uint32_t sequence = seg / 27, slot = seg % 27, m = j / 6, bi = j % 6;
    uint32_t mbx, mby;
    mb_coords(F->pal != 0, F->sequences, sequence, slot, m, &mbx, &mby);
    const uint32_t X = mbx * 8, Y = mby * 8;
    const uint32_t W = F->width, H = F->height, cw = F->cw, ch = F->ch;
    uint8_t *yp = F->planes, *cbp = F->planes + (size_t)W * H, *crp = cbp + (size_t)cw * ch;
    const bool chroma = bi >= 4;
    if (failed) row = 0x0101010101010101ull * (chroma ? 128u : 16u);
    if (F->pal || mbx >= 88) {
        if (!chroma) {
            store_row8(yp + (size_t)(Y + (bi >> 1) * 8 + r) * W + X + (bi & 1) * 8, row);
        } else {
            uint8_t *plane = bi == 4 ? crp : cbp;
            if (F->pal) {
                store_row8(plane + (size_t)(Y / 2 + r) * cw + X / 2, row);
            } else {  // put_split_chroma: columns 0-3 to rows y.., 4-7 to rows y+8..
                store_row4(plane + (size_t)(Y + r) * cw + X / 4, (uint32_t)row);
                store_row4(plane + (size_t)(Y + 8 + r) * cw + X / 4, (uint32_t)(row >> 32));
            }
        }
    } else {
        if (!chroma) store_row8(yp + (size_t)(Y + r) * W + X + bi * 8, row);
        else store_row8((bi == 4 ? crp : cbp) + (size_t)(Y + r) * cw + X / 4, row);
    }
}

}  // namespace

void launch_dv_decode(const DvLaunch &L, cudaStream_t s) {
    if (L.n_dif) dif_check_kernel<<<(L.n_dif + 255) / 256, 256, 0, s>>>(L);
    if (L.n_segments) segment_kernel<<<(L.n_segments + kSegThreads - 1) / kSegThreads, kSegThreads, 0, s>>>(L);
    if (L.n_frames) dv_resolve_kernel<<<(L.n_frames + 127) / 128, 128, 0, s>>>(L);
}

void launch_dv_idct(const DvLaunch &L, cudaStream_t s) {
    if (L.n_blocks == 0) return;
    const uint64_t grid = (L.n_blocks + kIdctBlocks - 1) / kIdctBlocks;
    dv_idct_kernel<<<(unsigned)grid, kIdctThreads, 0, s>>>(L);
}

}  // namespace mmr
