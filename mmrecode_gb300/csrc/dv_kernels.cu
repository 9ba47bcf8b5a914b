// DV25 decode kernels for sm_103a.
//
//   dif_check  one thread per 80-byte DIF block: identifier vs canonical layout
//              (crates/codecs/dv/src/dif.rs:181-253).
//   segment    a CTA per four video segments (5 macroblocks, 30 blocks each):
//              DC/mode/class fields, VLC decode and the three-level spill of
//              unused bits -- block region (a thread per block), macroblock pool
//              (a thread per macroblock), segment pool (a thread per segment)
//              (dv/src/decoder.rs:152-317); writes every dequantised coefficient.
//   resolve    first failing segment per frame (sequential semantics).
//   idct       eight threads per block (one per output row), 16 blocks per CTA:
//              fp32 separable 8-8 / 2-4-8 transform with a proven error bound;
//              samples within it of a rounding boundary are settled by the warp in
//              exact fixed point, or in the reference's binary64 order for genuine
//              near-ties (decoder.rs:520-602, dv_idct_core.h); then placement
//              (decoder.rs:395-505).
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

// A CTA per four video segments (dv/src/decoder.rs:152-317), in the reference's
// three levels, each level's independent parts in parallel:
//   1. a thread per block (120): DC/mode/class and the AC codes inside the
//      block's own region of its macroblock's payload;
//   2. a thread per macroblock (20): the leftover bits of its complete blocks, in
//      block order, make the macroblock pool, which its incomplete blocks
//      consume in order (decode_macroblock, decoder.rs:193-243);
//   3. a thread per segment (4): the macroblock pools' leftovers, in macroblock
//      order, make the segment pool, which the segment's incomplete blocks
//      consume in order (consume_pool_for_macroblocks, decoder.rs:225-233).
// Payload, pools and dequantised coefficients stay in shared memory; every
// block's 64 coefficients (zeros included) then leave as 16-byte stores.
constexpr int kSegPerCta = 4;
constexpr int kSegBlocks = kSegPerCta * 30;
constexpr int kSegThreads = 128;

struct SegSmem {
    __align__(16) int16_t coef[kSegBlocks][64];
    uint32_t pay[kSegPerCta][5 * 19 + 1];  // payload words of the five macroblocks (+1: reads past the end)
    uint32_t mbpool[kSegPerCta * 5][20];
    uint32_t segpool[kSegPerCta][5 * 19 + 2];
    DvBlock blk[kSegBlocks];
    uint16_t left_start[kSegBlocks], left_len[kSegBlocks];  // unused bits of a complete block's region
    uint16_t mb_pos[kSegPerCta * 5], mb_len[kSegPerCta * 5];
    uint32_t dif_off[kSegPerCta * 5];  // byte offset of each macroblock's DIF block in the frame
    uint32_t frame[kSegPerCta], local[kSegPerCta];
    uint8_t qno[kSegPerCta * 5];
    uint8_t bad[kSegBlocks];
    uint16_t kind[kSegPerCta];
};

__global__ void __launch_bounds__(kSegThreads) segment_kernel(DvLaunch L) {
    __shared__ SegSmem S;
    const uint32_t t = threadIdx.x;
    const uint32_t g0 = blockIdx.x * kSegPerCta;
    // segment records: frame, segment in frame, DIF blocks, damaged identifiers
    if (t < (uint32_t)kSegPerCta) {
        const uint32_t g = g0 + t;
        uint16_t kind = 0xffff;  // no segment
        if (g < L.n_segments) {
            const uint32_t f = upper_index32(L.seg_first, L.n_frames, g);
            const DvFrame &F = L.frames[f];
            const uint32_t local = g - L.seg_first[f];
            const uint32_t sequence = local / 27, slot = local % 27;
            kind = kDiagNone;
            for (int m = 0; m < 5; m++) {
                const uint32_t vn = slot * 5 + m;
                const uint32_t dif = sequence * 150 + 7 + (vn / 15) * 16 + vn % 15;
                if (kind == kDiagNone && L.flags[F.dif_first + dif]) kind = kDvDamagedId;
                S.dif_off[t * 5 + m] = dif * 80;
                S.qno[t * 5 + m] = F.in[(size_t)dif * 80 + 3] & 0x0f;
            }
            S.frame[t] = f;
            S.local[t] = local;
        }
        S.kind[t] = kind;
    }
    __syncthreads();
    // payload words (bytes 4..80 of each DIF block), big-endian
    for (uint32_t i = t; i < (uint32_t)kSegPerCta * 96; i += kSegThreads) {
        const uint32_t sg = i / 96, wi = i % 96;
        uint32_t v = 0;
        if (wi < 95 && S.kind[sg] == kDiagNone) {
            const uint32_t m = wi / 19;
            const uint8_t *src = L.frames[S.frame[sg]].in + S.dif_off[sg * 5 + m] + 4 + (wi % 19) * 4;
            v = ((uint32_t)src[0] << 24) | ((uint32_t)src[1] << 16) | ((uint32_t)src[2] << 8) | (uint32_t)src[3];
        }
        S.pay[sg][wi] = v;
    }
    for (uint32_t i = t; i < (uint32_t)kSegBlocks * 8; i += kSegThreads)
        reinterpret_cast<int4 *>(&S.coef[0][0])[i] = make_int4(0, 0, 0, 0);
    for (uint32_t i = t; i < (uint32_t)kSegPerCta * 5 * 20; i += kSegThreads) (&S.mbpool[0][0])[i] = 0;
    for (uint32_t i = t; i < (uint32_t)kSegPerCta * 97; i += kSegThreads) (&S.segpool[0][0])[i] = 0;
    __syncthreads();
    // 1. a thread per block: its own region
    if (t < (uint32_t)kSegBlocks) {
        const uint32_t sg = t / 30, b = t % 30, m = b / 6, bi = b % 6;
        DvBlock &B = S.blk[t];
        B.position = 0;
        B.complete = 0;
        B.mode = 0;
        B.cls = 0;
        B.pval = 0;
        B.plen = 0;
        B.pad = 0;
        uint16_t ls = 0, ll = 0;
        bool bad = false;
        if (S.kind[sg] == kDiagNone) {
            const uint32_t *w = S.pay[sg] + m * 19;
            const uint32_t r0 = bi < 4 ? bi * 112 : 448 + (bi - 4) * 80, bits = bi < 4 ? 112 : 80;
            const uint32_t head = get32(w, r0) >> 20;  // 12 bits: dc(9) mode(1) class(2)
            int32_t dc = (int32_t)(head >> 3);
            if (dc & 0x100) dc -= 512;
            B.mode = (head >> 2) & 1;
            B.cls = head & 3;
            S.coef[t][0] = (int16_t)(dc * 4 + 1024);
            uint32_t pos = r0 + 12;
            const uint32_t end = r0 + bits;
            consume_ac(B, w, pos, end, S.coef[t], S.qno[sg * 5 + m], L.vlc, bad);
            if (B.complete) {
                ls = (uint16_t)pos;
                ll = (uint16_t)(end - pos);
            }
        }
        S.left_start[t] = ls;
        S.left_len[t] = ll;
        S.bad[t] = bad ? 1 : 0;
    }
    __syncthreads();
    // 2. a thread per macroblock: its pool
    if (t < (uint32_t)kSegPerCta * 5) {
        const uint32_t sg = t / 5, m = t % 5;
        uint32_t pos = 0, mbn = 0;
        if (S.kind[sg] == kDiagNone) {
            const uint32_t *w = S.pay[sg] + m * 19;
            const uint32_t j0 = sg * 30 + m * 6;
            for (uint32_t j = j0; j < j0 + 6; j++)
                if (S.blk[j].complete) append_bits(S.mbpool[t], mbn, w, S.left_start[j], S.left_len[j]);
            bool bad = false;
            for (uint32_t j = j0; j < j0 + 6; j++)
                if (!S.blk[j].complete && pos < mbn)
                    consume_ac(S.blk[j], S.mbpool[t], pos, mbn, S.coef[j], S.qno[t], L.vlc, bad);
            if (bad) S.bad[j0] = 1;
        }
        S.mb_pos[t] = (uint16_t)pos;
        S.mb_len[t] = (uint16_t)mbn;
    }
    __syncthreads();
    // 3. a thread per segment: its pool, then its result
    if (t < (uint32_t)kSegPerCta && S.kind[t] == kDiagNone) {
        uint32_t segn = 0;
        for (uint32_t m = 0; m < 5; m++) {
            const uint32_t k = t * 5 + m;
            if (S.mb_pos[k] < S.mb_len[k])
                append_bits(S.segpool[t], segn, S.mbpool[k], S.mb_pos[k], S.mb_len[k] - S.mb_pos[k]);
        }
        uint32_t pos = 0;
        bool bad = false;
        for (uint32_t j = 0; j < 30; j++) {
            const uint32_t jj = t * 30 + j;
            if (!S.blk[jj].complete && pos < segn)
                consume_ac(S.blk[jj], S.segpool[t], pos, segn, S.coef[jj], S.qno[t * 5 + j / 6], L.vlc, bad);
        }
        for (uint32_t j = 0; j < 30; j++) bad |= S.bad[t * 30 + j] != 0;
        uint16_t kind = kDiagNone;
        if (bad) kind = kDvBadVlc;
        else
            for (uint32_t j = 0; j < 30; j++)
                if (!S.blk[t * 30 + j].complete) {
                    kind = kDvIncomplete;
                    break;
                }
        S.kind[t] = kind;
    }
    __syncthreads();
    // coefficients out (the CTA's segments are consecutive: blocks g0 * 30 ..), modes, results
    const uint32_t n_seg = min((uint32_t)kSegPerCta, L.n_segments - g0);
    int4 *dst = reinterpret_cast<int4 *>(L.coef + (uint64_t)g0 * 30 * 64);
    const int4 *src = reinterpret_cast<const int4 *>(&S.coef[0][0]);
    for (uint32_t i = t; i < n_seg * 30 * 8; i += kSegThreads) dst[i] = src[i];
    if (t < n_seg * 30) L.modes[(uint64_t)g0 * 30 + t] = S.blk[t].mode;
    if (t < n_seg) {
        const uint16_t kind = S.kind[t];
        L.seg_err[g0 + t] = (uint8_t)kind;
        if (kind != kDiagNone) {
            atomicMin(&L.states[S.frame[t]].bad_segment, S.local[t]);
            atomicAdd(&L.states[S.frame[t]].failed, 1u);
        }
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

// decoder.rs:395-422 macroblock_coordinates (in 8-sample units); the per-macroblock
// offsets in constant memory (indexed per lane, as local arrays they went to the stack)
__constant__ uint32_t c_mb_off[5] = {2, 6, 8, 0, 4};
__constant__ uint32_t c_mb_shuf3[5] = {18, 9, 27, 0, 36};
__constant__ uint32_t c_mb_lstart[5] = {9, 4, 13, 0, 18};

__device__ __forceinline__ void mb_coords(bool pal, uint32_t seqs, uint32_t sequence, uint32_t slot, uint32_t m,
                                          uint32_t *mbx, uint32_t *mby) {
    if (pal) {
        // SERPENT1[slot] = 0,1,2,2,1,0 repeating
        uint32_t s6 = slot % 6;
        uint32_t serp1 = s6 < 3 ? s6 : 5 - s6;
        uint32_t x = c_mb_shuf3[m] + slot / 3;
        uint32_t y = serp1 + ((sequence + c_mb_off[m]) % seqs) * 3;
        *mbx = x * 2;
        *mby = y * 2;
    } else {
        uint32_t row = (sequence + c_mb_off[m]) % seqs;
        uint32_t k = slot + ((m == 1 || m == 2) ? 3 : 0);
        uint32_t x = c_mb_lstart[m] + k / 6;
        // SERPENT2[k] = 0..5,5..0 repeating
        uint32_t k12 = k % 12;
        uint32_t serp2 = k12 < 6 ? k12 : 11 - k12;
        uint32_t y = serp2 + row * 6;
        if (x > 21) y = y * 2 - row * 6;
        *mbx = x * 4;
        *mby = y;
    }
}

constexpr int kIdctBlocks = 16;                  // blocks per CTA
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
    if (L.n_segments) segment_kernel<<<(L.n_segments + kSegPerCta - 1) / kSegPerCta, kSegThreads, 0, s>>>(L);
    if (L.n_frames) dv_resolve_kernel<<<(L.n_frames + 127) / 128, 128, 0, s>>>(L);
}

void launch_dv_idct(const DvLaunch &L, cudaStream_t s) {
    if (L.n_blocks == 0) return;
    const uint64_t grid = (L.n_blocks + kIdctBlocks - 1) / kIdctBlocks;
    dv_idct_kernel<<<(unsigned)grid, kIdctThreads, 0, s>>>(L);
}

}  // namespace mmr
