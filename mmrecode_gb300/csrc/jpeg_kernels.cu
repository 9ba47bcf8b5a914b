// MJPEG decode kernels for sm_103a.
//
//   scan_count / scan_prefix / scan_emit  marker scan of the entropy-coded data
//       (crates/codecs/mjpeg/src/parser.rs:373-414 and the byte-unstuffing of
//       entropy.rs:143-165), parallel over 4 KiB tiles: finds the terminating
//       marker, lists RSTn markers in order and writes the unstuffed bytes.
//   entropy  one restart interval per thread (decoder.rs:313-410, 495-548):
//       Huffman decode, DC prediction, run/level expansion; writes quantised AC
//       levels (natural order) and the dequantised DC of every block, and the
//       interval's restart-marker check (entropy.rs:111-134).
//   resolve  picks each frame's first failing interval (sequential semantics).
//   idct     dequantisation + the reference's binary64 IDCT (transform.rs:86-109)
//       in its exact operation order, +128, round-half-away, clamp, clipped
//       block write (decoder.rs:550-565).
#include <cuda_runtime.h>

#include "kernels.h"
#include "tables.h"

namespace mmr {

__constant__ int c_zigzag[64] = MMR_ZIGZAG_INIT;
__constant__ double c_idct[64] = MMR_IDCT_MATRIX_INIT;

namespace {

constexpr int kScanThreads = kScanTile / 16;  // 16 bytes per thread
constexpr int kEntropyThreads = 128;
constexpr int kStageStride = 72;              // int16 per staged block (144 B: conflict-free 16 B rows)

// Largest f with first[f] <= x (first has n + 1 ascending entries, first[0] = 0).
template <typename T>
__device__ __forceinline__ uint32_t upper_index(const T *first, uint32_t n, T x) {
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (first[mid] <= x) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Byte classes of the entropy-coded region.
enum : int { kByteNone = 0, kBytePlain = 1, kByteStuffed = 2, kByteRst = 3, kByteTerm = 4, kByteTrunc = 5 };

// Classifies position p given its byte and whether the previous scan byte was 0xFF.
// A maximal run of 0xFF starts a marker sequence whose code is the next non-FF byte
// (parser.rs:385-391): 0x00 = stuffed data byte, D0-D7 = RSTn, anything else ends
// the scan; a run reaching the end of the packet is a truncated marker.
__device__ __forceinline__ int classify(const uint8_t *in, uint32_t len, uint32_t p, uint8_t b, bool prev_ff,
                                        uint32_t *code) {
    if (b != 0xff) return prev_ff ? kByteNone : kBytePlain;
    if (prev_ff) return kByteNone;
    uint32_t q = p + 1;
    while (q < len && in[q] == 0xff) q++;
    if (q >= len) return kByteTrunc;
    uint32_t c = in[q];
    *code = c;
    if (c == 0x00) return kByteStuffed;
    if (c >= 0xd0 && c <= 0xd7) return kByteRst;
    return kByteTerm;
}

template <typename T>
__device__ __forceinline__ T warp_incl_scan(T v) {
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T n = __shfl_up_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) >= (unsigned)o) v += n;
    }
    return v;
}

// Block-wide exclusive scan of two counters; returns the block totals.
template <int NT>
__device__ __forceinline__ void block_excl_scan2(uint32_t a, uint32_t b, uint32_t &ea, uint32_t &eb, uint32_t &ta,
                                                 uint32_t &tb) {
    __shared__ uint32_t wa[NT / 32], wb[NT / 32];
    uint32_t ia = warp_incl_scan(a), ib = warp_incl_scan(b);
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 31) {
        wa[w] = ia;
        wb[w] = ib;
    }
    __syncthreads();
    if (w == 0) {
        uint32_t va = lane < NT / 32 ? wa[lane] : 0, vb = lane < NT / 32 ? wb[lane] : 0;
        va = warp_incl_scan(va);
        vb = warp_incl_scan(vb);
        if (lane < NT / 32) {
            wa[lane] = va;
            wb[lane] = vb;
        }
    }
    __syncthreads();
    uint32_t oa = w ? wa[w - 1] : 0, ob = w ? wb[w - 1] : 0;
    ea = oa + ia - a;
    eb = ob + ib - b;
    ta = wa[NT / 32 - 1];
    tb = wb[NT / 32 - 1];
    __syncthreads();
}

struct TileRef {
    uint32_t frame;
    uint32_t base;  // packet-relative first byte of this tile (16-aligned below data_start)
};

__device__ __forceinline__ TileRef tile_ref(const JpegLaunch &L, uint32_t t) {
    TileRef r;
    r.frame = upper_index(L.tile_first, L.n_frames, t);
    const JFrame &F = L.frames[r.frame];
    r.base = (F.data_start & ~15u) + (t - L.tile_first[r.frame]) * (uint32_t)kScanTile;
    return r;
}

__global__ void __launch_bounds__(kScanThreads) scan_count_kernel(JpegLaunch L) {
    uint32_t t = blockIdx.x;
    TileRef tr = tile_ref(L, t);
    const JFrame &F = L.frames[tr.frame];
    const uint8_t *in = F.in;
    uint32_t len = F.in_len, ds = F.data_start;
    uint32_t p0 = tr.base + threadIdx.x * 16;
    uint32_t tokens = 0, rsts = 0;
    unsigned long long term = ~0ull;
    if (p0 < len) {
        bool prev_ff = p0 > ds && in[p0 - 1] == 0xff;
#pragma unroll 4
        for (int k = 0; k < 16; k++) {
            uint32_t p = p0 + k;
            if (p >= len) break;
            if (p < ds) continue;
            uint8_t b = in[p];
            uint32_t code = 0;
            int kind = classify(in, len, p, b, prev_ff, &code);
            tokens += (kind == kBytePlain || kind == kByteStuffed);
            rsts += kind == kByteRst;
            if (kind == kByteTerm) term = min(term, ((unsigned long long)p << 9) | code);
            if (kind == kByteTrunc) term = min(term, ((unsigned long long)p << 9) | 256ull);
            prev_ff = b == 0xff;
        }
    }
    // reduce
    __shared__ uint32_t s_tok[kScanThreads / 32], s_rst[kScanThreads / 32];
    __shared__ unsigned long long s_term[kScanThreads / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        tokens += __shfl_down_sync(0xffffffffu, tokens, o);
        rsts += __shfl_down_sync(0xffffffffu, rsts, o);
        term = min(term, __shfl_down_sync(0xffffffffu, term, o));
    }
    if ((threadIdx.x & 31) == 0) {
        s_tok[threadIdx.x >> 5] = tokens;
        s_rst[threadIdx.x >> 5] = rsts;
        s_term[threadIdx.x >> 5] = term;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t a = 0, b = 0;
        unsigned long long m = ~0ull;
        for (int w = 0; w < kScanThreads / 32; w++) {
            a += s_tok[w];
            b += s_rst[w];
            m = min(m, s_term[w]);
        }
        L.tile_tok[t] = a;
        L.tile_rst[t] = b;
        if (m != ~0ull) atomicMin(&L.states[tr.frame].term, m);
    }
}

// Per frame: exclusive prefix of tile token / RST counts.
__global__ void __launch_bounds__(256) scan_prefix_kernel(JpegLaunch L) {
    uint32_t f = blockIdx.x;
    uint32_t t0 = L.tile_first[f], t1 = L.tile_first[f + 1];
    uint32_t carry_a = 0, carry_b = 0;
    for (uint32_t base = t0; base < t1; base += 256) {
        uint32_t t = base + threadIdx.x;
        uint32_t a = t < t1 ? L.tile_tok[t] : 0, b = t < t1 ? L.tile_rst[t] : 0;
        uint32_t ea, eb, ta, tb;
        block_excl_scan2<256>(a, b, ea, eb, ta, tb);
        if (t < t1) {
            L.tile_tok[t] = carry_a + ea;
            L.tile_rst[t] = carry_b + eb;
        }
        carry_a += ta;
        carry_b += tb;
    }
}

__global__ void __launch_bounds__(kScanThreads) scan_emit_kernel(JpegLaunch L) {
    uint32_t t = blockIdx.x;
    TileRef tr = tile_ref(L, t);
    const JFrame &F = L.frames[tr.frame];
    unsigned long long termv = L.states[tr.frame].term;
    if (termv == ~0ull || ((termv >> 8) & 1)) return;  // parse error: no usable scan end
    uint32_t term = (uint32_t)(termv >> 9);
    if (tr.base >= term) return;
    const uint8_t *in = F.in;
    uint32_t len = F.in_len, ds = F.data_start;
    uint32_t p0 = tr.base + threadIdx.x * 16;
    uint8_t kinds[16], bytes[16];
    uint32_t tokens = 0, rsts = 0;
    bool prev_ff = p0 > ds && p0 < len && in[p0 - 1] == 0xff;
#pragma unroll
    for (int k = 0; k < 16; k++) {
        uint32_t p = p0 + k;
        kinds[k] = kByteNone;
        bytes[k] = 0;
        if (p < ds || p >= term) continue;
        uint8_t b = in[p];
        uint32_t code = 0;
        int kind = classify(in, len, p, b, prev_ff, &code);
        kinds[k] = (uint8_t)kind;
        bytes[k] = kind == kByteRst ? (uint8_t)(code - 0xd0) : b;
        tokens += (kind == kBytePlain || kind == kByteStuffed);
        rsts += kind == kByteRst;
        prev_ff = b == 0xff;
    }
    uint32_t etok, erst, ttok, trst;
    block_excl_scan2<kScanThreads>(tokens, rsts, etok, erst, ttok, trst);
    uint32_t tok_pos = L.tile_tok[t] + etok;
    uint32_t rst_idx = L.tile_rst[t] + erst;
    RstEntry *rst = L.rsts + F.rst_off;
#pragma unroll
    for (int k = 0; k < 16; k++) {
        int kind = kinds[k];
        if (kind == kBytePlain) F.tok[tok_pos++] = bytes[k];
        else if (kind == kByteStuffed) F.tok[tok_pos++] = 0xff;
        else if (kind == kByteRst) {
            if (rst_idx < F.n_intervals) {
                RstEntry e;
                e.tok = tok_pos;
                e.number = bytes[k];
                rst[rst_idx] = e;
            }
            rst_idx++;
        }
    }
    // The last tile that starts before the terminator publishes the totals (the
    // terminator may sit exactly on the next tile's first byte).
    if (threadIdx.x == 0 && term <= tr.base + (uint32_t)kScanTile) {
        L.states[tr.frame].n_tokens = L.tile_tok[t] + ttok;
        L.states[tr.frame].n_rst = L.tile_rst[t] + trst;
    }
}

// ------------------------------------------------------------ entropy -----

struct BitStream {
    const uint8_t *tok;
    uint32_t pos;   // next token to load
    uint32_t end;   // barrier: first token this interval may not read
    uint64_t buf;   // next bits, MSB first
    int nbits;      // valid bits in buf
    uint32_t used;  // bits consumed in this interval
};

__device__ __forceinline__ void fill(BitStream &s) {
    while (s.nbits <= 56 && s.pos < s.end) {
        s.buf |= (uint64_t)s.tok[s.pos] << (56 - s.nbits);
        s.pos++;
        s.nbits += 8;
    }
}

__device__ __forceinline__ void consume(BitStream &s, int n) {
    s.buf <<= n;
    s.nbits -= n;
    s.used += n;
}

// Next Huffman symbol (entropy.rs:57-70). Returns the code length, 0 if no code
// of length <= 16 matches the (zero-padded) next bits.
__device__ __forceinline__ int huff_peek(const HuffLut *__restrict__ lut, const uint8_t *__restrict__ symbols,
                                         const BitStream &s, uint32_t *sym) {
    uint32_t e = lut->fast[s.buf >> 55];
    if (e) {
        *sym = e & 0xff;
        return (int)(e >> 8);
    }
    uint32_t code16 = (uint32_t)(s.buf >> 48);
#pragma unroll 1
    for (int l = 10; l <= 16; l++) {
        int32_t c = (int32_t)(code16 >> (16 - l));
        if (c <= lut->maxcode[l]) {
            *sym = symbols[lut->sym_off + lut->valptr[l] + c];
            return l;
        }
    }
    return 0;
}

struct EntropyError {
    uint16_t kind;
    uint32_t bitpos;  // reader position in bits from the interval start
    uint32_t aux, aux2;
};

template <int MAXC>
__device__ void decode_interval(const JpegLaunch &L, uint32_t item, int16_t *stage) {
    uint2 it = L.items[item];
    uint32_t f = it.x, iv = it.y;
    const JFrame &F = L.frames[f];
    JState *st = &L.states[f];
    Diag out = make_diag(kDiagNone);
    unsigned long long termv = st->term;
    if (!F.decode || termv == ~0ull || ((termv >> 8) & 1)) return;
    uint32_t n_rst = min(st->n_rst, F.n_intervals);
    uint32_t n_tok = st->n_tokens;
    const RstEntry *rst = L.rsts + F.rst_off;
    uint32_t start;
    if (iv == 0) start = 0;
    else if (iv - 1 < n_rst) start = rst[iv - 1].tok;
    else return;  // no RST precedes this interval: an earlier interval fails its restart check
    bool barrier_rst = iv < n_rst;
    uint32_t barrier = barrier_rst ? rst[iv].tok : n_tok;

    BitStream s;
    s.tok = F.tok;
    s.pos = start;
    s.end = barrier;
    s.buf = 0;
    s.nbits = 0;
    s.used = 0;
    int32_t pred[MAXC];
    for (int c = 0; c < MAXC; c++) pred[c] = 0;

    EntropyError err;
    err.kind = kDiagNone;
    uint32_t mcu0 = iv * F.ri;
    uint32_t mcu1 = min(mcu0 + F.ri, F.total_mcus);
    const JSched *sched = L.sched + F.sched_off;
    const JComp *comps = L.comps + F.comp_off;
    int4 *stage4 = reinterpret_cast<int4 *>(stage);

    for (uint32_t mcu = mcu0; mcu < mcu1 && err.kind == kDiagNone; mcu++) {
        uint32_t mx = mcu % F.mcu_cols, my = mcu / F.mcu_cols;
        for (uint32_t si = 0; si < F.sched_len; si++) {
            JSched e = sched[si];
            const JComp &C = comps[e.comp];
            const HuffLut *dct = L.luts + F.lut[e.dc];
            const HuffLut *act = L.luts + F.lut[4 + e.ac];
            const uint16_t *Q = L.quant + F.quant_off + C.q * 64;
#pragma unroll
            for (int k = 0; k < 8; k++) stage4[k] = make_int4(0, 0, 0, 0);
            // DC (decoder.rs:501-515)
            fill(s);
            uint32_t sym;
            int len = huff_peek(dct, L.symbols, s, &sym);
            if (len == 0 || len > s.nbits) {
                err.kind = (len == 0 && s.nbits >= 16) ? kJNoHuffCode : (barrier_rst ? kJMarkerInData : kJEndOfData);
                err.bitpos = s.used + 16;
                break;
            }
            consume(s, len);
            if (sym > 11) {
                err.kind = kJDcCategory;
                err.bitpos = s.used;
                break;
            }
            int32_t diff = 0;
            if (sym) {
                if (s.nbits < (int)sym) {
                    err.kind = barrier_rst ? kJMarkerInData : kJEndOfData;
                    break;
                }
                int32_t v = (int32_t)(s.buf >> (64 - sym));
                consume(s, sym);
                diff = v < (1 << (sym - 1)) ? v + 1 - (1 << sym) : v;
            }
            int64_t p = (int64_t)pred[e.comp] + diff;
            if (p > INT32_MAX || p < INT32_MIN) {
                err.kind = kJDcPredOverflow;
                err.bitpos = s.used;
                break;
            }
            pred[e.comp] = (int32_t)p;
            int64_t dq = p * (int64_t)Q[0];
            if (dq > INT32_MAX || dq < INT32_MIN) {
                err.kind = kJDcDeqOverflow;
                err.bitpos = s.used;
                break;
            }
            // AC (decoder.rs:517-546)
            int k = 1;
            while (k < 64) {
                fill(s);
                len = huff_peek(act, L.symbols, s, &sym);
                if (len == 0 || len > s.nbits) {
                    err.kind = (len == 0 && s.nbits >= 16) ? kJNoHuffCode : (barrier_rst ? kJMarkerInData : kJEndOfData);
                    err.bitpos = s.used + 16;
                    break;
                }
                consume(s, len);
                int run = sym >> 4, size = sym & 15;
                if (size == 0) {
                    if (run == 0) break;
                    if (run != 15) {
                        err.kind = kJAcZeroSize;
                        err.bitpos = s.used;
                        break;
                    }
                    k += 16;
                    if (k > 64) {
                        err.kind = kJZrlOverrun;
                        err.bitpos = s.used;
                        break;
                    }
                    continue;
                }
                if (size > 10) {
                    err.kind = kJAcCategory;
                    err.bitpos = s.used;
                    break;
                }
                k += run;
                if (k >= 64) {
                    err.kind = kJAcRun;
                    err.bitpos = s.used;
                    break;
                }
                if (s.nbits < size) {
                    err.kind = barrier_rst ? kJMarkerInData : kJEndOfData;
                    break;
                }
                int32_t v = (int32_t)(s.buf >> (64 - size));
                consume(s, size);
                v = v < (1 << (size - 1)) ? v + 1 - (1 << size) : v;
                stage[c_zigzag[k]] = (int16_t)v;
                k++;
            }
            if (err.kind != kDiagNone) break;
            // block write (levels + dequantised DC)
            uint32_t gx, gy;
            if (F.interleaved) {
                gx = mx * C.h + e.bx;
                gy = my * C.v + e.by;
            } else {
                gx = mx;
                gy = my;
            }
            uint64_t blk = F.blk_off + C.blk_base + (uint64_t)gy * C.bw + gx;
            int4 *dst = reinterpret_cast<int4 *>(L.coef + blk * 64);
#pragma unroll
            for (int q = 0; q < 8; q++) dst[q] = stage4[q];
            L.dc[blk] = (int32_t)dq;
        }
    }

    if (err.kind != kDiagNone) {
        uint32_t offset;
        if (err.kind == kJMarkerInData) {
            offset = barrier;
            out = make_diag(kJMarkerInData, offset, 0xd0 + rst[iv].number);
        } else if (err.kind == kJEndOfData) {
            out = make_diag(kJEndOfData, n_tok);
        } else {
            offset = start + (err.bitpos + 7) / 8;
            out = make_diag(err.kind, offset);
        }
    } else if (iv + 1 < F.n_intervals) {
        // consume_restart before the next interval (entropy.rs:111-134)
        uint32_t tend = start + (s.used + 7) / 8;
        uint32_t expected = iv & 7;
        if (barrier_rst && rst[iv].tok == tend) {
            if (rst[iv].number != expected) out = make_diag(kJRstMismatch, tend, expected, 0xd0 + rst[iv].number);
        } else if (tend < n_tok && F.tok[tend] == 0xff) {
            out = make_diag(kJRstMismatch, tend, expected, 0x00);
        } else {
            out = make_diag(kJExpectRst, tend);
        }
    }
    L.results[item] = out;
    if (out.kind != kDiagNone) atomicMin(&st->bad_interval, iv);
}

template <int MAXC>
__global__ void __launch_bounds__(kEntropyThreads) entropy_kernel(JpegLaunch L, uint32_t first, uint32_t count) {
    __shared__ __align__(16) int16_t s_stage[kEntropyThreads * kStageStride];
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    decode_interval<MAXC>(L, first + i, s_stage + threadIdx.x * kStageStride);
}

__global__ void resolve_kernel(JpegLaunch L) {
    uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= L.n_frames) return;
    const JFrame &F = L.frames[f];
    JState *st = &L.states[f];
    unsigned long long termv = st->term;
    bool ok = F.decode && termv != ~0ull && !((termv >> 8) & 1);
    if (st->bad_interval != 0xffffffffu) {
        st->diag = L.results[F.item_base + st->bad_interval];
        ok = false;
    }
    if (!ok) L.item_ok[F.item] = 0;
}

// ---------------------------------------------------------------- IDCT ----
//
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
//   fp32 path (M and c rounded to fp32, FMA accumulation, u = 2^-24):
//        |s32 - S| <= (2u + 8u) + (u + 8u) ... = 19u * B + O(u^2) B   (pass 1 error
//        10u A with A = sum_u |M||c|, propagated through pass 2, plus pass 2's
//        own 8u; standard recursive-summation bounds, Higham ch. 3)
//   binary64 reference: |s64 - S| <= 16 * 2^-53 * B, and its +128.0 rounds
//        by at most 2^-53 |s + 128|.
// With delta = 2^-21 * C1 + 2^-40 |s32| + 2^-30 (2^-21 * C1 >= 19u * 0.2405 C1
// with 1.7x margin), if no half-integer lies within delta of s32 + 128 both
// values round to the same integer; samples certain to clamp are kept too.
// Every other sample is queued and recomputed in the exact reference order by
// fixup_kernel (or in place when the queue is full). Zero coefficients are
// skipped in the exact path: a zero term adds +-0.0, which leaves any sum that
// is not -0.0 unchanged, and these sums are never -0.0.

__constant__ float c_idct32[64] = MMR_IDCT_MATRIX_INIT;

__device__ __forceinline__ uint8_t exact_sample(const int32_t *c, int stride, int y, int x) {
    double t[8];
#pragma unroll
    for (int v = 0; v < 8; v++) {
        double acc = 0.0;
#pragma unroll
        for (int u = 0; u < 8; u++) {
            int32_t cv = c[v * stride + u];
            if (cv) acc = __dadd_rn(acc, __dmul_rn(c_idct[x * 8 + u], (double)cv));
        }
        t[v] = acc;
    }
    double acc = 0.0;
#pragma unroll
    for (int v = 0; v < 8; v++)
        if (t[v] != 0.0) acc = __dadd_rn(acc, __dmul_rn(c_idct[y * 8 + v], t[v]));
    double px = round(__dadd_rn(acc, 128.0));
    return (uint8_t)fmin(fmax(px, 0.0), 255.0);
}

constexpr int kIdctBlocks = 32;  // blocks per CTA, 8 threads (one column each) per block

__device__ __forceinline__ uint32_t find_range(const JpegLaunch &L, uint64_t g) {
    uint32_t lo = 0, hi = L.n_ranges;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (L.ranges[mid].first <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(kIdctBlocks * 8) idct_kernel(JpegLaunch L) {
    __shared__ int32_t s_c[kIdctBlocks][65];
    __shared__ float s_f[kIdctBlocks][65];
    int lb = threadIdx.x >> 3, x = threadIdx.x & 7;
    uint64_t g = (uint64_t)blockIdx.x * kIdctBlocks + lb;
    bool valid = g < L.n_blocks;
    uint32_t r = 0;
    const JFrame *F = nullptr;
    const JComp *C = nullptr;
    if (valid) {
        r = find_range(L, g);
        F = &L.frames[L.ranges[r].frame];
        C = &L.comps[F->comp_off + L.ranges[r].comp];
        valid = L.item_ok[F->item] != 0;
    }
    uint64_t l1 = 0;  // sum |c| over this thread's row
    if (valid) {
        const uint16_t *Q = L.quant + F->quant_off + C->q * 64;
        int4 v = reinterpret_cast<const int4 *>(L.coef + g * 64)[x];
        const int16_t *lv = reinterpret_cast<const int16_t *>(&v);
#pragma unroll
        for (int j = 0; j < 8; j++) {
            int32_t c = (j == 0 && x == 0) ? L.dc[g] : (int32_t)lv[j] * (int32_t)Q[x * 8 + j];
            s_c[lb][x * 8 + j] = c;
            s_f[lb][x * 8 + j] = (float)c;
            l1 += (uint64_t)(c < 0 ? -(int64_t)c : (int64_t)c);
        }
    }
    // C1 over the block's 8 threads (lanes 8k..8k+7 of the warp)
#pragma unroll
    for (int o = 1; o < 8; o <<= 1) l1 += __shfl_xor_sync(0xffffffffu, l1, o);
    __syncthreads();
    if (!valid) return;
    float mrow[8];
#pragma unroll
    for (int u = 0; u < 8; u++) mrow[u] = c_idct32[x * 8 + u];
    float t[8];
#pragma unroll
    for (int v = 0; v < 8; v++) {
        float acc = 0.0f;
#pragma unroll
        for (int u = 0; u < 8; u++) acc = fmaf(mrow[u], s_f[lb][v * 8 + u], acc);
        t[v] = acc;
    }
    const float delta_base = (float)l1 * 0x1p-21f + 0x1p-30f;
    uint64_t local = g - L.ranges[r].first;
    uint32_t gx = (uint32_t)(local % C->bw), gy = (uint32_t)(local / C->bw);
    uint32_t col = gx * 8 + x;
    uint8_t *plane = F->planes + C->out_off;
#pragma unroll
    for (int y = 0; y < 8; y++) {
        float acc = 0.0f;
#pragma unroll
        for (int v = 0; v < 8; v++) acc = fmaf(c_idct32[y * 8 + v], t[v], acc);
        uint32_t row = gy * 8 + y;
        if (row >= C->plane_h || col >= C->plane_w) continue;
        float delta = delta_base + fabsf(acc) * 0x1p-40f;
        int out;
        bool certain = true;
        if (acc + delta < 0.5f - 128.0f) out = 0;
        else if (acc - delta > 254.5f - 128.0f) out = 255;
        else {
            float fl = floorf(acc);
            float fr = acc - fl;  // exact for |acc| < 2^23
            certain = fabsf(fr - 0.5f) > delta && delta < 0.25f;
            int rr = (int)fl + (fr > 0.5f ? 1 : 0) + 128;
            out = rr < 0 ? 0 : rr > 255 ? 255 : rr;
        }
        uint64_t dst = (uint64_t)row * C->plane_w + col;
        if (certain) {
            plane[dst] = (uint8_t)out;
            continue;
        }
        uint32_t slot = atomicAdd(L.fix_count, 1u);
        if (slot < L.fix_capacity) L.fix[slot] = (g << 6) | (uint64_t)(y * 8 + x);
        else plane[dst] = exact_sample(&s_c[lb][0], 8, y, x);  // queue full: exact in place
    }
}

// Exact reference-order recomputation of the queued samples.
__global__ void __launch_bounds__(256) idct_fixup_kernel(JpegLaunch L) {
    uint32_t n = min(*L.fix_count, L.fix_capacity);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        unsigned long long e = L.fix[i];
        uint64_t g = e >> 6;
        int y = (int)(e >> 3) & 7, x = (int)e & 7;
        uint32_t r = find_range(L, g);
        const JFrame *F = &L.frames[L.ranges[r].frame];
        const JComp *C = &L.comps[F->comp_off + L.ranges[r].comp];
        const uint16_t *Q = L.quant + F->quant_off + C->q * 64;
        int32_t c[64];
        const int4 *src = reinterpret_cast<const int4 *>(L.coef + g * 64);
#pragma unroll
        for (int k = 0; k < 8; k++) {
            int4 v = src[k];
            const int16_t *lv = reinterpret_cast<const int16_t *>(&v);
#pragma unroll
            for (int j = 0; j < 8; j++) c[k * 8 + j] = (int32_t)lv[j] * (int32_t)Q[k * 8 + j];
        }
        c[0] = L.dc[g];
        uint64_t local = g - L.ranges[r].first;
        uint32_t gx = (uint32_t)(local % C->bw), gy = (uint32_t)(local / C->bw);
        F->planes[C->out_off + (uint64_t)(gy * 8 + y) * C->plane_w + gx * 8 + x] = exact_sample(c, 8, y, x);
    }
}

}  // namespace

void launch_jpeg_scan(const JpegLaunch &L, cudaStream_t s) {
    if (L.n_tiles == 0) return;
    scan_count_kernel<<<L.n_tiles, kScanThreads, 0, s>>>(L);
    scan_prefix_kernel<<<L.n_frames, 256, 0, s>>>(L);
    scan_emit_kernel<<<L.n_tiles, kScanThreads, 0, s>>>(L);
}

void launch_jpeg_entropy(const JpegLaunch &L, cudaStream_t s) {
    if (L.n_items_small)
        entropy_kernel<4><<<(L.n_items_small + kEntropyThreads - 1) / kEntropyThreads, kEntropyThreads, 0, s>>>(
            L, 0, L.n_items_small);
    uint32_t big = L.n_items - L.n_items_small;
    if (big)
        entropy_kernel<256><<<(big + kEntropyThreads - 1) / kEntropyThreads, kEntropyThreads, 0, s>>>(
            L, L.n_items_small, big);
    if (L.n_frames) resolve_kernel<<<(L.n_frames + 127) / 128, 128, 0, s>>>(L);
}

void launch_jpeg_idct(const JpegLaunch &L, cudaStream_t s) {
    if (L.n_blocks == 0) return;
    uint64_t grid = (L.n_blocks + kIdctBlocks - 1) / kIdctBlocks;
    idct_kernel<<<(unsigned)grid, kIdctBlocks * 8, 0, s>>>(L);
    idct_fixup_kernel<<<L.fixup_grid, 256, 0, s>>>(L);
}

}  // namespace mmr
