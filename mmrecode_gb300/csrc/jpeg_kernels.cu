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
//   idct     planar output: dequantisation + the IDCT in fp32 with a proven error
//       bound (idct_core.h), +128, round-half-away, clamp, clipped block write
//       (decoder.rs:550-565); idct_fixup settles the samples the bound leaves
//       undecided, a warp per block, in exact fixed point or the reference's
//       binary64 order (transform.rs:86-109).
#include <cuda_runtime.h>

#include "entropy_core.h"
#include "idct_core.h"
#include "kernels.h"
#include "tables.h"

namespace mmr {

__constant__ int c_zigzag[64] = MMR_ZIGZAG_INIT;

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

// True when the 16 bytes at p (p >= data_start, p + 16 <= len) hold no 0xFF and the
// byte before them is not 0xFF: then all 16 are plain data bytes. Loads the bytes
// into *v (one 16-byte load when the packet is 16-byte aligned).
__device__ __forceinline__ bool plain_chunk(const uint8_t *in, uint32_t ds, uint32_t p, uint4 *v) {
    if ((((uintptr_t)in) & 15) != 0) return false;
    *v = *reinterpret_cast<const uint4 *>(in + p);
    const uint32_t w[4] = {v->x, v->y, v->z, v->w};
    bool ff = p > ds && in[p - 1] == 0xff;
#pragma unroll
    for (int i = 0; i < 4; i++) ff |= any_ff(w[i]) != 0;
    return !ff;
}

// Bytes of a 16-byte chunk equal to b: bit i set when byte i (in address order) is b.
__device__ __forceinline__ uint32_t byte_mask(const uint4 &v, uint32_t b) {
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
    uint32_t m = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const uint32_t e = zero_bytes(w[i] ^ (b * 0x01010101u));  // 0x80 per equal byte
        m |= ((e >> 7) & 1u | (e >> 14) & 2u | (e >> 21) & 4u | (e >> 28) & 8u) << (4 * i);
    }
    return m;
}

// A chunk whose 0xFF bytes are all stuffed data bytes: each followed by 0x00 (the
// next chunk's first byte for the last one), none next to another 0xFF, and the
// byte before the chunk, when 0xFF, followed by 0x00 here. Then every byte is a
// token except the stuffing zeros (parser.rs:385-391): returns true with their
// positions clear in *keep. Chunks with a marker or fill bytes return false.
// (p >= data_start; p + 16 <= end of the scanned range.)
__device__ __forceinline__ bool stuffed_chunk(const uint8_t *in, uint32_t len, uint32_t ds, uint32_t p, const uint4 &v,
                                              uint32_t *keep) {
    const uint32_t ff = byte_mask(v, 0xff), zero = byte_mask(v, 0x00);
    const uint32_t prev = p > ds && in[p - 1] == 0xff ? 1u : 0u;
    if ((ff & (ff >> 1)) || (prev & ff)) return false;                     // 0xFF next to 0xFF
    const uint32_t drop = ((ff << 1) | prev) & 0xffffu;                    // bytes after a 0xFF
    if (drop & ~zero) return false;                                        // a marker code
    if (ff & 0x8000u && (p + 16 >= len || in[p + 16] != 0x00)) return false;
    *keep = ~drop & 0xffffu;
    return true;
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
    uint4 v;
    uint32_t keep;
    const bool in_range = p0 >= ds && p0 + 16 <= len;
    if (in_range && plain_chunk(in, ds, p0, &v)) {
        tokens = 16;
    } else if (in_range && (((uintptr_t)in) & 15) == 0 && stuffed_chunk(in, len, ds, p0, v, &keep)) {
        tokens = __popc(keep);
    } else if (p0 < len) {
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
    // tokens of this tile, staged at their destination's offset within a 16-byte line
    __shared__ __align__(16) uint8_t s_tok[kScanTile + 32];
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
    uint4 v;
    uint32_t keep = 0xffffu;  // tokens of a plain or stuffed chunk
    const bool in_range = p0 >= ds && p0 + 16 <= term;
    bool plain = in_range && plain_chunk(in, ds, p0, &v);
    const bool stuffed = !plain && in_range && (((uintptr_t)in) & 15) == 0 && stuffed_chunk(in, len, ds, p0, v, &keep);
    plain |= stuffed;
    if (plain) {
        tokens = __popc(keep);
    } else {
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
    }
    uint32_t etok, erst, ttok, trst;
    block_excl_scan2<kScanThreads>(tokens, rsts, etok, erst, ttok, trst);
    const uint32_t tile_tok = L.tile_tok[t];
    const uint32_t mis = (uint32_t)((uintptr_t)(F.tok + tile_tok) & 15);
    uint8_t *st = s_tok + mis + etok;
    if (plain) {
        const uint32_t w[4] = {v.x, v.y, v.z, v.w};
        uint32_t n = 0;
#pragma unroll
        for (int i = 0; i < 16; i++) {
            if (keep & (1u << i)) st[n++] = (uint8_t)(w[i >> 2] >> (8 * (i & 3)));
        }
    } else {
        uint32_t tok_pos = tile_tok + etok, n = 0;
        uint32_t rst_idx = L.tile_rst[t] + erst;
        RstEntry *rst = L.rsts + F.rst_off;
#pragma unroll
        for (int k = 0; k < 16; k++) {
            int kind = kinds[k];
            if (kind == kBytePlain) st[n++] = bytes[k];
            else if (kind == kByteStuffed) st[n++] = 0xff;
            else if (kind == kByteRst) {
                if (rst_idx < F.n_intervals) {
                    RstEntry e;
                    e.tok = tok_pos + n;
                    e.number = bytes[k];
                    rst[rst_idx] = e;
                }
                rst_idx++;
            }
        }
    }
    __syncthreads();
    // copy out: whole 16-byte lines as vectors, the partial first and last lines by byte
    uint8_t *dst = F.tok + tile_tok - mis;  // 16-byte aligned
    const uint32_t span = mis + ttok, lines = (span + 15) / 16;
    for (uint32_t l = threadIdx.x; l < lines; l += blockDim.x) {
        const uint32_t b0 = l * 16, b1 = b0 + 16;
        if (b0 >= mis && b1 <= span) {
            *reinterpret_cast<uint4 *>(dst + b0) = *reinterpret_cast<const uint4 *>(s_tok + b0);
        } else {
            for (uint32_t b = max(b0, mis); b < min(b1, span); b++) dst[b] = s_tok[b];
        }
    }
    // The last tile that starts before the terminator publishes the totals (the
    // terminator may sit exactly on the next tile's first byte).
    if (threadIdx.x == 0 && term <= tr.base + (uint32_t)kScanTile) {
        L.states[tr.frame].n_tokens = tile_tok + ttok;
        L.states[tr.frame].n_rst = L.tile_rst[t] + trst;
    }
}

// ------------------------------------------------------------ entropy -----
//
// Frames with more than four components (their DC predictors do not fit the
// chunked decoder's per-slice sums): one restart interval per thread, a flat
// loop decoding one Huffman symbol per iteration (entropy_core.h).

template <int MAXC>
__device__ void decode_interval(const JpegLaunch &L, uint32_t item, int16_t *stage, const uint8_t *s_zz) {
    uint2 it = L.items[item];
    const uint32_t f = it.x, iv = it.y;
    const JFrame *Fp = L.frames + f;
    JState *st = L.states + f;
    unsigned long long termv = st->term;
    if (!Fp->decode || termv == ~0ull || ((termv >> 8) & 1)) return;
    const uint32_t n_int = Fp->n_intervals, ri = Fp->ri, total_mcus = Fp->total_mcus, mcu_cols = Fp->mcu_cols;
    const uint32_t sched_len = Fp->sched_len;
    const uint64_t blk_off = Fp->blk_off;
    const uint32_t n_rst = min(st->n_rst, n_int), n_tok = st->n_tokens;
    const RstEntry *rst = L.rsts + Fp->rst_off;
    uint32_t start;
    if (iv == 0) start = 0;
    else if (iv - 1 < n_rst) start = rst[iv - 1].tok;
    else return;  // no RST precedes this interval: an earlier interval fails its restart check
    const bool barrier_rst = iv < n_rst;
    const uint32_t barrier = barrier_rst ? rst[iv].tok : n_tok;
    const uint32_t limit = (barrier - start) * 8;

    Bits r;
    bits_init(r, Fp->tok, (unsigned long long)start * 8, 0);
    int32_t pred[MAXC];
#pragma unroll
    for (int c = 0; c < MAXC; c++) pred[c] = 0;
    int4 *stage4 = reinterpret_cast<int4 *>(stage);

    uint32_t mcu = iv * ri;
    const uint32_t mcu1 = min(mcu + ri, total_mcus);
    if (mcu >= mcu1 || sched_len == 0) return;
    uint32_t si = 0, comp = 0;
    const HuffLut *dcl = nullptr, *acl = nullptr;
    int32_t q0 = 0, dq = 0;
    uint64_t blk = 0;
    const JBlockRec *recs = L.brec + Fp->sched_off;
    auto setup_block = [&]() {
        const JBlockRec R = recs[si];
        comp = R.comp;
        const uint32_t mx = mcu % mcu_cols, my = mcu / mcu_cols;
        blk = blk_off + R.base_off + mx * R.mul_x + (uint64_t)my * R.mul_y;
        q0 = R.q0;
        dcl = L.luts + R.dc_lut;
        acl = L.luts + R.ac_lut;
    };
    setup_block();
    int k = 0;
    uint16_t kind = kDiagNone;
    uint32_t errpos = 0;
    for (;;) {
        int32_t val;
        uint16_t err;
        uint32_t eb;
        const int k0 = k;
        if (!decode_symbol(r, limit - r.used, k0 == 0 ? dcl : acl, L.symbols, k, val, err, eb)) {
            kind = err;
            errpos = eb;
            break;
        }
        if (k0 == 0) {  // decoder.rs:507-515
            int64_t p = (int64_t)pred[comp] + val;
            if (p > INT32_MAX || p < INT32_MIN) {
                kind = kJDcPredOverflow;
                errpos = r.used;
                break;
            }
            pred[comp] = (int32_t)p;
            int64_t d = p * (int64_t)q0;
            if (d > INT32_MAX || d < INT32_MIN) {
                kind = kJDcDeqOverflow;
                errpos = r.used;
                break;
            }
            dq = (int32_t)d;
            continue;
        }
        stage[s_zz[k - 1]] = (int16_t)val;
        if (k < 64) continue;
        // block complete: levels + dequantised DC out, staging cleared
        int4 *dst = reinterpret_cast<int4 *>(L.coef + blk * 64);
#pragma unroll
        for (int q = 0; q < 8; q++) {
            dst[q] = stage4[q];
            stage4[q] = make_int4(0, 0, 0, 0);
        }
        L.dc[blk] = dq;
        if (++si == sched_len) {
            si = 0;
            if (++mcu == mcu1) break;
        }
        setup_block();
        k = 0;
    }

    Diag out = make_diag(kDiagNone);
    if (kind != kDiagNone) {
        if (kind == kBarrierErr)
            out = barrier_rst ? make_diag(kJMarkerInData, barrier, 0xd0 + rst[iv].number) : make_diag(kJEndOfData, n_tok);
        else out = make_diag(kind, start + (errpos + 7) / 8);
    } else if (iv + 1 < n_int) {
        // consume_restart before the next interval (entropy.rs:111-134)
        uint32_t tend = start + (r.used + 7) / 8;
        uint32_t expected = iv & 7;
        if (barrier_rst && rst[iv].tok == tend) {
            if (rst[iv].number != expected) out = make_diag(kJRstMismatch, tend, expected, 0xd0 + rst[iv].number);
        } else if (tend < n_tok && Fp->tok[tend] == 0xff) {
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
    __shared__ uint8_t s_zz[64];
    int4 *mine = reinterpret_cast<int4 *>(s_stage + threadIdx.x * kStageStride);
#pragma unroll
    for (int q = 0; q < 8; q++) mine[q] = make_int4(0, 0, 0, 0);
    if (threadIdx.x < 64) s_zz[threadIdx.x] = (uint8_t)c_zigzag[threadIdx.x];
    __syncthreads();
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    decode_interval<MAXC>(L, first + i, s_stage + threadIdx.x * kStageStride, s_zz);
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
// (the transform core and its exactness bound live in idct_core.h)

constexpr int kIdctBlocks = 64;  // blocks per CTA, all of one (frame, component) range
constexpr int kIdctThreads = kIdctBlocks * 4;
constexpr int kIdctStride = 68;     // floats per staged block: 16-byte rows, 8 blocks on distinct banks
constexpr int kIdctOutStride = 72;  // output bytes per staged block: 8-byte rows, 8 blocks on distinct banks

__device__ __forceinline__ uint32_t find_range(const JpegLaunch &L, uint64_t g) {
    uint32_t lo = 0, hi = L.n_ranges;
    while (hi - lo > 1) {
        uint32_t mid = (lo + hi) >> 1;
        if (L.ranges[mid].first <= g) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Planar output: a CTA transforms 64 blocks of one (frame, component) range, four
// threads per block, and writes each block row as one 8-byte store.
__global__ void __launch_bounds__(kIdctThreads, 4) idct_kernel(JpegLaunch L) {
    __shared__ __align__(16) float s_f[kIdctBlocks * kIdctStride];
    __shared__ __align__(16) uint8_t s_o[kIdctBlocks * kIdctOutStride];
    __shared__ __align__(16) float s_q[64];
    __shared__ uint32_t s_range;
    if (threadIdx.x == 0) {
        uint32_t lo = 0, hi = L.n_ranges;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (L.idct_cta_first[mid] <= blockIdx.x) lo = mid;
            else hi = mid;
        }
        s_range = lo;
    }
    __syncthreads();
    const uint32_t r = s_range;
    const JBlockRange R = L.ranges[r];
    const JFrame &F = L.frames[R.frame];
    if (!L.item_ok[F.item]) return;
    const JComp &C = L.comps[F.comp_off + R.comp];
    if (threadIdx.x < 64) s_q[threadIdx.x] = (float)L.quant[F.quant_off + C.q * 64 + threadIdx.x];
    __syncthreads();
    const uint32_t nblk = C.bw * C.bh;
    const uint32_t lb = threadIdx.x >> 2, q = threadIdx.x & 3;
    const uint32_t local = (blockIdx.x - L.idct_cta_first[r]) * kIdctBlocks + lb;
    const bool valid = local < nblk;
    const uint64_t g = R.first + local;
    float *blk = s_f + lb * kIdctStride;
    float l1 = valid ? stage_rows(block_levels(L, g), L.dc, g, q, s_q, blk) : 0.0f;
#pragma unroll
    for (int o = 1; o < 4; o <<= 1) l1 += __shfl_xor_sync(0xffffffffu, l1, o);
    __syncwarp();
    const uint32_t gx = local % C.bw, gy = local / C.bw;
    unsigned long long mask = 0;
    if (valid) {
        mask = idct_block(blk, q, l1, s_o + lb * kIdctOutStride, 8);
    }
    if (mask) {
        // only samples inside the plane are written, and only those go to the exact pass
        const uint32_t vis_w = gx * 8 >= C.plane_w ? 0 : min(8u, C.plane_w - gx * 8);
        const uint32_t vis_h = gy * 8 >= C.plane_h ? 0 : min(8u, C.plane_h - gy * 8);
        const unsigned long long colm = 0x0101010101010101ull * ((1u << vis_w) - 1u);
        const unsigned long long rowm = vis_h >= 8 ? ~0ull : ((1ull << (8 * vis_h)) - 1ull);
        mask &= colm & rowm;
    }
#pragma unroll
    for (int o = 1; o < 4; o <<= 1) mask |= __shfl_xor_sync(0xffffffffu, mask, o);
    if (q == 0 && mask) {  // one entry per block: the queue holds n_blocks entries
        const uint32_t slot = atomicAdd(L.fix_count, 1u);
        L.fix[slot] = make_ulonglong2(g, mask);
        atomicAdd(L.fix_count + 1, (uint32_t)__popcll(mask));
    }
    __syncwarp();
    if (!valid) return;
    // rows 2q and 2q+1 of the block, 8 bytes each, clipped to the plane (blocks of
    // the MCU padding may lie wholly outside it)
    uint8_t *plane = F.planes + C.out_off;
    const uint32_t col0 = gx * 8;
    if (col0 >= C.plane_w) return;
    const uint32_t ncol = min(8u, C.plane_w - col0);
#pragma unroll
    for (int h = 0; h < 2; h++) {
        const uint32_t row = 2 * q + h, prow = gy * 8 + row;
        if (prow >= C.plane_h) continue;
        uint8_t *dst = plane + (uint64_t)prow * C.plane_w + col0;
        const uint8_t *srow = s_o + lb * kIdctOutStride + row * 8;
        if (ncol == 8 && (((uintptr_t)dst) & 7) == 0) {
            *reinterpret_cast<uint2 *>(dst) = *reinterpret_cast<const uint2 *>(srow);
        } else {
            for (uint32_t c = 0; c < ncol; c++) dst[c] = srow[c];
        }
    }
}

// The queued samples the fp32 transform could not decide, a warp per queued
// block: its exact coefficients into shared memory, then settle_samples
// (fixed-point value, or the reference order for genuine near-ties).
__global__ void __launch_bounds__(256) idct_fixup_kernel(JpegLaunch L) {
    __shared__ int32_t s_c[8][64];
    const uint32_t n = *L.fix_count;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int32_t *c = s_c[w];
    for (uint32_t i = blockIdx.x * 8 + w; i < n; i += gridDim.x * 8) {
        const ulonglong2 e = L.fix[i];
        const uint64_t g = e.x;
        const uint32_t r = find_range(L, g);
        const JFrame *F = &L.frames[L.ranges[r].frame];
        const JComp *C = &L.comps[F->comp_off + L.ranges[r].comp];
        const uint16_t *Q = L.quant + F->quant_off + C->q * 64;
        const int16_t *lv = block_levels(L, g);
        c[lane] = lane == 0 ? L.dc[g] : (int32_t)lv[lane] * (int32_t)Q[lane];
        c[lane + 32] = (int32_t)lv[lane + 32] * (int32_t)Q[lane + 32];
        __syncwarp();
        const uint32_t local = (uint32_t)(g - L.ranges[r].first);
        const uint32_t gx = local % C->bw, gy = local / C->bw;
        uint8_t *plane = F->planes + C->out_off;
        settle_samples(L.fixw, c, e.y, [&](int y, int x, uint8_t v) {
            plane[(uint64_t)(gy * 8 + y) * C->plane_w + gx * 8 + x] = v;
        });
        __syncwarp();
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
    uint32_t big = L.n_items - L.n_items_small;
    if (big)
        entropy_kernel<256><<<(big + kEntropyThreads - 1) / kEntropyThreads, kEntropyThreads, 0, s>>>(
            L, L.n_items_small, big);
    if (L.n_frames) resolve_kernel<<<(L.n_frames + 127) / 128, 128, 0, s>>>(L);
}

uint32_t idct_ctas(uint32_t blocks) { return (blocks + kIdctBlocks - 1) / kIdctBlocks; }

void launch_jpeg_idct(const JpegLaunch &L, cudaStream_t s) {
    if (L.n_blocks == 0 || L.n_idct_ctas == 0) return;
    idct_kernel<<<L.n_idct_ctas, kIdctThreads, 0, s>>>(L);
    idct_fixup_kernel<<<L.fixup_grid, 256, 0, s>>>(L);
}

}  // namespace mmr
