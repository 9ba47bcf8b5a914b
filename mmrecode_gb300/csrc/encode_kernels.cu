// Batch JPEG encoder on the GPU (sm_103a): the reference encoder's forward DCT,
// quantisation and Huffman coding (crates/codecs/mjpeg/src/encoder.rs:341-545,
// transform.rs:111-134), byte-identical to it, for many frames per pass.
//
//   fdct_kernel        8 threads per 8x8 block: edge-replicated samples, fp32 row and
//                      column passes, quantisation; a coefficient whose quotient lies
//                      within its error bound of a half-integer is recomputed in
//                      binary64 in the reference's operation order
//   bits_kernel        thread per block: Huffman bit count (DC difference against the
//                      previous block of the component in its restart interval)
//   scan (3 kernels)   exclusive prefix of the bit counts, of the segment words and
//                      chunks, of the 0xFF counts and of the frame sizes
//   segment_kernel     thread per restart interval ("segment"): its bits, bytes,
//                      words and 16-byte chunks
//   write_bits_kernel  thread per block: its codes into the segment's bit buffer
//                      (interior words stored, the two shared edge words OR-ed)
//   ff_count_kernel    thread per 16-byte chunk: 0xFF bytes (each gets a stuffed 0x00)
//   layout_kernel      thread per frame: where each segment lands after stuffing
//   emit_kernel        thread per chunk: stuffed bytes, then RSTn or EOI after the
//                      segment's last chunk
// The header bytes (SOI .. SOS) are the host plan's (plan_jpeg_encode).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "common.h"
#include "encode.h"
#include "encode_gpu.h"
#include "fdct_core.h"
#include "tables.h"

namespace mmr {
namespace {


struct EncFrame {
    const uint8_t *plane[3];
    uint32_t pw[3], ph[3];
    size_t stride[3];
    uint32_t mcu_cols, mcus, bpm, ri;  // MCUs per row, MCUs, blocks per MCU, restart interval (0: none)
    uint64_t block_base;               // first block of the frame (scan order, batch-wide)
    uint32_t seg_base, nseg;           // first segment, segments (restart intervals)
    uint8_t sched_comp[10], sched_bx[10], sched_by[10];
    uint8_t comp_first[3], comp_count[3], comp_h[3], comp_v[3], comp_tq[3], comp_tab[3];
};

struct EncLaunch {
    const EncFrame *frames;
    uint32_t n_frames;
    uint64_t n_blocks;
    uint32_t n_segs;
    const uint8_t *qt;        // [2][64] natural order
    const uint32_t *codes;    // [dc 0, dc 1, ac 0, ac 1][256]: bits | length << 16
    const float *rq;          // [2][64] fp32 reciprocals of qt
    const uint8_t *nat2zz;    // [64] zigzag position of each natural index
    int16_t *coef;            // 64 per block, zigzag order
    uint32_t *block_bits;     // per block
    uint64_t *bit_off;        // n_blocks + 1
    uint32_t *seg_words;      // per segment, 4 per chunk (scanned into seg_word_off)
    uint32_t *seg_chunks;     // per segment (scanned into seg_chunk_off)
    uint64_t *seg_bits;       // per segment
    uint64_t *seg_word_off;   // n_segs + 1
    uint64_t *seg_chunk_off;  // n_segs + 1
    uint32_t *raw;            // segment bit buffers, big-endian words
    uint32_t *chunk_ff;       // per chunk
    uint64_t *ff_off;         // n_chunks + 1
    uint32_t *seg_out;        // per segment: its offset in the frame's entropy bytes
    uint32_t *frame_len;      // per frame: entropy bytes, markers and EOI
    uint64_t *frame_off;      // n_frames + 1
    uint8_t *out;             // entropy bytes of all frames
    unsigned long long *exact;  // coefficients recomputed in binary64
};

// frame holding global block b (frames sorted by block_base)
__device__ __forceinline__ uint32_t frame_of_block(const EncLaunch &L, uint64_t b) {
    uint32_t lo = 0, hi = L.n_frames - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (L.frames[mid].block_base <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ uint32_t frame_of_segment(const EncLaunch &L, uint32_t s) {
    uint32_t lo = 0, hi = L.n_frames - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (L.frames[mid].seg_base <= s) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

__device__ __forceinline__ uint32_t segment_of_chunk(const EncLaunch &L, uint64_t c) {
    uint32_t lo = 0, hi = L.n_segs - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (L.seg_chunk_off[mid] <= c) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ----------------------------------------------------------------- FDCT ---

constexpr int kEncBlocksPerCta = 32;

__global__ void __launch_bounds__(256) fdct_kernel(EncLaunch L) {
    __shared__ float s_in[kEncBlocksPerCta][8][9];
    __shared__ float s_row[kEncBlocksPerCta][8][9];
    __shared__ float s_mag[kEncBlocksPerCta][8][9];  // sum_x |M[x][u]| |S[r][x]|
    __shared__ uint8_t s_raw[kEncBlocksPerCta][64];
    const int lb = threadIdx.x >> 3, r = threadIdx.x & 7;
    const uint64_t blk = (uint64_t)blockIdx.x * kEncBlocksPerCta + lb;
    const bool valid = blk < L.n_blocks;
    uint32_t tq = 0;
    if (valid) {
        const EncFrame &F = L.frames[frame_of_block(L, blk)];
        const uint64_t i = blk - F.block_base;
        const uint32_t mcu = (uint32_t)(i / F.bpm), k = (uint32_t)(i % F.bpm);
        const uint32_t c = F.sched_comp[k];
        tq = F.comp_tq[c];
        const uint32_t mx = mcu % F.mcu_cols, my = mcu / F.mcu_cols;
        const uint32_t x0 = (mx * F.comp_h[c] + F.sched_bx[k]) * 8, y0 = (my * F.comp_v[c] + F.sched_by[k]) * 8;
        // read_block (encoder.rs:392-402): rows and columns past the plane repeat its last
        const uint32_t sy = min(y0 + r, F.ph[c] - 1);
        const uint8_t *row = F.plane[c] + (size_t)sy * F.stride[c];
        uint8_t px[8];
        if (x0 + 8 <= F.pw[c] && (reinterpret_cast<uintptr_t>(row + x0) & 7) == 0) {  // one 8-byte load
            const uint2 w = *reinterpret_cast<const uint2 *>(row + x0);
#pragma unroll
            for (int xx = 0; xx < 8; xx++) px[xx] = (uint8_t)((xx < 4 ? w.x : w.y) >> (8 * (xx & 3)));
        } else {
#pragma unroll
            for (int xx = 0; xx < 8; xx++) px[xx] = row[min(x0 + xx, F.pw[c] - 1)];
        }
#pragma unroll
        for (int xx = 0; xx < 8; xx++) {
            s_raw[lb][r * 8 + xx] = px[xx];
            s_in[lb][r][xx] = (float)px[xx] - 128.0f;
        }
    }
    __syncthreads();
    if (valid) {  // row pass: t[r][u] = sum_x M[x][u] S[r][x], and its magnitude sum
#pragma unroll
        for (int u = 0; u < 8; u++) fdct_row_pass(s_in[lb][r], u, s_row[lb][r][u], s_mag[lb][r][u]);
    }
    __syncthreads();
    __shared__ __align__(16) int16_t s_out[kEncBlocksPerCta][64];  // the block in zigzag order
    if (valid) {
        const int u = r;  // column pass: this thread's column
        const uint8_t *qt = L.qt + tq * 64;
        const float *rq = L.rq + tq * 64;
#pragma unroll
        for (int v = 0; v < 8; v++) {
            bool exact;
            int k = fdct_quantise(&s_row[lb][0][0], &s_mag[lb][0][0], 9, s_raw[lb], u, v, qt[v * 8 + u],
                                  rq[v * 8 + u], exact);
            if (exact) atomicAdd(L.exact, 1ull);
            if (v | u) k = min(max(k, -1023), 1023);  // encode_scan (encoder.rs:372-374)
            s_out[lb][L.nat2zz[v * 8 + u]] = (int16_t)k;
        }
    }
    __syncthreads();
    if (valid)  // 16 bytes per thread: the block's 128 bytes in one coalesced row
        reinterpret_cast<uint4 *>(L.coef + blk * 64)[r] = reinterpret_cast<const uint4 *>(s_out[lb])[r];
}

// ------------------------------------------------------------- Huffman ---

__device__ __forceinline__ uint32_t category(int v) { return v ? 32u - __clz(v < 0 ? -v : v) : 0u; }

// Walks the symbols of block blk (encode_block, encoder.rs:404-425) and hands each
// code and amplitude to emit(value, bits).
template <class Emit>
__device__ __forceinline__ void block_symbols(const EncLaunch &L, const EncFrame &F, uint64_t blk, Emit emit) {
    const uint64_t i = blk - F.block_base;
    const uint32_t mcu = (uint32_t)(i / F.bpm), k = (uint32_t)(i % F.bpm);
    const uint32_t c = F.sched_comp[k];
    // the DC prediction: the previous block of the component in this restart interval
    const bool interval_start = F.ri ? mcu % F.ri == 0 : mcu == 0;
    int pred = 0;
    if (k != F.comp_first[c]) pred = L.coef[(blk - 1) * 64];
    else if (!interval_start) pred = L.coef[(blk - F.bpm + F.comp_count[c] - 1) * 64];
    // the block's coefficients in zigzag order, eight 16-byte loads
    const uint4 *cz = reinterpret_cast<const uint4 *>(L.coef + blk * 64);
    const uint32_t *dc = L.codes + F.comp_tab[c] * 256, *ac = L.codes + (2 + F.comp_tab[c]) * 256;
    uint4 q = cz[0];
    const int diff = (int)(int16_t)(q.x & 0xffffu) - pred;
    const uint32_t dsz = category(diff);
    const uint32_t dcode = __ldg(dc + dsz);
    emit(dcode & 0xffffu, dcode >> 16);
    if (dsz) emit((uint32_t)(diff < 0 ? diff + (1 << dsz) - 1 : diff) & ((1u << dsz) - 1), dsz);
    uint32_t run = 0;
#pragma unroll 1
    for (int ch = 0; ch < 8; ch++) {
        if (ch) q = cz[ch];
        const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int j = 0; j < 8; j++) {
            if (ch == 0 && j == 0) continue;  // the DC
            const int v = (int)(int16_t)(w[j >> 1] >> (16 * (j & 1)));
            if (v == 0) {
                run++;
                continue;
            }
            const uint32_t zrl = __ldg(ac + 0xf0);
            for (; run >= 16; run -= 16) emit(zrl & 0xffffu, zrl >> 16);
            const uint32_t sz = category(v);
            const uint32_t code = __ldg(ac + ((run << 4) | sz));
            emit(code & 0xffffu, code >> 16);
            emit((uint32_t)(v < 0 ? v + (1 << sz) - 1 : v) & ((1u << sz) - 1), sz);
            run = 0;
        }
    }
    if (run) {
        const uint32_t eob = __ldg(ac);
        emit(eob & 0xffffu, eob >> 16);
    }
}

__global__ void __launch_bounds__(256) bits_kernel(EncLaunch L) {
    const uint64_t blk = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (blk >= L.n_blocks) return;
    const EncFrame &F = L.frames[frame_of_block(L, blk)];
    uint32_t bits = 0;
    block_symbols(L, F, blk, [&](uint32_t, uint32_t n) { bits += n; });
    L.block_bits[blk] = bits;
}

// first block (batch-wide) of segment j of frame F, j <= nseg
__device__ __forceinline__ uint64_t segment_block(const EncFrame &F, uint32_t j) {
    const uint32_t mcu = F.ri ? min(j * F.ri, F.mcus) : (j ? F.mcus : 0u);
    return F.block_base + (uint64_t)mcu * F.bpm;
}

__global__ void segment_kernel(EncLaunch L) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= L.n_segs) return;
    const EncFrame &F = L.frames[frame_of_segment(L, s)];
    const uint32_t j = s - F.seg_base;
    const uint64_t bits = L.bit_off[segment_block(F, j + 1)] - L.bit_off[segment_block(F, j)];
    const uint64_t bytes = (bits + 7) / 8;  // the last byte padded with 1 bits
    L.seg_bits[s] = bits;
    // whole 16-byte chunks, so that every chunk's 16-byte load is aligned and inside its segment
    L.seg_chunks[s] = (uint32_t)((bytes + 15) / 16);
    L.seg_words[s] = 4 * L.seg_chunks[s];
}

// Writes block blk's codes at its bit offset in its segment's big-endian word
// buffer (zeroed): whole words of this block are stored, the first word (shared
// with the previous block unless the block starts on a word) and the last partial
// one are OR-ed. The segment's last block pads its final byte with 1 bits
// (EntropyWriter::finish, encoder.rs:530-543).
__global__ void __launch_bounds__(256) write_bits_kernel(EncLaunch L) {
    const uint64_t blk = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (blk >= L.n_blocks) return;
    const EncFrame &F = L.frames[frame_of_block(L, blk)];
    const uint32_t mcu = (uint32_t)((blk - F.block_base) / F.bpm);
    const uint32_t j = F.ri ? mcu / F.ri : 0u;
    const uint64_t seg0 = segment_block(F, j), seg1 = segment_block(F, j + 1);
    const uint64_t p = L.bit_off[blk] - L.bit_off[seg0];
    uint32_t *words = L.raw + L.seg_word_off[F.seg_base + j];
    uint64_t w = p >> 5;
    uint64_t acc = 0;
    uint32_t nacc = (uint32_t)(p & 31);  // pending bits, counting the word's earlier bits as zeros
    bool shared_first = nacc != 0;
    auto emit = [&](uint32_t value, uint32_t n) {
        acc = (acc << n) | value;
        nacc += n;
        if (nacc >= 32) {
            nacc -= 32;
            const uint32_t word = (uint32_t)(acc >> nacc);
            if (shared_first) atomicOr(words + w, word);
            else words[w] = word;
            shared_first = false;
            w++;
            acc &= (1ull << nacc) - 1;
        }
    };
    block_symbols(L, F, blk, emit);
    if (blk + 1 == seg1) {
        const uint32_t pad = (8u - (uint32_t)((L.bit_off[seg1] - L.bit_off[seg0]) & 7)) & 7u;
        if (pad) emit((1u << pad) - 1, pad);
    }
    if (nacc) atomicOr(words + w, (uint32_t)(acc << (32 - nacc)));
}

// big-endian word: stream byte b of the word is bits 31 - 8b .. 24 - 8b; the first
// nv bytes as a mask of their top bits
__device__ __forceinline__ uint32_t lead_bytes_mask(int nv) {
    return nv >= 4 ? 0x80808080u : nv <= 0 ? 0u : (0x80808080u << (8 * (4 - nv)));
}

__device__ __forceinline__ void chunk_of(const EncLaunch &L, uint64_t c, uint32_t *s, uint64_t *k, uint32_t *n) {
    *s = segment_of_chunk(L, c);
    *k = c - L.seg_chunk_off[*s];
    const uint64_t bytes = (L.seg_bits[*s] + 7) / 8;
    *n = (uint32_t)min((uint64_t)16, bytes - 16 * *k);
}

__global__ void __launch_bounds__(256) ff_count_kernel(EncLaunch L, uint64_t n_chunks) {
    const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_chunks) return;
    uint32_t s, n;
    uint64_t k;
    chunk_of(L, c, &s, &k, &n);
    const uint4 v = *reinterpret_cast<const uint4 *>(L.raw + L.seg_word_off[s] + 4 * k);
    const uint32_t w[4] = {v.x, v.y, v.z, v.w};
    uint32_t count = 0;
#pragma unroll
    for (int q = 0; q < 4; q++) count += __popc(zero_bytes(~w[q]) & lead_bytes_mask((int)n - 4 * q));
    L.chunk_ff[c] = count;
}

// thread per frame: each segment's offset in the frame's entropy bytes, each
// segment followed by its marker (RSTn, or EOI after the last)
__global__ void layout_kernel(EncLaunch L) {
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= L.n_frames) return;
    const EncFrame &F = L.frames[f];
    uint64_t pos = 0;
    for (uint32_t j = 0; j < F.nseg; j++) {
        const uint32_t s = F.seg_base + j;
        L.seg_out[s] = (uint32_t)pos;
        const uint64_t ff = L.ff_off[L.seg_chunk_off[s + 1]] - L.ff_off[L.seg_chunk_off[s]];
        pos += (L.seg_bits[s] + 7) / 8 + ff + 2;
    }
    L.frame_len[f] = (uint32_t)pos;
}

// thread per chunk: its bytes with a 0x00 after each 0xFF (EntropyWriter::push,
// encoder.rs:519-528), then the segment's marker after its last chunk
__global__ void __launch_bounds__(256) emit_kernel(EncLaunch L, uint64_t n_chunks) {
    const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_chunks) return;
    uint32_t s, n;
    uint64_t k;
    chunk_of(L, c, &s, &k, &n);
    const EncFrame &F = L.frames[frame_of_segment(L, s)];
    const uint32_t j = s - F.seg_base;
    uint8_t *dst = L.out + L.frame_off[frame_of_segment(L, s)] + L.seg_out[s] + 16 * k +
                   (L.ff_off[c] - L.ff_off[L.seg_chunk_off[s]]);
    const uint32_t *w = L.raw + L.seg_word_off[s] + 4 * k;
    for (uint32_t b = 0; b < n; b++) {
        const uint8_t v = (uint8_t)(w[b >> 2] >> (24 - 8 * (b & 3)));
        *dst++ = v;
        if (v == 0xff) *dst++ = 0x00;
    }
    const uint64_t bytes = (L.seg_bits[s] + 7) / 8;
    if (16 * k + n == bytes) {
        dst[0] = 0xff;
        dst[1] = j + 1 < F.nseg ? (uint8_t)(0xd0 + (j & 7)) : (uint8_t)0xd9;
    }
}

// ----------------------------------------------------------------- scan ---

constexpr int kScanThreads = 1024;
constexpr int kScanItems = 4;  // consecutive values per thread
constexpr uint64_t kScanTile = (uint64_t)kScanThreads * kScanItems;

// exclusive prefix of v over the CTA (1024 threads); *total = the CTA's sum
__device__ __forceinline__ uint64_t cta_exclusive(uint64_t v, uint64_t *total) {
    __shared__ uint64_t s_warp[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t incl = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint64_t o = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d) incl += o;
    }
    if (lane == 31) s_warp[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint64_t w = s_warp[lane], wi = w;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint64_t o = __shfl_up_sync(0xffffffffu, wi, d);
            if (lane >= d) wi += o;
        }
        s_warp[lane] = wi - w;
        if (lane == 31) *total = wi;
    }
    __syncthreads();
    const uint64_t r = s_warp[warp] + incl - v;
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(kScanThreads) scan_reduce_kernel(const uint32_t *in, uint64_t n, uint64_t *part) {
    __shared__ uint64_t s_total;
    const uint64_t base = blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    uint64_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n) sum += in[base + k];
    cta_exclusive(sum, &s_total);
    __syncthreads();
    if (threadIdx.x == 0) part[blockIdx.x] = s_total;
}

// one CTA: exclusive prefix of the tile sums in place; the grand total to *total
__global__ void __launch_bounds__(kScanThreads) scan_partials_kernel(uint64_t *part, uint64_t np, uint64_t *total) {
    __shared__ uint64_t s_total;
    uint64_t carry = 0;
    for (uint64_t b = 0; b < np; b += kScanThreads) {
        const uint64_t i = b + threadIdx.x;
        const uint64_t v = i < np ? part[i] : 0;
        const uint64_t ex = cta_exclusive(v, &s_total);
        __syncthreads();
        if (i < np) part[i] = carry + ex;
        carry += s_total;
        __syncthreads();
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void __launch_bounds__(kScanThreads) scan_apply_kernel(const uint32_t *in, uint64_t n,
                                                                    const uint64_t *part, uint64_t *out) {
    __shared__ uint64_t s_total;
    const uint64_t base = blockIdx.x * kScanTile + (uint64_t)threadIdx.x * kScanItems;
    uint32_t v[kScanItems];
    uint64_t sum = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; k++) {
        v[k] = base + k < n ? in[base + k] : 0u;
        sum += v[k];
    }
    uint64_t run = part[blockIdx.x] + cta_exclusive(sum, &s_total);
#pragma unroll
    for (int k = 0; k < kScanItems; k++)
        if (base + k < n) {
            out[base + k] = run;
            run += v[k];
        }
}

// out[0, n) = exclusive prefix of in, out[n] = the sum (part: ceil(n / 4096) scratch)
void exclusive_scan(const uint32_t *in, uint64_t n, uint64_t *out, uint64_t *part, cudaStream_t s) {
    const uint64_t tiles = (n + kScanTile - 1) / kScanTile;
    if (tiles == 0) {
        cudaMemsetAsync(out, 0, sizeof(uint64_t), s);
        return;
    }
    scan_reduce_kernel<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, part);
    scan_partials_kernel<<<1, kScanThreads, 0, s>>>(part, tiles, out + n);
    scan_apply_kernel<<<(unsigned)tiles, kScanThreads, 0, s>>>(in, n, part, out);
}

}  // namespace

// ---------------------------------------------------------------- host ---

size_t jpeg_encode_bound(uint32_t format, size_t width, size_t height, uint16_t restart_interval) {
    size_t hmax = 1, vmax = 1, bpm = 1;
    switch (format) {
    case kYuv420: hmax = vmax = 2; bpm = 6; break;
    case kYuv422: hmax = 2; bpm = 4; break;
    case kYuv444: bpm = 3; break;
    default: break;
    }
    const size_t mcus = ((width + 8 * hmax - 1) / (8 * hmax)) * ((height + 8 * vmax - 1) / (8 * vmax));
    const size_t segs = restart_interval ? (mcus + restart_interval - 1) / restart_interval : 1;
    // DC: code <= 16 + amplitude 11 bits; 63 AC coefficients: code <= 16 + amplitude 10
    // bits: 1665 bits < 209 bytes, each possibly stuffed; per segment a padded byte
    // (stuffed) and a marker
    return 1024 + mcus * bpm * 418 + segs * 4 + 2;
}

namespace {

struct DBuf {
    void *p = nullptr;
    size_t cap = 0;
    void ensure(size_t bytes) {
        if (bytes <= cap) return;
        const size_t want = std::max(bytes, cap + cap / 2);
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        if (cudaMalloc(&p, want) != cudaSuccess) {
            cudaGetLastError();
            throw std::runtime_error("GPU encoder: out of device memory");
        }
        cap = want;
    }
    template <class T>
    T *as() const {
        return static_cast<T *>(p);
    }
    ~DBuf() {
        if (p) cudaFree(p);
    }
};

}  // namespace

struct GpuJpegEncoder::Impl {
    int device = 0;
    cudaStream_t s = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::mutex mu;
    DBuf frames, tabs, in, coef, block_bits, bit_off, part, seg_bits, seg_words, seg_chunks, seg_word_off,
        seg_chunk_off, raw, chunk_ff, ff_off, seg_out, frame_len, frame_off, out, exact;
};

GpuJpegEncoder::GpuJpegEncoder(int device) : impl_(new Impl) {
    impl_->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&impl_->s, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&impl_->ev0) != cudaSuccess || cudaEventCreate(&impl_->ev1) != cudaSuccess) {
        if (impl_->ev0) cudaEventDestroy(impl_->ev0);
        if (impl_->ev1) cudaEventDestroy(impl_->ev1);
        if (impl_->s) cudaStreamDestroy(impl_->s);
        cudaGetLastError();
        delete impl_;
        throw std::runtime_error("GPU encoder: cannot create its stream");
    }
}

GpuJpegEncoder::~GpuJpegEncoder() {
    cudaSetDevice(impl_->device);
    cudaStreamSynchronize(impl_->s);
    cudaStreamDestroy(impl_->s);
    cudaEventDestroy(impl_->ev0);
    cudaEventDestroy(impl_->ev1);
    delete impl_;
}

int32_t GpuJpegEncoder::encode(EncodeItem *items, size_t n, const JpegEncodeOptions &opt) {
    Impl &I = *impl_;
    std::lock_guard<std::mutex> g(I.mu);
    stats_ = EncodeStats();
    if (cudaSetDevice(I.device) != cudaSuccess) {
        cudaGetLastError();
        return kInternal;
    }
    // host plans: validation, tables and header bytes per frame
    std::vector<JpegEncodePlan> plans(n);
    std::vector<size_t> live;
    for (size_t i = 0; i < n; i++) {
        EncodeItem &it = items[i];
        it.status = kOk;
        it.message.clear();
        it.out_len = 0;
        if (!plan_jpeg_encode(it.frame, opt, &plans[i])) {
            it.status = plans[i].status;
            it.message = plans[i].message;
            continue;
        }
        live.push_back(i);
    }
    if (live.empty()) return kOk;
    const JpegEncodePlan &P0 = plans[live[0]];  // tables depend on the options only
    // device tables: qt [2][64] | codes [4][256] | fp32 reciprocals of qt [2][64] | zigzag
    // position of each natural index [64]
    std::vector<uint8_t> tab(128 + 4 * 256 * 4 + 2 * 64 * 4 + 64);
    memcpy(tab.data(), P0.qt, 128);
    float *rq = reinterpret_cast<float *>(tab.data() + 128 + 4096);
    for (int t = 0; t < 2; t++)
        for (int i = 0; i < 64; i++) rq[t * 64 + i] = 1.0f / (float)P0.qt[t][i];
    static const int kZigzagOrder[64] = MMR_ZIGZAG_INIT;
    for (int k = 0; k < 64; k++) tab[128 + 4096 + 512 + kZigzagOrder[k]] = (uint8_t)k;
    uint32_t *codes = reinterpret_cast<uint32_t *>(tab.data() + 128);
    for (int t = 0; t < 2; t++)
        for (int sym = 0; sym < 256; sym++) {
            codes[t * 256 + sym] = P0.dc[t][sym].bits | (uint32_t)P0.dc[t][sym].length << 16;
            codes[(2 + t) * 256 + sym] = P0.ac[t][sym].bits | (uint32_t)P0.ac[t][sym].length << 16;
        }
    // frame records; host planes go up packed (stride = width)
    std::vector<EncFrame> fr(live.size());
    uint64_t blocks = 0, in_bytes = 0;
    uint32_t segs = 0;
    for (size_t k = 0; k < live.size(); k++) {
        const EncodeItem &it = items[live[k]];
        const JpegEncodePlan &P = plans[live[k]];
        EncFrame &F = fr[k];
        memset(&F, 0, sizeof F);
        F.mcu_cols = (uint32_t)P.mcu_cols;
        F.mcus = (uint32_t)(P.mcu_cols * P.mcu_rows);
        F.ri = P.restart_interval;
        uint32_t bpm = 0;
        for (uint32_t c = 0; c < P.ncomp; c++) {
            F.comp_first[c] = (uint8_t)bpm;
            F.comp_count[c] = (uint8_t)(P.comp_h[c] * P.comp_v[c]);
            F.comp_h[c] = P.comp_h[c];
            F.comp_v[c] = P.comp_v[c];
            F.comp_tq[c] = P.comp_tq[c];
            F.comp_tab[c] = P.comp_table[c];
            for (uint32_t by = 0; by < P.comp_v[c]; by++)
                for (uint32_t bx = 0; bx < P.comp_h[c]; bx++) {
                    F.sched_comp[bpm] = (uint8_t)c;
                    F.sched_bx[bpm] = (uint8_t)bx;
                    F.sched_by[bpm] = (uint8_t)by;
                    bpm++;
                }
            const PlaneIn &pl = it.frame.planes[c];
            F.pw[c] = (uint32_t)pl.width;
            F.ph[c] = (uint32_t)pl.height;
            if (!it.in_on_device) in_bytes += (pl.width * pl.height + 255) / 256 * 256;
        }
        F.bpm = bpm;
        F.block_base = blocks;
        F.seg_base = segs;
        F.nseg = F.ri ? (F.mcus + F.ri - 1) / F.ri : 1;
        blocks += (uint64_t)F.mcus * bpm;
        segs += F.nseg;
    }
    stats_.blocks = blocks;
    try {
        cudaEventRecord(I.ev0, I.s);
        I.in.ensure(std::max<uint64_t>(in_bytes, 256));
        uint64_t at = 0;
        for (size_t k = 0; k < live.size(); k++) {
            const EncodeItem &it = items[live[k]];
            for (uint32_t c = 0; c < plans[live[k]].ncomp; c++) {
                const PlaneIn &pl = it.frame.planes[c];
                if (it.in_on_device) {
                    fr[k].plane[c] = pl.data;
                    fr[k].stride[c] = pl.stride;
                    continue;
                }
                uint8_t *dst = I.in.as<uint8_t>() + at;
                // contiguous planes go up as one linear copy, strided ones row by row
                const cudaError_t e =
                    pl.stride == pl.width
                        ? cudaMemcpyAsync(dst, pl.data, pl.width * pl.height, cudaMemcpyHostToDevice, I.s)
                        : cudaMemcpy2DAsync(dst, pl.width, pl.data, pl.stride, pl.width, pl.height,
                                            cudaMemcpyHostToDevice, I.s);
                if (e != cudaSuccess) throw std::runtime_error("GPU encoder: upload failed");
                fr[k].plane[c] = dst;
                fr[k].stride[c] = pl.width;
                at += (pl.width * pl.height + 255) / 256 * 256;
            }
        }
        const uint32_t nf = (uint32_t)live.size();
        I.frames.ensure(nf * sizeof(EncFrame));
        I.tabs.ensure(tab.size());
        cudaMemcpyAsync(I.frames.p, fr.data(), nf * sizeof(EncFrame), cudaMemcpyHostToDevice, I.s);
        cudaMemcpyAsync(I.tabs.p, tab.data(), tab.size(), cudaMemcpyHostToDevice, I.s);
        I.coef.ensure(blocks * 128);
        I.block_bits.ensure(blocks * 4);
        I.bit_off.ensure((blocks + 1) * 8);
        I.part.ensure(((std::max<uint64_t>(blocks, segs) + kScanTile - 1) / kScanTile + 1) * 8);
        I.seg_bits.ensure(segs * 8);
        I.seg_words.ensure(segs * 4);
        I.seg_chunks.ensure(segs * 4);
        I.seg_word_off.ensure((segs + 1) * 8);
        I.seg_chunk_off.ensure((segs + 1) * 8);
        I.seg_out.ensure(segs * 4);
        I.frame_len.ensure(nf * 4);
        I.frame_off.ensure((nf + 1) * 8);
        I.exact.ensure(8);
        EncLaunch L;
        memset(&L, 0, sizeof L);
        L.frames = I.frames.as<EncFrame>();
        L.n_frames = nf;
        L.n_blocks = blocks;
        L.n_segs = segs;
        L.qt = I.tabs.as<uint8_t>();
        L.codes = reinterpret_cast<const uint32_t *>(I.tabs.as<uint8_t>() + 128);
        L.rq = reinterpret_cast<const float *>(I.tabs.as<uint8_t>() + 128 + 4096);
        L.nat2zz = I.tabs.as<uint8_t>() + 128 + 4096 + 512;
        L.coef = I.coef.as<int16_t>();
        L.block_bits = I.block_bits.as<uint32_t>();
        L.bit_off = I.bit_off.as<uint64_t>();
        L.seg_words = I.seg_words.as<uint32_t>();
        L.seg_chunks = I.seg_chunks.as<uint32_t>();
        L.seg_bits = I.seg_bits.as<uint64_t>();
        L.seg_word_off = I.seg_word_off.as<uint64_t>();
        L.seg_chunk_off = I.seg_chunk_off.as<uint64_t>();
        L.seg_out = I.seg_out.as<uint32_t>();
        L.frame_len = I.frame_len.as<uint32_t>();
        L.frame_off = I.frame_off.as<uint64_t>();
        L.exact = I.exact.as<unsigned long long>();
        cudaMemsetAsync(L.exact, 0, 8, I.s);
        const unsigned bgrid = (unsigned)((blocks + 255) / 256);
        fdct_kernel<<<(unsigned)((blocks + kEncBlocksPerCta - 1) / kEncBlocksPerCta), 256, 0, I.s>>>(L);
        bits_kernel<<<bgrid, 256, 0, I.s>>>(L);
        exclusive_scan(L.block_bits, blocks, L.bit_off, I.part.as<uint64_t>(), I.s);
        segment_kernel<<<(segs + 255) / 256, 256, 0, I.s>>>(L);
        exclusive_scan(L.seg_words, segs, L.seg_word_off, I.part.as<uint64_t>(), I.s);
        exclusive_scan(L.seg_chunks, segs, L.seg_chunk_off, I.part.as<uint64_t>(), I.s);
        uint64_t totals[2] = {0, 0};
        cudaMemcpyAsync(&totals[0], L.seg_word_off + segs, 8, cudaMemcpyDeviceToHost, I.s);
        cudaMemcpyAsync(&totals[1], L.seg_chunk_off + segs, 8, cudaMemcpyDeviceToHost, I.s);
        if (cudaStreamSynchronize(I.s) != cudaSuccess) throw std::runtime_error("GPU encoder: device failure");
        const uint64_t words = totals[0], chunks = totals[1];
        I.raw.ensure(std::max<uint64_t>(words, 4) * 4);
        I.chunk_ff.ensure(std::max<uint64_t>(chunks, 1) * 4);
        I.ff_off.ensure((chunks + 1) * 8);
        I.part.ensure(((std::max<uint64_t>(chunks, nf) + kScanTile - 1) / kScanTile + 1) * 8);
        I.out.ensure(std::max<uint64_t>(chunks * 32 + (uint64_t)segs * 2, 16));
        L.raw = I.raw.as<uint32_t>();
        L.chunk_ff = I.chunk_ff.as<uint32_t>();
        L.ff_off = I.ff_off.as<uint64_t>();
        L.out = I.out.as<uint8_t>();
        cudaMemsetAsync(L.raw, 0, words * 4, I.s);
        write_bits_kernel<<<bgrid, 256, 0, I.s>>>(L);
        ff_count_kernel<<<(unsigned)((chunks + 255) / 256), 256, 0, I.s>>>(L, chunks);
        exclusive_scan(L.chunk_ff, chunks, L.ff_off, I.part.as<uint64_t>(), I.s);
        layout_kernel<<<(nf + 127) / 128, 128, 0, I.s>>>(L);
        exclusive_scan(L.frame_len, nf, L.frame_off, I.part.as<uint64_t>(), I.s);
        emit_kernel<<<(unsigned)((chunks + 255) / 256), 256, 0, I.s>>>(L, chunks);
        if (cudaGetLastError() != cudaSuccess) throw std::runtime_error("GPU encoder: launch failed");
        std::vector<uint32_t> len(nf);
        std::vector<uint64_t> off(nf + 1);
        uint64_t exact = 0;
        cudaMemcpyAsync(len.data(), L.frame_len, nf * 4, cudaMemcpyDeviceToHost, I.s);
        cudaMemcpyAsync(off.data(), L.frame_off, (nf + 1) * 8, cudaMemcpyDeviceToHost, I.s);
        cudaMemcpyAsync(&exact, L.exact, 8, cudaMemcpyDeviceToHost, I.s);
        if (cudaStreamSynchronize(I.s) != cudaSuccess) throw std::runtime_error("GPU encoder: device failure");
        stats_.exact_coefficients = exact;
        // header (host plan) + entropy bytes into each caller's buffer
        for (size_t k = 0; k < live.size(); k++) {
            EncodeItem &it = items[live[k]];
            const std::vector<uint8_t> &hdr = plans[live[k]].header;
            const size_t total = hdr.size() + len[k];
            if (!it.out || total > it.out_capacity) {
                it.status = kInvalidArgument;
                it.message = "output buffer is smaller than the encoded frame";
                continue;
            }
            const cudaMemcpyKind up = it.out_on_device ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
            if (it.out_on_device) cudaMemcpyAsync(it.out, hdr.data(), hdr.size(), up, I.s);
            else memcpy(it.out, hdr.data(), hdr.size());
            cudaMemcpyAsync(it.out + hdr.size(), L.out + off[k], len[k],
                            it.out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, I.s);
            it.out_len = total;
            stats_.bytes_out += total;
        }
        cudaEventRecord(I.ev1, I.s);
        if (cudaStreamSynchronize(I.s) != cudaSuccess) throw std::runtime_error("GPU encoder: device failure");
        cudaEventElapsedTime(&stats_.device_ms, I.ev0, I.ev1);
    } catch (const std::exception &) {
        cudaGetLastError();
        for (size_t i : live) {
            items[i].status = kInternal;
            items[i].message = "CUDA device failure during encode";
            items[i].out_len = 0;
        }
        return kInternal;
    }
    return kOk;
}

}  // namespace mmr
