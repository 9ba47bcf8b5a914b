// Chunked, self-synchronising Huffman decode of baseline JPEG scans (sm_103a).
//
// The reference decodes a scan serially, one restart interval after another
// (crates/codecs/mjpeg/src/decoder.rs:313-410, 495-548; entropy.rs:57-182). A
// thread per interval leaves a GB300 nearly idle (135 intervals per 1080p frame,
// one per scan without DRI), so every interval is cut into fixed-size bit slices
// that decode in parallel. Huffman codes resynchronise: a decode started at a
// wrong bit or in a wrong coefficient state soon meets the true decode at a
// symbol boundary with the same state, and from there both are identical.
//
//   slice_plan     per frame: interval token ranges, slice counts, slot -> interval map
//   slice_spec     every slice decoded from a guessed state spec_lead(S) bits before it
//                  (the first slice from the true one) up to its end; keeps the state
//                  at eight checkpoints (64 .. 2048 bits into the slice) and stores
//                  the levels of the blocks it owns
//   slice_sync     (kSyncPasses passes; one after a pass that changed nothing returns
//                  at once) each slice whose start no longer equals its predecessor's
//                  exit state re-decodes from that state, two symbols per lookup where
//                  both end before the next checkpoint, until it meets one of its own
//                  checkpoints (then the rest is known) or its end
//   slice_fix      per interval, only when the last sync pass still changed a state:
//                  walks the slices in order until every start equals the previous
//                  exit. Then slice 0 starts in the true state and each exit is the
//                  true state at that point, so every start is the true one.
//   slice_prefix   per interval: block index and DC predictors at each slice start
//   slice_place    the owned blocks past each slice's match point placed (DC
//                  predictors, block map); the slots with short work listed
//   slice_decode   the final decode from true states of what was not placed: quantised
//                  AC levels, dequantised DC, and each slice's first event (an error,
//                  or the interval's last block completed)
//   slice_resolve  per interval: the earliest event in stream order becomes the
//                  interval's result, or the restart-marker check (entropy.rs:111-134)
//
// A slice owns the blocks whose DC symbol starts between its start state and its
// exit state; it decodes the block that straddles its end to completion, and skips
// (decodes without output) the one straddling its start. Errors are reported only
// by the owner of the block they occur in, so the earliest reported event is the
// one the serial decoder stops at.
#include <cuda_runtime.h>

#include <algorithm>

#include "entropy_core.h"
#include "kernels.h"
#include "tables.h"

namespace mmr {
namespace {

__constant__ uint8_t c_slice_zz[64] = MMR_ZIGZAG_INIT;

constexpr unsigned long long kStErr = ~0ull;        // no state: the decode failed before this point
constexpr unsigned long long kStGuess = ~0ull - 1;  // start not yet derived from the predecessor
constexpr int kSliceThreads = 128;
constexpr int kStride = 72;  // int16 per staged block (144 B: conflict-free 16 B rows)
constexpr int kKeyBits = 26;
#ifndef MMR_SPEC_CTAS_PER_SM
#define MMR_SPEC_CTAS_PER_SM 8
#endif

__device__ __forceinline__ unsigned long long pack_state(unsigned long long p, uint32_t si, uint32_t k) {
    return (p << 16) | (si << 8) | k;
}

// Tables of MCU block si.
struct BlockTabs {
    const HuffLut *dc;
    const HuffLut *ac;
    uint32_t comp;
};

__device__ __forceinline__ BlockTabs block_tabs(const JpegLaunch &L, const JFrame &F, uint32_t si) {
    const JBlockRec &R = L.brec[F.sched_off + si];
    BlockTabs t;
    t.comp = R.comp;
    t.dc = L.luts + R.dc_lut;
    t.ac = L.luts + R.ac_lut;
    return t;
}

// Bit offset of checkpoint q from the nominal slice start (UINT32_MAX past the slice).
__constant__ uint32_t c_slice_marks[kSliceCheckpoints] = {64, 128, 256, 512, 768, 1024, 1536, 2048};

__device__ __forceinline__ uint32_t mark_of(uint32_t q, uint32_t S) {
    const uint32_t m = q < (uint32_t)kSliceCheckpoints ? c_slice_marks[q] : 0xffffffffu;
    return m < S ? m : 0xffffffffu;
}

__device__ __forceinline__ void add_dc(int32_t (&dc)[4], uint32_t comp, int32_t v) {
#pragma unroll
    for (int c = 0; c < 4; c++)
        if (comp == (uint32_t)c) dc[c] += v;
}

__device__ __forceinline__ void add_dc_at(int32_t *dc, uint32_t comp, int32_t v) { dc[comp] += v; }

struct SliceRef {
    uint32_t item, j;
    IvInfo v;
    const JFrame *F;
    bool last;
};

__device__ __forceinline__ bool slice_ref(const JpegLaunch &L, uint32_t slot, SliceRef &s) {
    if (slot >= L.n_slots) return false;
    s.item = L.slot_item[slot];
    if (s.item == 0xffffffffu) return false;
    s.v = L.ivs[s.item];
    s.j = slot - s.v.slot_first;
    s.F = L.frames + L.items[s.item].x;
    s.last = s.j + 1 == s.v.n_slices;
    return true;
}

// Nominal start (bits from the interval's start) and length of a slice that is
// not its interval's last.
__device__ __forceinline__ void slice_span(const SliceRef &s, uint32_t S, unsigned long long &start, uint32_t &len) {
    start = (unsigned long long)s.j * S;
    len = S;
    if (s.v.tail && s.j + 2 == s.v.n_slices)  // the next is the split-off last slice
        len = (uint32_t)((unsigned long long)(s.v.barrier - s.v.start) * 8 - s.v.tail - start);
}

__device__ __forceinline__ uint32_t clamp_u32(unsigned long long x) {
    return x > 0xffffffffull ? 0xffffffffu : (uint32_t)x;
}

// ------------------------------------------------------------------ plan ---

__global__ void slice_plan_kernel(JpegLaunch L) {
    const uint32_t f = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const uint32_t lane = threadIdx.x & 31;
    if (f >= L.n_frames) return;
    const JFrame &F = L.frames[f];
    if (!F.decode || F.ncomp > 4) return;
    const JState &st = L.states[f];
    const unsigned long long termv = st.term;
    const bool scan_ok = termv != ~0ull && !((termv >> 8) & 1);
    const uint32_t n_int = F.n_intervals;
    const uint32_t n_rst = min(st.n_rst, n_int), n_tok = st.n_tokens;
    const RstEntry *rst = L.rsts + F.rst_off;
    const uint32_t S = F.slice_bits;
    uint32_t used = 0;
    for (uint32_t c = 0; c < n_int; c += 32) {
        const uint32_t iv = c + lane;
        uint32_t n_s = 0, start = 0, barrier = 0, flags = 0, blocks = 0, tail = 0;
        if (iv < n_int) {
            bool dec = scan_ok;
            if (iv == 0) start = 0;
            else if (iv - 1 < n_rst) start = rst[iv - 1].tok;
            else dec = false;  // no RST precedes it: an earlier interval fails its restart check
            if (dec) {
                flags = iv < n_rst ? 1u : 0u;
                barrier = flags ? rst[iv].tok : n_tok;
                const unsigned long long lbits = (unsigned long long)(barrier - start) * 8;
                n_s = (uint32_t)max(1ull, (lbits + S - 1) / S);
                if (lbits - (unsigned long long)(n_s - 1) * S > kSliceTail) {  // split the end off
                    n_s++;
                    tail = kSliceTail;
                }
                const uint32_t mcu0 = iv * F.ri, mcu1 = min(mcu0 + F.ri, F.total_mcus);
                blocks = (mcu1 - mcu0) * F.sched_len;
            }
        }
        uint32_t incl = n_s;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= (uint32_t)d) incl += o;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        uint32_t first = used + incl - n_s;
        if (used + total > F.slot_count) {  // cannot happen: slot_count bounds the token count
            n_s = 0;
            first = used;
        }
        if (iv < n_int) {
            IvInfo v;
            v.start = start;
            v.barrier = barrier;
            v.slot_first = F.slot_first + first;
            v.n_slices = n_s;
            v.blocks = blocks;
            v.flags = flags;
            v.tail = tail;
            v.pad = 0;
            L.ivs[F.item_base + iv] = v;
            L.iv_key[F.item_base + iv] = ~0ull;
        }
        for (uint32_t t = 0; t < 32 && c + t < n_int; t++) {
            const uint32_t nt = __shfl_sync(0xffffffffu, n_s, t), ft = __shfl_sync(0xffffffffu, first, t);
            for (uint32_t x = lane; x < nt; x += 32) L.slot_item[F.slot_first + ft + x] = F.item_base + c + t;
        }
        if (used + total <= F.slot_count) used += total;
    }
    for (uint32_t x = used + lane; x < F.slot_count; x += 32) L.slot_item[F.slot_first + x] = 0xffffffffu;
}

// ------------------------------------------------------ speculative pass ---

// Stores the staged block as owned block n of the slot (allocating a scratch
// chunk at each chunk's first block) and clears the stage; false when the slot's
// chunks or the arena are exhausted.
__device__ __forceinline__ bool store_owned(const JpegLaunch &L, uint32_t slot, uint32_t n, uint32_t &chunk_base,
                                            int4 *stage4, int32_t dc_diff) {
    const uint32_t c = n / kOwnChunkBlocks, i = n % kOwnChunkBlocks;
    if (i == 0) {
        if (c >= (uint32_t)kOwnChunks) return false;
        const unsigned long long first = atomicAdd(L.scratch_next, (unsigned long long)kOwnChunkBlocks);
        if (first + kOwnChunkBlocks > L.scratch_blocks) return false;
        chunk_base = (uint32_t)first;
        L.own[slot].chunk[c] = chunk_base;
    }
    int4 *dst = reinterpret_cast<int4 *>(L.scratch + (uint64_t)(chunk_base + i) * 64);
#pragma unroll
    for (int q = 0; q < 8; q++) {
        dst[q] = stage4[q];
        stage4[q] = make_int4(0, 0, 0, 0);
    }
    L.scratch_dc[chunk_base + i] = (int16_t)dc_diff;
    return true;
}

// Besides the exit state, checkpoints and counts, the speculative decode stores
// the levels of the blocks it owns along its own path (SliceOwn): blocks whose DC
// symbol starts at or past the slice start and before the slice end, the last
// one decoded to completion past the end.
// Table indices of MCU block si (fewer live registers than pointers).
struct TabIdx {
    uint32_t dc, ac, comp;
};

__device__ __forceinline__ TabIdx tab_idx(const JpegLaunch &L, const JFrame &F, uint32_t si) {
    const JBlockRec &R = L.brec[F.sched_off + si];
    return TabIdx{R.dc_lut, R.ac_lut, R.comp};
}

// 8 CTAs per SM (64 registers): the pass is latency-bound, so resident warps are
// what it runs on (at 9 it spills and runs slower)
__global__ void __launch_bounds__(kSliceThreads, MMR_SPEC_CTAS_PER_SM) slice_spec_kernel(JpegLaunch L) {
    __shared__ __align__(16) int16_t s_stage[kSliceThreads * kStride];
    __shared__ uint8_t s_zz[64];
    // per thread: DC sums per component, the scratch chunk and the end of the last
    // stored block, touched once per block (kept out of registers for occupancy)
    __shared__ int32_t s_dc[kSliceThreads][4];
    __shared__ uint32_t s_chunk[kSliceThreads], s_end[kSliceThreads];
    int16_t *stage = s_stage + threadIdx.x * kStride;
    int4 *stage4 = reinterpret_cast<int4 *>(stage);
#pragma unroll
    for (int q = 0; q < 8; q++) stage4[q] = make_int4(0, 0, 0, 0);
    if (threadIdx.x < 64) s_zz[threadIdx.x] = c_slice_zz[threadIdx.x];
    __syncthreads();
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    SliceRef s;
    if (!slice_ref(L, slot, s)) return;
    const bool guess = s.j != 0;
    SliceSync out;
    out.start = guess ? kStGuess : pack_state(0, 0, 0);
    out.exit = kStErr;
    out.blocks = 0;
    out.pad = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) out.dc[c] = 0;
    {
        SliceMatch m;  // a first slice starts true; the sync pass finds the others' point
        m.q = guess ? kMatchNone : kMatchStart;
        m.blocks = 0;
#pragma unroll
        for (int c = 0; c < 4; c++) m.dc[c] = 0;
        L.match[slot] = m;
    }
    if (s.last) {  // nothing reads the last slice's exit or counts; the decode pass redoes it
        L.sync[slot] = out;
        L.own[slot].n = 0;
        L.own[slot].ok = 0;
        return;
    }
    const JFrame &F = *s.F;
    unsigned long long nominal;
    uint32_t S;  // this slice's length
    slice_span(s, F.slice_bits, nominal, S);
    // a guessed decode starts up to spec_lead(S) bits early; positions below are from p0
    const uint32_t lead = guess ? (uint32_t)min((unsigned long long)spec_lead(F.slice_bits), nominal) : 0;
    const unsigned long long p0 = nominal - lead;
    const uint32_t end = S + lead;
    auto mark_at = [&](uint32_t qq) {
        const uint32_t m = mark_of(qq, S);
        return m == 0xffffffffu ? m : m + lead;
    };
    const unsigned long long lbits = (unsigned long long)(s.v.barrier - s.v.start) * 8;
    const uint32_t lim = clamp_u32(lbits - p0);  // bits before the barrier, from p0
    Bits r;
    bits_init(r, F.tok, (uint64_t)s.v.start * 8 + p0, 0);
    int k = guess ? 1 : 0;
    uint32_t si = 0;
    TabIdx tb = tab_idx(L, F, si);
    uint32_t blocks = 0;
    int32_t *dc = s_dc[threadIdx.x];
#pragma unroll
    for (int c = 0; c < 4; c++) dc[c] = 0;
    int32_t dcv = 0;  // DC difference of the block in progress (0 before its DC symbol)
    uint32_t q = 0, recorded = 0;
    uint32_t next_mark = guess ? mark_at(0) : 0xffffffffu;
    unsigned long long exit_state = kStErr;
    bool entered = false;  // at or past the slice start
    bool own_blk = false;  // the block in progress is owned
    bool own_ok = true;    // the owned blocks so far are stored
    uint32_t own_n = 0;
    uint32_t &chunk_base = s_chunk[threadIdx.x];
    uint32_t &own_end = s_end[threadIdx.x];  // position (from p0) after the last stored one
    chunk_base = 0;
    own_end = 0;
    for (;;) {
        const uint32_t pr = r.used;
        if (pr >= end) {
            exit_state = pack_state(p0 + pr, si, k);
            break;
        }
        entered |= pr >= lead;
        if (pr >= next_mark) {
            while (pr >= mark_at(q)) {
                SlicePoint cp;
                cp.state = pack_state(p0 + pr, si, k);
                cp.blocks = blocks;
                cp.own_next = own_n + (own_blk && k != 0 ? 1u : 0u);
#pragma unroll
                for (int c = 0; c < 4; c++) cp.dc[c] = dc[c] + (tb.comp == (uint32_t)c ? dcv : 0);
                L.spec[slot].cp[q] = cp;
                recorded |= 1u << q;
                q++;
            }
            next_mark = mark_at(q);
        }
        const int k0 = k;
        blocks += k0 == 0;
        own_blk = k0 == 0 ? entered : own_blk;
        int32_t val;
        uint16_t err;
        uint32_t eb;
        if (!decode_symbol(r, lim - pr, L.luts + (k0 == 0 ? tb.dc : tb.ac), L.symbols, k, val, err, eb)) {
            if (!guess || err == kBarrierErr) break;  // exit_state stays kStErr
            // A decode from a guessed state met an invalid symbol: start again one bit
            // later; what came before cannot lead to the exit, so its checkpoints go,
            // and the owned blocks start again too (this path was not the true one).
            for (uint32_t x = 0; x < (uint32_t)kSliceCheckpoints; x++)
                if (recorded & (1u << x)) L.spec[slot].cp[x].state = kStErr;
            recorded = 0;
            blocks = 0;
#pragma unroll
            for (int c = 0; c < 4; c++) dc[c] = 0;
            dcv = 0;
            k = 1;
            si = 0;
            tb = tab_idx(L, F, si);
            // (the stage may hold a partial block, or one whose store failed)
#pragma unroll
            for (int x = 0; x < 8; x++) stage4[x] = make_int4(0, 0, 0, 0);
            own_blk = false;
            own_ok = true;
            own_n = 0;
            bits_init(r, F.tok, (uint64_t)L.ivs[s.item].start * 8 + p0 + pr + 1, pr + 1);
            continue;
        }
        if (own_blk && own_ok) stage[s_zz[k - 1]] = (int16_t)val;
        dcv = k0 == 0 ? val : dcv;
        if (k < 64) continue;
        if (own_blk && own_ok) {  // block complete
            own_ok = store_owned(L, slot, own_n, chunk_base, stage4, dcv);
            own_n++;
            own_end = r.used;
        }
        own_blk = false;
        add_dc_at(dc, tb.comp, dcv);
        dcv = 0;
        k = 0;
        si = si + 1 == F.sched_len ? 0 : si + 1;
        tb = tab_idx(L, F, si);
    }
    // the owned block straddling the slice end is decoded to completion
    if (exit_state != kStErr && own_blk && own_ok) {
        while (k < 64) {
            int32_t val;
            uint16_t err;
            uint32_t eb;
            if (!decode_symbol(r, lim - r.used, L.luts + tb.ac, L.symbols, k, val, err, eb)) {
                own_ok = false;
                break;
            }
            stage[s_zz[k - 1]] = (int16_t)val;
        }
        if (own_ok) {
            own_ok = store_owned(L, slot, own_n, chunk_base, stage4, dcv);
            own_n++;
            own_end = r.used;
        }
    }
    SliceOwn *own = L.own + slot;
    own->last_end = p0 + own_end;
    own->n = own_n;
    own->ok = own_ok && exit_state != kStErr;
    add_dc_at(dc, tb.comp, dcv);  // the block in progress is counted, with its DC if decoded
    if (guess) {
        for (uint32_t x = 0; x < (uint32_t)kSliceCheckpoints; x++)
            if (!(recorded & (1u << x))) L.spec[slot].cp[x].state = kStErr;
        SlicePoint e;
        e.state = exit_state;
        e.blocks = blocks;
        e.own_next = own_n;
#pragma unroll
        for (int c = 0; c < 4; c++) e.dc[c] = dc[c];
        L.spec[slot].exit = e;
    }
    out.exit = exit_state;
    out.blocks = blocks;
#pragma unroll
    for (int c = 0; c < 4; c++) out.dc[c] = dc[c];
    L.sync[slot] = out;
}

// ------------------------------------------------------------ sync pass ---

// Re-decodes slice `slot` (not the first, not the last) from state `from`, the
// exit of its predecessor, until it meets one of the slice's speculative
// checkpoints or passes the slice end. Returns whether the exit state changed.
__device__ bool resync_slice(const JpegLaunch &L, uint32_t slot, const SliceRef &s, unsigned long long from) {
    SliceSync out;
    out.start = from;
    out.pad = 0;
    out.blocks = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) out.dc[c] = 0;
    const unsigned long long old_exit = L.sync[slot].exit;
    SliceMatch m;
    m.q = kMatchNone;
    m.blocks = 0;
#pragma unroll
    for (int c = 0; c < 4; c++) m.dc[c] = 0;
    if (from == kStErr) {
        out.exit = kStErr;
        L.sync[slot] = out;
        L.match[slot] = m;
        return old_exit != kStErr;
    }
    const JFrame &F = *s.F;
    unsigned long long nominal;
    uint32_t S;  // this slice's length
    slice_span(s, F.slice_bits, nominal, S);
    const unsigned long long p0 = from >> 16;
    const uint32_t rel = (uint32_t)(p0 - nominal);  // < one symbol: from is the first boundary past nominal
    const unsigned long long lbits = (unsigned long long)(s.v.barrier - s.v.start) * 8;
    const uint32_t lim = clamp_u32(lbits - p0);
    Bits r;
    bits_init(r, F.tok, (uint64_t)s.v.start * 8 + p0, 0);
    int k = (int)(from & 0xff);
    uint32_t si = (uint32_t)(from >> 8) & 0xff;
    BlockTabs tb = block_tabs(L, F, si);
    uint32_t blocks = 0;
    int32_t dc[4] = {0, 0, 0, 0};
    int32_t dcv = 0;
    const SliceSpec *sp = L.spec + slot;
    uint32_t q = 0;
    while (mark_of(q, S) <= rel) q++;  // marks already behind
    uint32_t next_mark = mark_of(q, S);
    unsigned long long exit_state = kStErr;
    for (;;) {
        const uint32_t pr = r.used;
        const uint32_t pn = pr + rel;  // position from the nominal slice start
        if (pn >= S) {
            exit_state = pack_state(p0 + pr, si, k);
            break;
        }
        if (pn >= next_mark) {
            bool matched = false;
            while (pn >= mark_of(q, S)) {
                const unsigned long long cs = sp->cp[q].state;
                if (cs != kStErr && cs == pack_state(p0 + pr, si, k)) {
                    // the rest of the slice is the speculative decode's: take its tail
                    const SlicePoint cp = sp->cp[q], e = sp->exit;
                    exit_state = e.state;
                    add_dc(dc, tb.comp, dcv);
                    dcv = 0;
                    m.q = q;  // the true decode so far, where it meets the speculative one
                    m.blocks = blocks;
#pragma unroll
                    for (int c = 0; c < 4; c++) m.dc[c] = dc[c];
                    blocks += e.blocks - cp.blocks;
#pragma unroll
                    for (int c = 0; c < 4; c++) dc[c] += e.dc[c] - cp.dc[c];
                    matched = true;
                    break;
                }
                q++;
            }
            if (matched) break;
            next_mark = mark_of(q, S);
        }
        const int k0 = k;
        blocks += k0 == 0;
        int32_t val, val2;
        int km;
        uint16_t err;
        uint32_t eb;
        // two symbols per lookup where both end before the next checkpoint or the
        // slice end (the speculative decode's boundaries there are one-symbol ones)
        const uint32_t stop = min(next_mark, S) - pn;
        if (!decode_step(r, lim - pr, stop, k0 == 0 ? tb.dc : tb.ac, L.symbols, k, val, val2, km, err, eb)) break;
        dcv = k0 == 0 ? val : dcv;
        if (k < 64) continue;
        add_dc(dc, tb.comp, dcv);
        dcv = 0;
        k = 0;
        si = si + 1 == F.sched_len ? 0 : si + 1;
        tb = block_tabs(L, F, si);
    }
    add_dc(dc, tb.comp, dcv);
    out.exit = exit_state;
    out.blocks = blocks;
#pragma unroll
    for (int c = 0; c < 4; c++) out.dc[c] = dc[c];
    L.sync[slot] = out;
    L.match[slot] = m;
    return exit_state != old_exit;
}

// Persistent threads take slots from a counter: re-decode lengths vary a lot
// (most slices meet their first checkpoint, a few run to their end), so a lane
// that is done takes the next slot instead of idling beside the slow ones. The
// lanes that reach the counter together take consecutive slots with one atomic
// (one per slot serialised on the counter's address).
__global__ void __launch_bounds__(kSliceThreads) slice_sync_kernel(JpegLaunch L, uint32_t pass) {
    // a pass after one that changed no exit state has nothing to do: every start
    // then equals its predecessor's exit
    if (pass > 0 && *(volatile const uint32_t *)&L.sync_dirty[pass - 1] == 0) return;
    uint32_t *next = L.sync_dirty + kSyncPasses + pass;
    const uint32_t lane = threadIdx.x & 31;
    for (;;) {
        const unsigned act = __activemask();
        const int leader = __ffs(act) - 1;
        uint32_t base = 0;
        if ((int)lane == leader) base = atomicAdd(next, (uint32_t)__popc(act));
        base = __shfl_sync(act, base, leader);
        const uint32_t slot = base + __popc(act & ((1u << lane) - 1u));
        if (slot >= L.n_slots) return;
        SliceRef s;
        if (!slice_ref(L, slot, s) || s.j == 0) continue;
        const unsigned long long prev = *(volatile const unsigned long long *)&L.sync[slot - 1].exit;
        const unsigned long long cur = L.sync[slot].start;
        if (prev == cur) continue;
        if (s.last) {
            L.sync[slot].start = prev;
            continue;
        }
        if (resync_slice(L, slot, s, prev)) atomicAdd(&L.sync_dirty[pass], 1u);
    }
}

// One warp per interval; runs only when the last sync pass still changed an exit state.
__global__ void slice_fix_kernel(JpegLaunch L) {
    if (*(volatile uint32_t *)&L.sync_dirty[kSyncPasses - 1] == 0) return;
    const uint32_t item = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const uint32_t lane = threadIdx.x & 31;
    if (item >= L.n_items_small) return;
    const IvInfo v = L.ivs[item];
    for (uint32_t c = 1; c < v.n_slices; c += 32) {
        for (;;) {
            const uint32_t j = c + lane;
            bool bad = false;
            if (j < v.n_slices) {
                const uint32_t slot = v.slot_first + j;
                bad = *(volatile unsigned long long *)&L.sync[slot].start !=
                      *(volatile unsigned long long *)&L.sync[slot - 1].exit;
            }
            const uint32_t m = __ballot_sync(0xffffffffu, bad);
            if (!m) break;
            const uint32_t first = __ffs(m) - 1;
            if (lane == first) {
                const uint32_t slot = v.slot_first + j;
                SliceRef s;
                slice_ref(L, slot, s);
                const unsigned long long prev = *(volatile unsigned long long *)&L.sync[slot - 1].exit;
                if (s.last) L.sync[slot].start = prev;
                else resync_slice(L, slot, s, prev);
                __threadfence_block();
            }
            __syncwarp();
        }
    }
}

// ---------------------------------------------------------------- prefix ---

__global__ void slice_prefix_kernel(JpegLaunch L) {
    const uint32_t item = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const uint32_t lane = threadIdx.x & 31;
    if (item >= L.n_items_small) return;
    const IvInfo v = L.ivs[item];
    uint32_t carry_b = 0;
    long long carry_d[4] = {0, 0, 0, 0};
    for (uint32_t c = 0; c < v.n_slices; c += 32) {
        const uint32_t j = c + lane;
        uint32_t b = 0;
        long long d[4] = {0, 0, 0, 0};
        if (j + 1 < v.n_slices) {  // the last slice's counts are never needed
            const SliceSync &y = L.sync[v.slot_first + j];
            b = y.blocks;
#pragma unroll
            for (int q = 0; q < 4; q++) d[q] = y.dc[q];
        }
        uint32_t ib = b;
        long long id[4] = {d[0], d[1], d[2], d[3]};
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t tb = __shfl_up_sync(0xffffffffu, ib, o);
            long long td[4];
#pragma unroll
            for (int q = 0; q < 4; q++) td[q] = __shfl_up_sync(0xffffffffu, id[q], o);
            if (lane >= (uint32_t)o) {
                ib += tb;
#pragma unroll
                for (int q = 0; q < 4; q++) id[q] += td[q];
            }
        }
        if (j < v.n_slices) {
            SlicePrefix P;
            P.base = carry_b + ib - b;
            P.pad = 0;
#pragma unroll
            for (int q = 0; q < 4; q++) P.dc[q] = carry_d[q] + id[q] - d[q];
            L.prefix[v.slot_first + j] = P;
        }
        carry_b += __shfl_sync(0xffffffffu, ib, 31);
#pragma unroll
        for (int q = 0; q < 4; q++) carry_d[q] += __shfl_sync(0xffffffffu, id[q], 31);
    }
}

// ----------------------------------------------------------------- place ---

// Records a slice's first event: an error, or the interval's completion.
__device__ __forceinline__ void report(const JpegLaunch &L, const SliceRef &s, uint32_t slot, unsigned long long pos,
                                       const Diag &d, uint32_t complete) {
    SliceEvent e;
    e.diag = d;
    e.complete = complete;
    L.events[slot] = e;
    atomicMin(&L.iv_key[s.item], (pos << kKeyBits) | s.j);
}


// A thread per slice. The owned blocks that start after the point where the
// slice's true decode met its speculative decode (SliceMatch) are final: their
// DC predictors are settled as the final decode would (decoder.rs:507-515) and
// the block map points at their levels. The final decode pass writes the blocks
// before that point, and the whole slice when there is no such point, anything
// failed, or it is the interval's last slice
// (its decode reports the interval's completion; a placed last block reports it
// here). A DC overflow among the placed blocks also sends the whole slice there
// (reported with its position). Returns the final decode pass's work in the
// slice: the leading blocks it writes (0: none, UINT32_MAX: all).
__device__ uint32_t place_slice(const JpegLaunch &L, uint32_t slot, const SliceRef &s) {
    const SliceSync y = L.sync[slot];
    if (y.start == kStErr || y.start == kStGuess) return 0;  // not reached: nothing to decode
    const SlicePrefix P = L.prefix[slot];
    const uint32_t B = s.v.blocks;
    if (P.base >= B) return 0;
    const uint32_t nown = s.last ? B - P.base : min(y.blocks, B - P.base);
    if (nown == 0) return 0;
    const SliceOwn *O = L.own + slot;
    const SliceMatch M = L.match[slot];
    uint32_t spec_first = 0;
    bool usable = !s.last && O->ok && M.q != kMatchNone && M.blocks <= nown;
    if (usable && M.q != kMatchStart) spec_first = L.spec[slot].cp[M.q].own_next;
    usable = usable && spec_first <= O->n && O->n - spec_first == nown - M.blocks;
    if (usable && M.blocks < nown) {
        const JFrame &F = *s.F;
        const uint32_t sched_len = F.sched_len, mcu_cols = F.mcu_cols;
        const uint32_t b0 = P.base + M.blocks;  // interval-relative block of the first placed one
        const uint32_t mcu = L.items[s.item].y * F.ri + b0 / sched_len;
        uint32_t mx = mcu % mcu_cols, my = mcu / mcu_cols, si = b0 % sched_len;
        const JBlockRec *recs = L.brec + F.sched_off;
        long long pred[4];
#pragma unroll
        for (int c = 0; c < 4; c++) pred[c] = P.dc[c] + M.dc[c];
        for (uint32_t i = 0; i < nown - M.blocks; i++) {
            const JBlockRec R = recs[si];
            const uint64_t blk = F.blk_off + R.base_off + mx * R.mul_x + (uint64_t)my * R.mul_y;
            const uint32_t own_i = spec_first + i;
            const uint32_t sb = O->chunk[own_i / kOwnChunkBlocks] + own_i % kOwnChunkBlocks;
            long long pc = 0;
#pragma unroll
            for (int c = 0; c < 4; c++)
                if (R.comp == (uint32_t)c) pc = pred[c];
            const long long pn = pc + L.scratch_dc[sb];
            const long long d = pn * (long long)R.q0;
            if (pn > INT32_MAX || pn < INT32_MIN || d > INT32_MAX || d < INT32_MIN) {
                usable = false;
                break;
            }
#pragma unroll
            for (int c = 0; c < 4; c++)
                if (R.comp == (uint32_t)c) pred[c] = pn;
            L.dc[blk] = (int32_t)d;
            L.blk_map[blk] = sb;
            if (++si == sched_len) {
                si = 0;
                if (++mx == mcu_cols) {
                    mx = 0;
                    my++;
                }
            }
        }
    }
    if (usable && M.blocks < nown && P.base + nown == B) {  // the interval's last block, placed
        const unsigned long long endbit = O->last_end;
        report(L, s, slot, endbit, make_diag(kDiagNone, s.v.start + (uint32_t)((endbit + 7) / 8)), 1);
    }
    const uint32_t redo = usable ? M.blocks : 0xffffffffu;
    L.redo[slot] = redo;
    return redo;
}

// Adds the lanes' flags to a counter, one atomic per warp.
__device__ __forceinline__ void count_lanes(uint32_t *counter, bool flag) {
    const uint32_t m = __ballot_sync(0xffffffffu, flag);
    if ((threadIdx.x & 31) == 0 && m) atomicAdd(counter, (uint32_t)__popc(m));
}

// Also lists the slots with short work for the final decode (leading blocks, or an
// interval's last slice, at most kSliceTail bits), so that its warps take those
// tasks packed and lanes without work do not ride along. Whole slices redone from
// their start stay in slot order: few and long, they run best spread over the
// warps (a packed warp of them waits on 32 lanes' loads per step).
__global__ void __launch_bounds__(kSliceThreads) slice_place_kernel(JpegLaunch L) {
    const uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    SliceRef s;
    const bool valid = slice_ref(L, slot, s);
    count_lanes(L.fix_count + 3, valid);
    uint32_t redo = 0;
    if (valid) redo = place_slice(L, slot, s);
    count_lanes(L.fix_count + 2, redo != 0);
    count_lanes(L.fix_count + 5, redo == 0xffffffffu);
    const uint32_t lane = threadIdx.x & 31;
    const unsigned shrt = __ballot_sync(0xffffffffu, redo != 0 && (redo != 0xffffffffu || s.last));
    uint32_t base = 0;
    if (lane == 0 && shrt) base = atomicAdd(L.fix_count + 4, (uint32_t)__popc(shrt));
    base = __shfl_sync(0xffffffffu, base, 0);
    if (shrt & (1u << lane)) L.work[base + __popc(shrt & ((1u << lane) - 1u))] = slot;
}


// ---------------------------------------------------------------- decode ---


__global__ void __launch_bounds__(kSliceThreads) slice_decode_kernel(JpegLaunch L) {
    __shared__ __align__(16) int16_t s_stage[kSliceThreads * kStride];
    __shared__ uint8_t s_zz[64];  // lanes index it freely: a shared table serves them in one pass
    int16_t *stage = s_stage + threadIdx.x * kStride;
    int4 *stage4 = reinterpret_cast<int4 *>(stage);
#pragma unroll
    for (int q = 0; q < 8; q++) stage4[q] = make_int4(0, 0, 0, 0);
    if (threadIdx.x < 64) s_zz[threadIdx.x] = c_slice_zz[threadIdx.x];
    __syncthreads();
    // The first half of the grid takes the short tasks, packed from the work list
    // (slice_place_kernel); the second half the whole slices redone from their
    // start, in slot order.
    const uint32_t half = gridDim.x >> 1;
    uint32_t slot;
    if (blockIdx.x < half) {
        const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
        if (t >= L.fix_count[4]) return;
        slot = L.work[t];
    } else {
        slot = (blockIdx.x - half) * blockDim.x + threadIdx.x;
    }
    SliceRef s;
    if (!slice_ref(L, slot, s)) return;
    const uint32_t redo = L.redo[slot];  // leading blocks to write; the rest are placed
    if (!redo || (blockIdx.x >= half && (redo != 0xffffffffu || s.last))) return;
    const unsigned long long from = L.sync[slot].start;
    if (from == kStErr || from == kStGuess) return;
    const SlicePrefix P = L.prefix[slot];
    const uint32_t B = s.v.blocks;
    if (P.base >= B) return;
    const uint32_t nown = min(s.last ? B - P.base : min(L.sync[slot].blocks, B - P.base), redo);
    if (nown == 0) return;
    const JFrame &F = *s.F;
    const uint32_t iv = L.items[s.item].y;
    const unsigned long long p0 = from >> 16;
    const unsigned long long lbits = (unsigned long long)(s.v.barrier - s.v.start) * 8;
    const uint32_t lim = clamp_u32(lbits - p0);
    const uint32_t sched_len = F.sched_len;
    Bits r;
    bits_init(r, F.tok, (uint64_t)s.v.start * 8 + p0, 0);
    int k = (int)(from & 0xff);
    uint32_t si = (uint32_t)(from >> 8) & 0xff;
    int32_t val;
    uint16_t err;
    uint32_t eb;
    if (k != 0) {  // the block straddling the start belongs to an earlier slice
        const HuffLut *acl = block_tabs(L, F, si).ac;
        while (k < 64)
            if (!decode_symbol(r, lim - r.used, acl, L.symbols, k, val, err, eb)) return;
        si = si + 1 == sched_len ? 0 : si + 1;
        k = 0;
    }
    long long pred[4];
#pragma unroll
    for (int c = 0; c < 4; c++) pred[c] = P.dc[c];
    // MCU of the first owned block, then advanced block by block
    const uint32_t mcu = iv * F.ri + P.base / sched_len;
    const uint32_t mcu_cols = F.mcu_cols;
    uint32_t mx = mcu % mcu_cols, my = mcu / mcu_cols;
    uint32_t b = P.base;
    const uint32_t bend = P.base + nown;
    const HuffLut *dcl, *acl;
    uint64_t blk;
    int32_t q0;
    uint32_t comp;
    const JBlockRec *recs = L.brec + F.sched_off;
    auto setup = [&]() {
        const JBlockRec R = recs[si];
        comp = R.comp;
        dcl = L.luts + R.dc_lut;
        acl = L.luts + R.ac_lut;
        blk = F.blk_off + R.base_off + mx * R.mul_x + (uint64_t)my * R.mul_y;
        q0 = R.q0;
    };
    setup();
    // The DC difference is staged at zigzag index 0 like a level and turned into the
    // dequantised DC when the block completes; an error inside the block first
    // settles the DC checks the reference makes right after the DC symbol.
    uint32_t blk_at = r.used;  // start of the block's DC symbol
    uint32_t dc_end = 0;       // reader position after the DC difference
    for (;;) {
        const uint32_t sym_at = r.used;
        const int k0 = k;
        const bool ok = decode_symbol(r, lim - sym_at, k0 == 0 ? dcl : acl, L.symbols, k, val, err, eb);
        if (ok) {
            stage[s_zz[k - 1]] = (int16_t)val;
            dc_end = k0 == 0 ? r.used : dc_end;
            if (k < 64) continue;
        }
        // block complete, or an error: the block's DC checks (decoder.rs:507-515) first
        uint16_t kind = kDiagNone;
        uint32_t errpos = 0, ev_at = sym_at;
        int32_t dq = 0;
        if (ok || k0 > 0) {
            long long pc = 0;
#pragma unroll
            for (int c = 0; c < 4; c++)
                if (comp == (uint32_t)c) pc = pred[c];
            const long long pn = pc + stage[0];
            if (pn > INT32_MAX || pn < INT32_MIN) {
                kind = kJDcPredOverflow;
                errpos = dc_end;
                ev_at = blk_at;
            } else {
#pragma unroll
                for (int c = 0; c < 4; c++)
                    if (comp == (uint32_t)c) pred[c] = pn;
                const long long d = pn * (long long)q0;
                if (d > INT32_MAX || d < INT32_MIN) {
                    kind = kJDcDeqOverflow;
                    errpos = dc_end;
                    ev_at = blk_at;
                }
                dq = (int32_t)d;
            }
        }
        if (kind == kDiagNone && !ok) {
            kind = err;
            errpos = eb;
        }
        if (kind != kDiagNone) {
            Diag d;
            if (kind == kBarrierErr) {
                d = (s.v.flags & 1)
                        ? make_diag(kJMarkerInData, s.v.barrier, 0xd0 + L.rsts[F.rst_off + iv].number)
                        : make_diag(kJEndOfData, L.states[L.items[s.item].x].n_tokens);
            } else {
                d = make_diag(kind, s.v.start + (uint32_t)((p0 + errpos + 7) / 8));
            }
            report(L, s, slot, p0 + ev_at, d, 0);
            return;
        }
        int4 *dst = reinterpret_cast<int4 *>(L.coef + blk * 64);
#pragma unroll
        for (int q = 0; q < 8; q++) {
            dst[q] = stage4[q];
            stage4[q] = make_int4(0, 0, 0, 0);
        }
        L.dc[blk] = dq;
        L.blk_map[blk] = kLevelsInPlace;  // (place may have mapped the first blocks before an overflow)
        if (b + 1 == B) {
            const unsigned long long endbit = p0 + r.used;
            report(L, s, slot, endbit, make_diag(kDiagNone, s.v.start + (uint32_t)((endbit + 7) / 8)), 1);
            return;
        }
        if (++b == bend) return;
        if (++si == sched_len) {
            si = 0;
            if (++mx == mcu_cols) {
                mx = 0;
                my++;
            }
        }
        setup();
        k = 0;
        blk_at = r.used;
    }
}

// --------------------------------------------------------------- resolve ---

__global__ void slice_resolve_kernel(JpegLaunch L) {
    const uint32_t item = blockIdx.x * blockDim.x + threadIdx.x;
    if (item >= L.n_items_small) return;
    const IvInfo v = L.ivs[item];
    if (v.n_slices == 0) return;
    const uint2 it = L.items[item];
    const JFrame &F = L.frames[it.x];
    JState *st = L.states + it.x;
    const uint32_t iv = it.y;
    const unsigned long long key = L.iv_key[item];
    Diag out = make_diag(kDiagNone);
    if (key == ~0ull) {
        out = make_diag(kDeviceError);  // every decoded interval ends in an event
    } else {
        const SliceEvent e = L.events[v.slot_first + (uint32_t)(key & ((1u << kKeyBits) - 1))];
        if (!e.complete) {
            out = e.diag;
        } else if (iv + 1 < F.n_intervals) {
            // consume_restart before the next interval (entropy.rs:111-134)
            const uint32_t tend = e.diag.offset, expected = iv & 7, n_tok = st->n_tokens;
            const RstEntry *rst = L.rsts + F.rst_off;
            if ((v.flags & 1) && rst[iv].tok == tend) {
                if (rst[iv].number != expected) out = make_diag(kJRstMismatch, tend, expected, 0xd0 + rst[iv].number);
            } else if (tend < n_tok && F.tok[tend] == 0xff) {
                out = make_diag(kJRstMismatch, tend, expected, 0x00);
            } else {
                out = make_diag(kJExpectRst, tend);
            }
        }
    }
    L.results[item] = out;
    if (out.kind != kDiagNone) atomicMin(&st->bad_interval, iv);
}

}  // namespace

int jpeg_slice_launches(const JpegLaunch &L) { return L.n_items_small ? 7 + kSyncPasses : 0; }

void launch_jpeg_slices(const JpegLaunch &L, cudaStream_t s, cudaEvent_t *marks, bool capturing) {
    auto mark = [&](int k) {
        if (marks) capturing ? cudaEventRecordWithFlags(marks[k], s, cudaEventRecordExternal) : cudaEventRecord(marks[k], s);
    };
    const bool run = L.n_items_small && L.n_slots;
    const uint32_t warps_per_cta = 4;
    const uint32_t grid = (L.n_slots + kSliceThreads - 1) / kSliceThreads;
    const uint32_t ivgrid = (L.n_items_small + warps_per_cta - 1) / warps_per_cta;
    if (run) {
        slice_plan_kernel<<<(L.n_frames + warps_per_cta - 1) / warps_per_cta, 32 * warps_per_cta, 0, s>>>(L);
        slice_spec_kernel<<<grid, kSliceThreads, 0, s>>>(L);
    }
    mark(0);
    if (run) {
        const uint32_t sync_grid = std::min<uint32_t>(grid, 152 * 8);
        for (uint32_t p = 0; p < (uint32_t)kSyncPasses; p++) slice_sync_kernel<<<sync_grid, kSliceThreads, 0, s>>>(L, p);
        slice_fix_kernel<<<ivgrid, 32 * warps_per_cta, 0, s>>>(L);
        slice_prefix_kernel<<<ivgrid, 32 * warps_per_cta, 0, s>>>(L);
    }
    mark(1);
    if (run) {
        slice_place_kernel<<<grid, kSliceThreads, 0, s>>>(L);
        slice_decode_kernel<<<2 * grid, kSliceThreads, 0, s>>>(L);
    }
    mark(2);
    if (run) slice_resolve_kernel<<<(L.n_items_small + 127) / 128, 128, 0, s>>>(L);
}

}  // namespace mmr
