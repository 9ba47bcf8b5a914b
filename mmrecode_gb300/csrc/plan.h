// Device-visible plan records for one decode batch (host builds, kernels read).
#pragma once

#include "common.h"

namespace mmr {

// ---------------------------------------------------------------- MJPEG ----

// Canonical-Huffman lookup for one DHT table (crates/codecs/mjpeg/src/entropy.rs:18-70).
// fast[] resolves every code of length <= 9 from the next 9 bits; longer codes use
// maxcode/valptr (JPEG Annex F.2.2.3), which for canonical codes finds the same
// code as the reference's length-by-length search.
constexpr int kHuffFastBits = 11;
constexpr uint32_t kFastEob = 1u << 12;
constexpr uint32_t kFastCode = 1u << 13;
constexpr uint32_t kFastPair = kFastEob | kFastCode;  // (no single entry has both)

struct HuffLut {
    uint16_t fast[512];    // (length << 8) | symbol; 0 when the code is longer than 9 bits or absent
    // Whole symbols within the next 11 bits: value << 16 | eob << 12 | advance << 5 |
    // total bits (code + magnitude). advance moves the coefficient index k: 1 for a
    // DC difference (size 0..11), run + 1 for an AC level (size 1..10), 16 for ZRL;
    // EOB sets k to 64. Codes of at most 11 bits whose magnitude bits reach past
    // them: size << 16 | kFastCode | advance << 5 | code length (the magnitude is
    // read from the bits after the code). 0: slow path (codes longer than 11 bits,
    // and every symbol the reference rejects).
    uint32_t fastv[1 << kHuffFastBits];
    // fastv with two AC symbols in one entry where both lie whole within the next
    // 11 bits, the first not EOB, with levels in -64..63 and -32..31:
    //   level2 << 26 | level1 << 19 | advance2 << 14 | kFastPair | advance1 << 5 | total bits
    // (advance2 0: the second is EOB). The same as fastv for DC tables.
    uint32_t fastp[1 << kHuffFastBits];
    int32_t maxcode[18];   // largest code of each length 1..16, -1 if none
    int32_t valptr[18];    // symbol index of a length's first code, minus that code
    uint32_t sym_off;      // first symbol in the symbol pool
    uint32_t nsym;
    uint32_t pad[2];       // size multiple of 16
};

// One frame component (SOF0 order).
struct JComp {
    uint32_t plane_w, plane_h;  // visible samples (decoder.rs:440-445)
    uint32_t bw, bh;            // block grid covered by the MCUs
    uint32_t blk_base;          // frame-relative index of block (0,0)
    uint32_t out_off;           // offset of this plane in the frame's planar buffer
    uint8_t h, v, q, pad;       // sampling factors and quantisation slot
    uint32_t pad2;
};

// One block of an MCU, in the scan's component order (decoder.rs:374-400).
struct JSched {
    uint16_t comp;   // frame component index
    uint8_t bx, by;  // block position inside the MCU
    uint8_t dc, ac;  // Huffman table slots
    uint8_t pad[2];
};

// Everything the entropy decoders need for one MCU block position, in one
// 32-byte record (parallel to the schedule): lookups, DC quantiser, and the
// block index of MCU (mx, my) as base_off + mx * mul_x + my * mul_y.
struct JBlockRec {
    uint32_t dc_lut, ac_lut;
    uint32_t base_off;  // frame-relative block of MCU (0, 0)
    uint32_t mul_y;
    uint32_t mul_x;
    uint32_t comp;      // frame component (scan components = frame components)
    int32_t q0;         // DC quantiser
    uint32_t pad;
};

struct JFrame {
    const uint8_t *in;      // packet (device)
    uint8_t *tok;           // unstuffed entropy-coded bytes (device), capacity in_len
    uint8_t *planes;        // planar samples (device): the output itself, or scratch for RGB output
    uint32_t in_len;
    uint32_t data_start;    // first entropy-coded byte
    uint32_t width, height;
    uint32_t ncomp, interleaved;
    uint32_t mcu_cols, mcu_rows, total_mcus;
    uint32_t ri;            // MCUs per restart interval (total_mcus when there is no DRI)
    uint32_t n_intervals;
    uint32_t item_base;     // first (frame, interval) work item
    uint32_t sched_off, sched_len;
    uint32_t comp_off;
    uint32_t lut[8];        // HuffLut index of DC 0..3 then AC 0..3; UINT32_MAX when undefined
    uint32_t quant_off;     // 4 tables x 64 entries, natural order
    uint32_t rst_off;       // restart table (capacity n_intervals)
    uint32_t tile_first;    // first marker-scan tile
    uint32_t decode;        // 0: the header already failed; only the marker scan runs
    uint64_t blk_off;       // first block in the coefficient arena
    uint32_t n_blocks;
    uint32_t item;          // caller's batch item
    uint32_t slot_first;    // first slice slot of the chunked entropy decoder
    uint32_t slot_count;    // slots reserved: ceil(8 * in_len / slice_bits) + 2 * n_intervals
    uint32_t slice_bits;    // bits per slice (multiple of 32, >= 128)
    uint32_t pad;
};

// --------------------------------------------- chunked entropy decoding ----
//
// A decoder state is packed as (bit position << 16) | (MCU block index << 8) | k,
// the bit position counted from the interval's first entropy-coded token and k
// the zigzag index of the next coefficient (0: the DC symbol comes next).

// One restart interval (the whole scan without DRI) of a frame with <= 4 components.
struct IvInfo {
    uint32_t start;       // first token
    uint32_t barrier;     // tokens before the RST marker (or the end of the scan) that ends it
    uint32_t slot_first;  // first slice slot
    uint32_t n_slices;    // 0: not decoded (header failure, or no RST precedes it)
    uint32_t blocks;      // coefficient blocks in the interval
    uint32_t flags;       // bit 0: the barrier is an RST marker
    uint32_t tail;        // bits of the last slice when the interval's end was split off (else 0)
    uint32_t pad;
};

// Slices are slice_bits long from the interval's start, except that the last one
// is at most kSliceTail bits: when the remainder is longer, its end is split off
// as an extra slice (the final decode pass redoes every last slice in full).
constexpr uint32_t kSliceTail = 256;

// Per slice: the state its decode starts from and what that decode produced.
struct SliceSync {
    unsigned long long start;  // start state (guess marker before the first sync pass)
    unsigned long long exit;   // state at the first symbol boundary at or past the slice end
    uint32_t blocks;           // blocks whose DC symbol starts in [start, exit)
    int32_t dc[4];             // sum of their DC differences, per scan component
    uint32_t pad;
};

// A point of the speculative decode: its state and the counts accumulated before
// it, and the index among its owned blocks (SliceOwn) of the first block that
// starts at or after it.
struct SlicePoint {
    unsigned long long state;
    uint32_t blocks;
    int32_t dc[4];
    uint32_t own_next;
};

// Checkpoints 64, 128, 256, 512, 768, 1024, 1536 and 2048 bits into a slice
// (those inside it). The speculative decode of a slice starts spec_lead(S) bits
// before the slice: the synchronisation distance of Huffman-coded JPEG data is a
// few hundred bits (longer where the MCU's block phase must also fall into
// place), so it has usually met the true decode by the first checkpoint, and a
// re-decode from the predecessor's exit matches there after a few symbols; the
// later ones bound how far the final decode pass must redo a slice whose
// speculative decode met the true one late. Short slices take a longer lead
// relative to their length: their sync passes and serial fix-up cost more than
// the extra decoding (measured: 1024-bit slices of 4:2:0 VGA frames 512 -> 1024
// -> 1536 bits, 1.29 -> 1.14 -> 1.13 ms per 30 frames, 2048 bits no better;
// 4096-bit slices of 4:2:2 1080p frames 512 -> 768 bits, 5.71 -> 5.68 ms of
// entropy decode per 300 frames).
constexpr int kSliceCheckpoints = 8;
MMR_HD constexpr uint32_t spec_lead(uint32_t slice_bits) { return slice_bits <= 1024 ? 1536u : slice_bits <= 2048 ? 1024u : 768u; }

struct SliceSpec {
    SlicePoint exit;                      // end of the speculative decode
    SlicePoint cp[kSliceCheckpoints];     // state at the first symbol boundary past each mark
};

// The levels of the blocks a speculative decode owns along its own path (the
// blocks whose DC symbol starts in [slice start, slice end), counted from its
// last restart), written to a scratch arena in chunks of kOwnChunkBlocks while
// the decode runs. Where the true decode of the slice meets the speculative one
// (at the slice start for a slice's first slice, else at the checkpoint the sync
// pass matched), every owned block that starts after that point is final; the
// final decode pass writes only the blocks before it (all of them when there is
// no such point, or anything went wrong).
constexpr uint32_t kOwnChunkBlocks = 16;
constexpr int kOwnChunks = 16;
constexpr uint32_t kLevelsInPlace = 0xffffffffu;  // block map: levels in the coefficient arena

struct SliceOwn {
    unsigned long long last_end; // bit position (from the interval's start) after the last one
    uint32_t n;                  // owned blocks written
    uint32_t ok;                 // 1: all n are complete, error-free and stored
    uint32_t chunk[kOwnChunks];  // first scratch block of each chunk
};

// Where the true decode of a slice met its speculative decode.
constexpr uint32_t kMatchNone = 0xffffffffu;
constexpr uint32_t kMatchStart = 0xfffffffeu;  // a first slice: the speculative decode is the true one
struct SliceMatch {
    uint32_t q;        // checkpoint index, kMatchStart, or kMatchNone
    uint32_t blocks;   // true blocks started before the point (counting the one in progress)
    int32_t dc[4];     // their DC differences, per scan component
};

// Block index and DC predictors at a slice's start (interval-relative).
struct SlicePrefix {
    uint32_t base;
    uint32_t pad;
    long long dc[4];
};

// The first event of a slice's final decode: an error, or the interval's last block done.
struct SliceEvent {
    Diag diag;          // error; for completion, offset = tokens consumed by the interval
    uint32_t complete;
};

// Written by the kernels, copied back to the host.
struct JState {
    unsigned long long term;  // (offset << 9) | (truncated << 8) | code of the first terminator; ~0 if none
    uint32_t n_tokens;
    uint32_t n_rst;
    uint32_t bad_interval;    // first interval that failed (UINT32_MAX if none)
    uint32_t pad;
    Diag diag;                // that interval's diagnostic (offset = tokens consumed)
};

struct RstEntry {
    uint32_t tok;     // tokens before the marker
    uint32_t number;  // n of RSTn
};

// One (frame, component) run of coefficient blocks, for the transform kernel.
struct JBlockRange {
    uint64_t first;  // first global block
    uint32_t frame;
    uint32_t comp;   // frame component index
};

// ---------------------------------------------------------------- DV25 -----

struct DvFrame {
    const uint8_t *in;   // 120000 / 144000 bytes (device)
    uint8_t *planes;     // planar samples (device): the output itself, or scratch for RGB output
    uint32_t pal;        // 0: 525/60, 1: 625/50
    uint32_t sequences;  // 10 or 12
    uint32_t width, height, cw, ch;
    uint32_t conceal;
    uint32_t item;
    uint64_t blk_off;    // first block in the DV coefficient arena (sequences*27*30 blocks)
    uint32_t seg_first;  // first segment in the segment arrays
    uint32_t dif_first;  // first DIF block in the issue-flag array
};

struct DvState {
    uint32_t bad_segment;  // first failing segment (sequence*27+slot), UINT32_MAX if none
    uint32_t failed;       // number of failing segments
    Diag diag;
};

// ---------------------------------------------------------------- colour ---

// One frame to convert to interleaved RGB24 (crates/cli/src/terminal_preview.rs:7159-7236, 1:1).
struct RgbJob {
    const uint8_t *planes;
    uint8_t *out;
    uint32_t w, h;
    uint32_t lw, lh, cbw, cbh, crw, crh;
    uint32_t cb_off, cr_off;  // offsets of Cb / Cr in planes (Y at 0)
    uint32_t limited;         // ColorRange::Limited
    uint32_t gray;
    uint32_t item;
    uint32_t pad;
};

}  // namespace mmr
