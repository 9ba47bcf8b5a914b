// Kernel launchers (host-callable) for the MJPEG and DV25 decode stages.
#pragma once

#include <cuda_runtime.h>

#include "plan.h"

namespace mmr {

constexpr int kScanTile = 4096;  // bytes of entropy-coded data per marker-scan CTA

struct JpegLaunch {
    const JFrame *frames;        // device
    JState *states;              // device
    uint32_t n_frames;
    const uint32_t *tile_first;  // n_frames + 1 prefix of marker-scan tiles
    uint32_t n_tiles;
    uint32_t *tile_tok;          // per tile: token count, then its exclusive prefix
    uint32_t *tile_rst;
    RstEntry *rsts;
    const JSched *sched;
    const JBlockRec *brec;       // parallel to sched
    const JComp *comps;
    const HuffLut *luts;
    uint32_t n_luts;
    const uint8_t *symbols;
    const uint16_t *quant;       // natural order
    const uint2 *items;          // (frame, interval); frames with <= 4 components first
    uint32_t n_items_small;
    uint32_t n_items;
    Diag *results;               // per item
    int16_t *coef;               // 64 levels per block
    int32_t *dc;                 // dequantised DC per block
    const JBlockRange *ranges;
    uint32_t n_ranges;
    const uint32_t *idct_cta_first;  // n_ranges + 1 prefix of transform CTAs (idct_ctas per range)
    uint32_t n_idct_ctas;
    uint64_t n_blocks;
    uint32_t *item_ok;           // per batch item: 1 while decoding has not failed
    ulonglong2 *fix;             // blocks the fp32 IDCT could not fully decide: (block, sample mask)
    uint32_t *fix_count;         // entries, samples, slices redone, slices, short redos listed, slices
                                 // redone whole (8 counters, zeroed per batch)
    uint32_t fixup_grid;         // CTAs of the grid-stride fixup pass
    // chunked entropy decoder (frames with <= 4 components; items [0, n_items_small))
    uint32_t n_slots;
    uint32_t *slot_item;         // per slot: item, UINT32_MAX when unused
    IvInfo *ivs;                 // per item
    SliceSync *sync;             // per slot
    SliceSpec *spec;             // per slot
    SlicePrefix *prefix;         // per slot
    SliceEvent *events;          // per slot
    unsigned long long *iv_key;  // per item: (position << 26 | slice) of its first event
    uint32_t *sync_dirty;        // per sync pass: slices whose exit state changed, then per pass the
                                 // next slot to take (2 x kSyncPasses, zeroed per batch)
    // levels written by the speculative decode (SliceOwn): per slot what it owns,
    // the scratch arena, its allocation counter (zeroed per batch), and per block
    // where its levels are (scratch block, or kLevelsInPlace: the coefficient arena)
    SliceOwn *own;
    SliceMatch *match;           // per slot (written by the speculative and sync passes)
    uint32_t *redo;              // per slot: leading owned blocks the final decode pass writes
                                 // (0: none, UINT32_MAX: all; zeroed per batch)
    uint32_t *work;              // n_slots: slots with short work for the final decode (count in fix_count[4])
    int16_t *scratch;            // 64 levels per scratch block
    int16_t *scratch_dc;         // DC difference per scratch block
    uint32_t scratch_blocks;
    unsigned long long *scratch_next;
    uint32_t *blk_map;           // per block (all 0xff per batch); nullptr: levels in place
    const long long *fixw;       // fixed-point IDCT weights (exact_fixed.h)
};

// Parallel sync passes before the serial fix-up walk; a pass after one that changed
// nothing returns at once (measured: 4 passes take VGA 4:2:0 restart-less frames
// from 0.49 to 0.42 ms of sync per 30 frames and cost 1080p batches nothing; 6 are
// slower again)
constexpr int kSyncPasses = 4;

void launch_jpeg_scan(const JpegLaunch &L, cudaStream_t s);
void launch_jpeg_entropy(const JpegLaunch &L, cudaStream_t s);   // frames with > 4 components
// frames with <= 4 components; marks (optional, 3 events) are recorded after the
// speculative pass, after the sync passes + prefix, and after the final decode
// (as external event nodes when the stream is being captured into a graph)
void launch_jpeg_slices(const JpegLaunch &L, cudaStream_t s, cudaEvent_t *marks = nullptr, bool capturing = false);
int jpeg_slice_launches(const JpegLaunch &L);
void launch_jpeg_idct(const JpegLaunch &L, cudaStream_t s);
uint32_t idct_ctas(uint32_t blocks);

// MJPEG frames decoded straight to RGB24 (three components, chroma 1x1, luma
// 1x1, 2x1 or 2x2): one launch per layout, a CTA per strip of MCUs.
struct FusedJob {
    uint32_t frame;     // JFrame index
    uint32_t strips_x;  // strips per MCU row
    uint32_t width, height;
    uint8_t *out;       // width * height * 3 bytes
};

struct FusedLaunch {
    const FusedJob *jobs;
    const uint32_t *cta_first;  // n_jobs + 1 prefix of CTAs (strips_x * mcu_rows per job)
    uint32_t n_jobs;
    uint32_t n_ctas;
};

int fused_variant(uint32_t hmax, uint32_t vmax);  // 0: 1x1, 1: 2x1, 2: 2x2, -1: not fused
// launch slot of a layout variant with a narrow or wide strip (MCUs per CTA:
// 8 or 16 at 1x1, 4 or 8 otherwise); kFusedSlots launches, one per slot
constexpr int kFusedSlots = 6;
int fused_slot(int variant, bool wide);
uint32_t fused_slot_mcus(int slot);
uint32_t fused_strips_x(int slot, uint32_t mcu_cols);
void launch_jpeg_idct_rgb(const JpegLaunch &L, const FusedLaunch *FL, cudaStream_t s);  // FL[kFusedSlots]
int fused_launches(const FusedLaunch &FL);

struct DvLaunch {
    const DvFrame *frames;
    DvState *states;
    uint32_t n_frames;
    const uint32_t *seg_first;   // n_frames + 1 prefix of segments
    uint32_t n_segments;
    const uint32_t *dif_first;   // n_frames + 1 prefix of DIF blocks
    uint32_t n_dif;
    uint8_t *flags;              // per DIF block: 1 if its identifier is damaged
    uint8_t *seg_err;            // per segment: DiagKind (0 = ok)
    int16_t *coef;               // 64 per block, natural order
    uint8_t *modes;              // per block: 1 = 2-4-8
    const uint32_t *vlc;         // two-level VLC table
    const long long *fixw;       // fixed-point transform weights: 8-8 then 2-4-8 (exact_fixed.h)
    uint64_t n_blocks;
    uint32_t *item_ok;
};

void launch_dv_decode(const DvLaunch &L, cudaStream_t s);
void launch_dv_idct(const DvLaunch &L, cudaStream_t s);

struct RgbLaunch {
    const RgbJob *jobs;
    const uint32_t *cta_first;  // n_jobs + 1 prefix of CTAs (rgb_ctas per job)
    uint32_t n_jobs;
    uint32_t n_ctas;
    const uint32_t *item_ok;
};

uint32_t rgb_ctas(uint32_t w, uint32_t h);
void launch_rgb(const RgbLaunch &L, cudaStream_t s);

// DV VLC lookup: level-1 indexed by the next 10 bits; long codes index a
// 64-entry level-2 block with the following 6 bits. Entry layout:
//   bit 31 set: level-2 block at bits 0..15 (entry index)
//   otherwise: len (bits 0..4), run (bits 5..11), level + 256 (bits 12..20); len 0 = no code
constexpr int kDvVlcL1Bits = 10;

}  // namespace mmr
