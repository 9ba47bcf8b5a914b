// Batch decode engine: plans a batch of MJPEG / DV25 packets on the host,
// runs the decode kernels on one CUDA stream and resolves per-item status in
// the reference decoder's error order.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "common.h"

namespace mmr {

enum Codec : uint32_t { kCodecMjpeg = 1, kCodecDv = 2 };
enum ItemFlags : uint32_t { kFlagConceal = 1 };

struct Item {
    // input: `data` must be host-readable (headers are planned on the host);
    // `dev_data`, when set, is a device copy of the same bytes and is used instead
    // of uploading `data`.
    const uint8_t *data = nullptr;
    const uint8_t *dev_data = nullptr;
    size_t len = 0;
    uint32_t codec = kCodecMjpeg;
    uint32_t output = kOutPlanar;
    uint32_t flags = 0;
    uint8_t *out = nullptr;  // destination (host memory, or device memory when out_on_device)
    size_t out_capacity = 0;
    bool out_on_device = false;
    // planar host output written plane by plane (each pointer holds that plane's
    // width*height bytes); used instead of `out` when plane_out[0] is set
    uint8_t *plane_out[3] = {nullptr, nullptr, nullptr};
    // results
    int32_t status = kOk;
    Diag diag{};
    std::string message;
    uint32_t format = 0, range = 0;
    size_t width = 0, height = 0, plane_count = 0;
    size_t plane_offset[3] = {0, 0, 0}, plane_width[3] = {0, 0, 0}, plane_height[3] = {0, 0, 0};
    size_t out_bytes = 0;
    std::vector<std::pair<uint32_t, uint32_t>> concealed;  // (sequence, slot)
};

// Header-only geometry of one packet (no decode).
struct Probe {
    int32_t status = kOk;
    Diag diag{};
    uint32_t format = 0, range = 0;
    size_t width = 0, height = 0, plane_count = 0;
    size_t plane_width[3] = {0, 0, 0}, plane_height[3] = {0, 0, 0};
    size_t planar_bytes = 0, rgb_bytes = 0;
};

Probe probe_packet(uint32_t codec, const uint8_t *data, size_t len);

// Tuning class of an MJPEG packet (restart layout, log2 compressed bits per
// interval), UINT32_MAX when its headers fail or it has more than 4 components.
uint32_t jpeg_tune_class(const uint8_t *data, size_t len);

// Transform tiling class of an MJPEG packet decoded to RGB24 (fused layout
// variant << 8 | bit length of the MCU columns), UINT32_MAX when the fused
// kernel does not take its layout.
uint32_t jpeg_tile_class(const uint8_t *data, size_t len);
// MCUs per CTA of the fused transform's narrow or wide strip for the layout
// variant of a tiling class (tiling class >> 8).
uint32_t fused_strip_mcus(uint32_t tile_class, bool wide);

// Renders a diagnostic as the reference's message. `data` is the packet, used
// to turn token counts into byte offsets for entropy-stage errors.
std::string render_message(const Diag &d, const uint8_t *data, size_t len, uint32_t data_start, uint32_t term);

// CUDA-event times on the engine stream for the last decode() call.
struct EngineTimes {
    float device_ms = 0;    // first upload .. last read-back
    float upload_ms = 0;    // plan + packet uploads
    float scan_ms = 0;      // MJPEG marker scan
    float entropy_ms = 0;   // MJPEG Huffman decode + resolve
    float idct_ms = 0;      // MJPEG dequantisation + IDCT
    float dv_ms = 0;        // DV segment decode + transform
    float rgb_ms = 0;       // colour conversion
    float download_ms = 0;  // read-back
    // inside entropy_ms: the chunked decoder's speculative pass, its sync passes +
    // block prefix, and its final decode
    float slice_spec_ms = 0, slice_sync_ms = 0, slice_decode_ms = 0;
    // inside dv_ms: DIF check + segment decode, then the transform and placement
    float dv_segment_ms = 0, dv_idct_ms = 0;
    uint64_t input_bytes = 0, output_bytes = 0, jpeg_blocks = 0, dv_blocks = 0, rgb_pixels = 0;
    uint64_t idct_exact_samples = 0;  // MJPEG samples recomputed in exact binary64 order
    uint32_t graph_replays = 0;       // batches whose launches replayed a captured CUDA graph
    uint64_t slices = 0;              // slices of the chunked entropy decoder
    uint64_t slices_redone = 0;       // of which the final decode pass redid (the rest were placed)
    uint64_t slices_redone_whole = 0; // of those, redone from their start (no usable speculative part)
};

class Engine {
public:
    // `levels`: streams at that many CUDA priorities, highest first (1: one
    // stream at the default priority); set_level picks the next batch's.
    explicit Engine(int device, int levels = 1);
    ~Engine();
    Engine(const Engine &) = delete;
    Engine &operator=(const Engine &) = delete;

    // Decodes `n` items; blocks until done. Returns kOk, or kInternal when the
    // device failed (then every item carries kDeviceError).
    int32_t decode(Item *items, size_t n, EngineTimes *times = nullptr);

    int device() const { return device_; }
    cudaStream_t stream() const { return stream_; }
    // Runs the following batches on the stream of priority level `l` (0 = highest,
    // clamped to the levels the engine has). Kernels of a higher level go first
    // when engines share the GPU.
    void set_level(int l) { stream_ = streams_[std::min<size_t>(std::max(l, 0), streams_.size() - 1)]; }
    int levels() const { return (int)streams_.size(); }
    // Number of this engine's kernel launches in the last decode() call.
    uint32_t last_launches() const { return launches_; }
    // Replay repeated identical batches from a captured CUDA graph (default on).
    void set_graphs(bool on) { graphs_ = on; }
    bool last_batch_from_graph() const { return graph_replayed_; }
    // Bits per slice of the chunked entropy decoder (a multiple of 32 in
    // 128..2^20); 0 selects the automatic per-frame choice.
    uint32_t slice_bits() const { return slice_bits_; }
    bool set_slice_bits(uint32_t bits) {
        if (bits != 0 && (bits < 128 || bits % 32 || bits > (1u << 20))) return false;
        slice_bits_ = bits;
        return true;
    }
    // Slice bits per tuning class, used when no fixed size is set.
    // (The tables may change while another thread decodes: a batch reads a copy
    // taken at its start.)
    void set_tuned(const std::map<uint32_t, uint32_t> &t) {
        std::lock_guard<std::mutex> g(tables_mu_);
        tuned_ = t;
    }
    // Fused-transform strip per tiling class (1: wide, 0: narrow), and a width
    // forcing every frame (-1: the tuned or default width).
    void set_tuned_tiles(const std::map<uint32_t, uint32_t> &t) {
        std::lock_guard<std::mutex> g(tables_mu_);
        tuned_tile_ = t;
    }
    void set_fused_wide(int wide) {
        std::lock_guard<std::mutex> g(tables_mu_);
        fused_wide_ = wide;
    }

    struct Impl;

private:
    int device_;
    cudaStream_t stream_ = nullptr;      // the current level's stream
    std::vector<cudaStream_t> streams_;  // one per priority level
    uint32_t launches_ = 0;
    uint32_t slice_bits_;
    bool graphs_ = true;
    std::mutex tables_mu_;
    std::map<uint32_t, uint32_t> tuned_;
    std::map<uint32_t, uint32_t> tuned_tile_;
    int fused_wide_ = -1;
    bool graph_replayed_ = false;
    Impl *impl_;
};

}  // namespace mmr
