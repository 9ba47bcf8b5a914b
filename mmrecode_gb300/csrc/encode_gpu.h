// Batch JPEG encoder on the GPU: the reference encoder (crates/codecs/mjpeg/src/
// encoder.rs:44-87, 341-545) for many frames per pass, byte-identical to it and to
// the CPU restatement (encode_jpeg) with the same options.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

#include "encode.h"

namespace mmr {

struct EncodeItem {
    FrameIn frame;              // planes in host memory, or device memory with in_on_device
    bool in_on_device = false;
    uint8_t *out = nullptr;     // the JPEG bytes (host, or device with out_on_device)
    size_t out_capacity = 0;
    bool out_on_device = false;
    // results
    int32_t status = 0;         // Status
    std::string message;        // without the status prefix
    size_t out_len = 0;
};

struct EncodeStats {
    float device_ms = 0;              // uploads, kernels and downloads of the last batch
    uint64_t blocks = 0;
    uint64_t exact_coefficients = 0;  // quotients recomputed in binary64 (near a half-integer in fp32)
    uint64_t bytes_out = 0;
};

// Upper bound of an encoded frame's size: headers, and per 8x8 block every
// coefficient coded at the longest code and amplitude with each byte stuffed.
size_t jpeg_encode_bound(uint32_t format, size_t width, size_t height, uint16_t restart_interval);

class GpuJpegEncoder {
public:
    explicit GpuJpegEncoder(int device);
    ~GpuJpegEncoder();
    GpuJpegEncoder(const GpuJpegEncoder &) = delete;
    GpuJpegEncoder &operator=(const GpuJpegEncoder &) = delete;

    // Encodes the items with one set of options and sets each item's status.
    // Returns kOk, or kInternal when the device failed.
    int32_t encode(EncodeItem *items, size_t n, const JpegEncodeOptions &opt);
    EncodeStats last_stats() const { return stats_; }

private:
    struct Impl;
    Impl *impl_;
    EncodeStats stats_;
};

}  // namespace mmr
