// CPU encoders: restatements of the reference MJPEG and DV25 encoders, plus
// stream-generation options the reference lacks (Annex K Huffman tables and
// restart markers for MJPEG; per-block 2-4-8 DCT mode for DV).
#pragma once

#include <stddef.h>
#include <stdint.h>

#include <string>
#include <vector>

namespace mmr {

struct PlaneIn {
    const uint8_t *data;
    size_t data_len, stride, width, height;
};

struct FrameIn {
    uint32_t format;  // PixelFormat
    uint32_t range;   // ColorRange
    size_t width, height;
    size_t plane_count;
    PlaneIn planes[3];
};

struct JpegEncodeOptions {
    uint8_t quality = 75;
    bool annex_k = false;           // standard Annex K Huffman tables instead of the reference's simple tables
    uint16_t restart_interval = 0;  // MCUs per restart interval (0 = no DRI)
};

struct EncodeResult {
    int32_t status = 0;  // Status
    std::string message;
    std::vector<uint8_t> data;
};

// encode_jpeg (crates/codecs/mjpeg/src/encoder.rs:44-87) with default options is
// byte-identical to the reference.
EncodeResult encode_jpeg(const FrameIn &frame, const JpegEncodeOptions &opt);

// Everything of encode_jpeg but the scan: validation (with the reference's
// messages), quantisation tables, Huffman codes and the header bytes up to and
// including SOS. Shared by the CPU encoder and the GPU batch encoder.
struct HuffCode {
    uint16_t bits;
    uint8_t length;
    bool present;
};

struct JpegEncodePlan {
    int32_t status = 0;
    std::string message;
    uint32_t ncomp = 0;
    uint8_t comp_h[3] = {1, 1, 1}, comp_v[3] = {1, 1, 1}, comp_tq[3] = {0, 0, 0};
    uint8_t comp_table[3] = {0, 0, 0};  // Huffman table selector of each component
    uint8_t hmax = 1, vmax = 1;
    size_t mcu_cols = 0, mcu_rows = 0;
    uint16_t restart_interval = 0;
    uint8_t qt[2][64];                  // natural order
    HuffCode dc[2][256], ac[2][256];
    std::vector<uint8_t> header;        // SOI .. SOS
};

bool plan_jpeg_encode(const FrameIn &frame, const JpegEncodeOptions &opt, JpegEncodePlan *plan);

enum DvModePolicy : uint32_t {
    kDvMode88 = 0,        // reference behaviour: every block in 8-8 mode
    kDvModeActivity = 1,  // 2-4-8 where inter-field activity exceeds intra-field activity
};

// encode_video (crates/codecs/dv/src/encoder.rs:67-103) with kDvMode88 is
// byte-identical to the reference.
EncodeResult encode_dv(const FrameIn &frame, uint32_t mode_policy);

}  // namespace mmr
