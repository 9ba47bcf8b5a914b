// Whole-stream decode: framing of concatenated JFIF images and raw DV frames,
// batch decode, and the Y4M byte stream the reference CLI's `decode` command
// writes (crates/cli/src/main.rs:1533-1580, 1605-1633; crates/containers/y4m/src/
// lib.rs:219-300).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include "common.h"

namespace mmr {

class EnginePool;

// ApiError Display (crates/capi/src/lib.rs:73-80) and core Error Display
// (crates/core/src/error.rs:18-27): the message behind its status's prefix.
std::string with_prefix(int32_t status, const std::string &message);

// Appends to out[0, cap) every position q < len - 1 of in[0, len) whose byte is
// 0xFF and whose next byte is not 0x00, 0xFF or 0xD0..0xD7 (in no particular
// order); *count (zeroed by the caller) receives how many there are, also past cap.
void launch_marker_candidates(const uint8_t *in, uint64_t len, uint64_t *out, uint32_t cap, uint32_t *count,
                              int sm_count, cudaStream_t s);

// Stream kinds in the order the CLI tests for them (main.rs:1536-1553).
enum StreamKind : uint32_t {
    kStreamNone = 0,    // empty input
    kStreamMjpeg = 1,   // concatenated JFIF images
    kStreamDv = 2,      // raw DV frames of one profile
    kStreamMpegTs = 3,  // MPEG transport stream (outside this library)
    kStreamMpeg2 = 4,   // MPEG-2 video elementary stream (outside this library)
};

// is_mpegts, is_mpeg2_video (main.rs:1908-1921) and detect_profile_prefix
// (crates/codecs/dv/src/profile.rs:107-123), in the CLI's order.
StreamKind detect_stream(const uint8_t *data, size_t len);

// parse_jpeg (parser.rs:18-81) over in[0, len), the bytes that remain of a
// stream, with each entropy-coded segment ended at the first marker candidate
// at or after its start (cand: sorted positions in the stream, base: the
// stream position of in[0]). On success *consumed is the image's length (up to
// and including EOI); otherwise *status and *message are parse_jpeg's error.
bool jpeg_frame_extent(const uint8_t *in, size_t len, const uint64_t *cand, size_t ncand, uint64_t base,
                       size_t *consumed, int32_t *status, std::string *message);

// The 8-bit Y4M stream header of a frame (Y4mWriter::write_frame, lib.rs:
// 246-260): interlace 'b' (bottom field first, the DV decoder's frames) or 'p'
// (progressive, the MJPEG decoder's), or the writer's error for formats it cannot
// represent.
bool y4m_header(uint32_t format, uint32_t range, bool bottom_first, size_t width, size_t height,
                std::string *header, int32_t *status, std::string *message);

struct StreamResult {
    int32_t status = kOk;
    std::string message;     // with the reference's Display prefix ("invalid data: ...")
    size_t frames_written = 0;
    size_t bytes_written = 0;
};

// One stream: framed at construction (host bytes uploaded once, marker
// candidates found on the device), decoded to Y4M by decode_y4m. The host bytes
// must stay valid until the object is destroyed.
class Stream {
public:
    Stream(EnginePool &pool, const uint8_t *data, size_t len, const std::string &input_name);
    ~Stream();
    Stream(const Stream &) = delete;
    Stream &operator=(const Stream &) = delete;

    StreamKind kind() const { return kind_; }
    // framing outcome: frames found before the first framing error (if any)
    int32_t frame_status() const { return frame_status_; }
    const std::string &frame_message() const { return frame_message_; }
    size_t frame_count() const { return frames_.size(); }
    uint64_t frame_offset(size_t i) const { return frames_[i].first; }
    uint64_t frame_length(size_t i) const { return frames_[i].second; }
    // bytes decode_y4m needs: header + every framed frame's "FRAME\n" and planes
    size_t y4m_bytes() const { return y4m_bytes_; }
    // device time of the upload and of the candidate scan (ms), candidates found
    float upload_ms() const { return upload_ms_; }
    float scan_ms() const { return scan_ms_; }
    uint64_t candidates() const { return n_cand_; }

    // Decodes every framed frame on the pool and lays the Y4M stream out in
    // out[0, capacity): what the CLI writes before its first error (a frame that
    // fails to decode, one the writer rejects, or the framing error).
    StreamResult decode_y4m(uint8_t *out, size_t capacity);

private:
    void frame_mjpeg();
    void frame_dv();

    EnginePool &pool_;
    const uint8_t *data_;
    size_t len_;
    std::string input_name_;
    StreamKind kind_ = kStreamNone;
    int32_t frame_status_ = kOk;
    std::string frame_message_;
    std::vector<std::pair<uint64_t, uint64_t>> frames_;
    std::vector<size_t> planar_;    // planar bytes of each frame (0 if its headers fail)
    std::vector<size_t> payload_;   // Y4M offset of each frame's planes
    size_t header_len_ = 0;
    size_t y4m_bytes_ = 0;
    uint8_t *dev_ = nullptr;        // the stream on the device
    cudaStream_t s_ = nullptr;
    float upload_ms_ = 0, scan_ms_ = 0;
    uint64_t n_cand_ = 0;
};

}  // namespace mmr
