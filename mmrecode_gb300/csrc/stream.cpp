// Whole-stream decode to Y4M: detection, framing, batch decode, Y4M layout.
#include "stream.h"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <thread>

#include "engine.h"
#include "jpeg_syntax.h"
#include "runtime.h"

namespace mmr {

std::string with_prefix(int32_t st, const std::string &m) {
    switch (st) {
    case kInvalidArgument: return "invalid argument: " + m;
    case kInvalidData: return "invalid data: " + m;
    case kUnsupported: return "unsupported: " + m;
    case kInvalidState: return "invalid state: " + m;
    default: return m;
    }
}

StreamKind detect_stream(const uint8_t *d, size_t len) {
    if (len == 0) return kStreamNone;
    // is_mpegts (main.rs:1915-1921): TS_PACKET_SIZE (188) bytes at least, and each
    // of the first three 188-byte chunks starts with the sync byte 0x47
    if (len >= 188) {
        bool ts = true;
        for (size_t c = 0; c < 3 && c * 188 < len; c++) ts = ts && d[c * 188] == 0x47;
        if (ts) return kStreamMpegTs;
    }
    // is_mpeg2_video (main.rs:1908-1913): a sequence header code among the first
    // 256 four-byte windows
    for (size_t i = 0; i < 256 && i + 4 <= len; i++)
        if (d[i] == 0 && d[i + 1] == 0 && d[i + 2] == 1 && d[i + 3] == 0xb3) return kStreamMpeg2;
    // detect_profile_prefix (profile.rs:107-123): four bytes, the first DIF block a header
    if (len >= 4 && (d[0] >> 5) == 0) return kStreamDv;
    return kStreamMjpeg;
}

bool jpeg_frame_extent(const uint8_t *in, size_t len, const uint64_t *cand, size_t ncand, uint64_t base,
                       size_t *consumed, int32_t *status, std::string *message) {
    using namespace jpeg_detail;
    Diag err = make_diag(kDiagNone);
    auto fail = [&](const Diag &d) {
        *status = d.status;
        *message = with_prefix(d.status, render_message(d, in, len, 0, 0));
        return false;
    };
    JpegHeader h;
    jpeg_header_init(&h);
    size_t soi_off = 0, pos = 0;
    uint8_t soi = 0;
    if (!read_marker(in, len, 0, &soi_off, &soi, &pos, &err)) return fail(err);
    if (soi != 0xd8 || soi_off != 0) return fail(make_diag(kJExpectSoi, (uint32_t)soi_off));
    bool pending = false;
    size_t p_off = 0, p_after = 0;
    uint8_t p_code = 0;
    for (;;) {
        size_t offset = 0, after = 0;
        uint8_t code = 0;
        if (pending) {
            offset = p_off;
            code = p_code;
            after = p_after;
            pending = false;
        } else if (!read_marker(in, len, pos, &offset, &code, &after, &err)) {
            return fail(err);
        }
        pos = after;
        if (code == 0xd9) {  // EOI: the rest is trailing data, the next image
            *consumed = pos;
            return true;
        }
        if (!has_length(code)) continue;
        if (pos + 2 > len) return fail(make_diag(kJTruncLength, (uint32_t)pos));
        const uint16_t length = be16(in + pos);
        if (length < 2) return fail(make_diag(kJBadLength, (uint32_t)pos));
        const size_t payload_offset = pos + 2, payload_length = (size_t)length - 2;
        const size_t payload_end = payload_offset + payload_length;
        if (payload_end > len) return fail(make_diag(kJTruncPayload, (uint32_t)payload_offset, code));
        if (!parse_segment(in, code, payload_offset, payload_length, !h.have_sos, &h, &err)) return fail(err);
        pos = payload_end;
        if (code != 0xda) continue;
        // scan_entropy_data (parser.rs:373-414): the first candidate at or after the
        // segment's start; its 0xFF run starts no earlier than the segment
        const uint64_t *it = std::lower_bound(cand, cand + ncand, base + pos);
        if (it == cand + ncand) {
            // no terminating marker: a 0xFF run at the very end is a truncated marker
            const bool trunc = len > pos && in[len - 1] == 0xff;
            char b[160];
            snprintf(b, sizeof b, "JPEG at byte 0x%08zx: %s", len,
                     trunc ? "truncated marker in entropy-coded data" : "entropy-coded scan has no terminating marker");
            *status = kInvalidData;
            *message = with_prefix(kInvalidData, b);
            return false;
        }
        const size_t q = (size_t)(*it - base);
        size_t run = q;
        while (run > pos && in[run - 1] == 0xff) run--;
        p_off = run;
        p_code = in[q + 1];
        p_after = q + 2;
        pending = true;
        pos = p_after;
    }
}

namespace {

// chroma_tag (lib.rs:283-299)
bool chroma_tag(uint32_t format, const char **tag, int32_t *status, std::string *message) {
    switch (format) {
    case kGray8: *tag = "Cmono"; return true;
    case kYuv420: *tag = "C420jpeg"; return true;
    case kYuv411: *tag = "C411"; return true;
    case kYuv422: *tag = "C422"; return true;
    case kYuv444: *tag = "C444"; return true;
    default:
        *status = kUnsupported;
        *message = with_prefix(kUnsupported, "pixel format has no Y4M representation");
        return false;
    }
}

// plane_dimensions (lib.rs:340-373) checked against a decoded frame's planes
// (validate_planes, lib.rs:313-338: a planar output has stride == width).
bool planes_ok(const Item &it, int32_t *status, std::string *message) {
    const size_t w = it.width, h = it.height, hw = (w + 1) / 2, qw = (w + 3) / 4, hh = (h + 1) / 2;
    size_t ew[3] = {w, w, w}, eh[3] = {h, h, h}, n = 3;
    switch (it.format) {
    case kGray8: n = 1; break;
    case kYuv420: ew[1] = ew[2] = hw; eh[1] = eh[2] = hh; break;
    case kYuv411: ew[1] = ew[2] = qw; break;
    case kYuv422: ew[1] = ew[2] = hw; break;
    default: break;
    }
    if (it.plane_count != n) {
        static const char *names[6] = {"?", "Gray8", "Yuv420p8", "Yuv422p8", "Yuv444p8", "Yuv411p8"};
        char b[160];
        snprintf(b, sizeof b, "Y4M %s frame requires %zu plane(s), found %zu", names[it.format < 6 ? it.format : 0], n,
                 it.plane_count);
        *status = kInvalidData;
        *message = with_prefix(kInvalidData, b);
        return false;
    }
    for (size_t c = 0; c < n; c++) {
        if (it.plane_width[c] != ew[c] || it.plane_height[c] != eh[c]) {
            char b[160];
            snprintf(b, sizeof b, "Y4M plane %zu has inconsistent dimensions, stride, or storage", c);
            *status = kInvalidData;
            *message = with_prefix(kInvalidData, b);
            return false;
        }
    }
    return true;
}

}  // namespace

bool y4m_header(uint32_t format, uint32_t range, bool bottom_first, size_t width, size_t height, std::string *header,
                int32_t *status, std::string *message) {
    const char *chroma = nullptr;
    if (!chroma_tag(format, &chroma, status, message)) return false;
    // color_range_tag (lib.rs:272-281), interlace_tag (lib.rs:301-311): the MJPEG
    // decoder's frames are progressive, the DV decoder's bottom field first
    const char *rt = range == kRangeFull ? " XCOLORRANGE=FULL" : range == kRangeLimited ? " XCOLORRANGE=LIMITED" : "";
    char b[160];
    snprintf(b, sizeof b, "YUV4MPEG2 W%zu H%zu I%c %s%s\n", width, height, bottom_first ? 'b' : 'p', chroma, rt);
    *header = b;
    return true;
}

// ---------------------------------------------------------------- stream ---

Stream::Stream(EnginePool &pool, const uint8_t *data, size_t len, const std::string &input_name)
    : pool_(pool), data_(data), len_(len), input_name_(input_name) {
    kind_ = detect_stream(data, len);
    switch (kind_) {
    case kStreamNone:  // decode (main.rs:1538-1540)
        frame_status_ = kInvalidData;
        frame_message_ = "input contains no media frames";
        return;
    case kStreamMpegTs:
        frame_status_ = kUnsupported;
        frame_message_ = with_prefix(kUnsupported, "MPEG transport streams are outside this library, which "
                                                   "implements the MJPEG and DV25 paths");
        return;
    case kStreamMpeg2:
        frame_status_ = kUnsupported;
        frame_message_ = with_prefix(kUnsupported, "MPEG-2 video is outside this library, which implements the "
                                                   "MJPEG and DV25 paths");
        return;
    default: break;
    }
    if (cudaSetDevice(pool_.device()) != cudaSuccess || cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking) != cudaSuccess ||
        cudaMalloc(&dev_, len_) != cudaSuccess) {
        cudaGetLastError();
        if (dev_) cudaFree(dev_);
        if (s_) cudaStreamDestroy(s_);
        throw std::runtime_error("cannot allocate the stream on the device");
    }
    try {
        if (kind_ == kStreamDv) frame_dv();
        else frame_mjpeg();
    } catch (...) {  // a constructor that throws runs no destructor: free the device copy here
        cudaStreamSynchronize(s_);
        cudaStreamDestroy(s_);
        cudaFree(dev_);
        cudaGetLastError();
        throw;
    }
    // Y4M layout: the first frame's header, then "FRAME\n" and the planes of each
    const size_t nf = frames_.size();
    planar_.resize(nf);
    payload_.resize(nf);
    const uint32_t codec = kind_ == kStreamDv ? kCodecDv : kCodecMjpeg;
    std::vector<Probe> probes(nf);
    auto probe_range = [&](size_t a, size_t b) {
        for (size_t i = a; i < b; i++) probes[i] = probe_packet(codec, data_ + frames_[i].first, frames_[i].second);
    };
    // the frames' headers are independent: read them on several host threads
    const size_t threads = std::min<size_t>(std::max(1u, std::thread::hardware_concurrency()), (nf + 15) / 16);
    if (threads <= 1) {
        probe_range(0, nf);
    } else {
        std::vector<std::thread> pool;
        const size_t per = (nf + threads - 1) / threads;
        for (size_t t = 0; t < threads; t++) pool.emplace_back(probe_range, t * per, std::min(nf, (t + 1) * per));
        for (std::thread &t : pool) t.join();
    }
    for (size_t i = 0; i < nf; i++) planar_[i] = probes[i].planar_bytes;
    if (nf) {
        const Probe &p = probes[0];
        std::string hdr, msg;
        int32_t st = kOk;
        if (p.status == kOk && y4m_header(p.format, p.range, kind_ == kStreamDv, p.width, p.height, &hdr, &st, &msg))
            header_len_ = hdr.size();
    }
    size_t at = header_len_;
    for (size_t i = 0; i < frames_.size(); i++) {
        payload_[i] = at + 6;
        at += 6 + planar_[i];
    }
    y4m_bytes_ = frames_.empty() ? 0 : at;
}

Stream::~Stream() {
    if (s_) {
        cudaStreamSynchronize(s_);
        cudaStreamDestroy(s_);
    }
    if (dev_) cudaFree(dev_);
}

// decode_dv (main.rs:1605-1633): profile from the first frame's header, then
// exact frame-size chunks
void Stream::frame_dv() {
    const size_t fs = (data_[3] & 0x80) ? 144000 : 120000;
    if (len_ % fs != 0) {
        frame_status_ = kInvalidData;
        frame_message_ = "'" + input_name_ + "' ends with an incomplete raw DV frame";
        return;
    }
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, s_);
    cudaMemcpyAsync(dev_, data_, len_, cudaMemcpyHostToDevice, s_);
    cudaEventRecord(e1, s_);
    if (cudaStreamSynchronize(s_) != cudaSuccess) {
        cudaGetLastError();
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw std::runtime_error("device failure while uploading the stream");
    }
    cudaEventElapsedTime(&upload_ms_, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (size_t off = 0; off < len_; off += fs) frames_.push_back({off, fs});
}

// decode (main.rs:1555-1572): parse_jpeg on what remains, one image at a time,
// with the entropy-coded segments ended by the device's marker candidates
void Stream::frame_mjpeg() {
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, pool_.device());
    uint32_t cap = 1u << 16;
    uint64_t *d_cand = nullptr;
    uint32_t *d_count = nullptr;
    cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};
    std::vector<uint64_t> cand;
    auto cleanup = [&]() {
        if (d_cand) cudaFree(d_cand);
        if (d_count) cudaFree(d_count);
        for (cudaEvent_t &e : ev)
            if (e) cudaEventDestroy(e);
    };
    bool ok = cudaMalloc(&d_count, sizeof(uint32_t)) == cudaSuccess &&
              cudaMalloc(&d_cand, (size_t)cap * sizeof(uint64_t)) == cudaSuccess;
    for (cudaEvent_t &e : ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    ok = ok && cudaEventRecord(ev[0], s_) == cudaSuccess &&
         cudaMemcpyAsync(dev_, data_, len_, cudaMemcpyHostToDevice, s_) == cudaSuccess &&
         cudaEventRecord(ev[1], s_) == cudaSuccess;
    for (int pass = 0; ok && pass < 2; pass++) {
        if (!d_cand) ok = cudaMalloc(&d_cand, (size_t)cap * sizeof(uint64_t)) == cudaSuccess;
        ok = ok && cudaMemsetAsync(d_count, 0, sizeof(uint32_t), s_) == cudaSuccess;
        if (!ok) break;
        launch_marker_candidates(dev_, len_, d_cand, cap, d_count, sms, s_);
        uint32_t count = 0;
        ok = cudaGetLastError() == cudaSuccess && cudaEventRecord(ev[2], s_) == cudaSuccess &&
             cudaMemcpyAsync(&count, d_count, sizeof count, cudaMemcpyDeviceToHost, s_) == cudaSuccess &&
             cudaStreamSynchronize(s_) == cudaSuccess;
        if (!ok) break;
        n_cand_ = count;
        if (count <= cap) {
            cand.resize(count);
            ok = (!count || cudaMemcpy(cand.data(), d_cand, (size_t)count * sizeof(uint64_t), cudaMemcpyDeviceToHost) ==
                                cudaSuccess);
            if (ok) {
                cudaEventElapsedTime(&upload_ms_, ev[0], ev[1]);
                cudaEventElapsedTime(&scan_ms_, ev[1], ev[2]);
            }
            break;
        }
        cudaFree(d_cand);  // more candidates than room: once more with room for all
        d_cand = nullptr;
        cap = count;
        cudaEventRecord(ev[1], s_);
    }
    cleanup();
    if (!ok) {
        cudaGetLastError();
        throw std::runtime_error("device failure while framing the stream");
    }
    std::sort(cand.begin(), cand.end());
    uint64_t pos = 0;
    while (pos < len_) {
        size_t consumed = 0;
        int32_t st = kOk;
        std::string msg;
        if (!jpeg_frame_extent(data_ + pos, len_ - pos, cand.data(), cand.size(), pos, &consumed, &st, &msg)) {
            frame_status_ = st;
            frame_message_ = msg;
            return;
        }
        frames_.push_back({pos, consumed});
        pos += consumed;
    }
}

StreamResult Stream::decode_y4m(uint8_t *out, size_t capacity) {
    StreamResult r;
    const size_t n = frames_.size();
    if (n == 0) {
        r.status = frame_status_;
        r.message = frame_message_;
        return r;
    }
    if (!out || capacity < y4m_bytes_) {
        r.status = kInvalidArgument;
        r.message = with_prefix(kInvalidArgument, "output buffer is smaller than the stream's Y4M bytes");
        return r;
    }
    std::vector<Item> items(n);
    const uint32_t codec = kind_ == kStreamDv ? kCodecDv : kCodecMjpeg;
    for (size_t i = 0; i < n; i++) {
        Item &it = items[i];
        it.data = data_ + frames_[i].first;
        it.dev_data = dev_ + frames_[i].first;
        it.len = frames_[i].second;
        it.codec = codec;
        it.output = kOutPlanar;
        it.out = out + payload_[i];
        it.out_capacity = planar_[i];
        it.out_on_device = false;
    }
    EngineTimes t;
    if (pool_.decode(items.data(), n, &t) != kOk) {
        r.status = kInternal;
        r.message = "CUDA device failure during stream decode";
        return r;
    }
    // the CLI's loop: decode, then Y4mWriter::write_frame (lib.rs:246-267)
    const bool dv = kind_ == kStreamDv;
    for (size_t i = 0; i < n; i++) {
        const Item &it = items[i];
        if (it.status != kOk) {
            r.status = it.status;
            r.message = with_prefix(it.status, it.message);
            return r;
        }
        const char *chroma = nullptr;
        if (!chroma_tag(it.format, &chroma, &r.status, &r.message) || !planes_ok(it, &r.status, &r.message)) return r;
        const Item &f0 = items[0];
        if (i == 0) {
            std::string hdr;
            if (!y4m_header(it.format, it.range, dv, it.width, it.height, &hdr, &r.status, &r.message)) return r;
            if (hdr.size() != header_len_ || it.out_bytes != planar_[i]) {
                r.status = kInternal;
                r.message = "stream layout does not match the decoded first frame";
                return r;
            }
            memcpy(out, hdr.data(), hdr.size());
        } else if (it.width != f0.width || it.height != f0.height || it.format != f0.format) {
            r.status = kInvalidData;
            r.message = with_prefix(kInvalidData, "Y4M stream dimensions or pixel format changed between frames");
            return r;
        }
        if (it.out_bytes != planar_[i]) {
            r.status = kInternal;
            r.message = "stream layout does not match a decoded frame";
            return r;
        }
        memcpy(out + payload_[i] - 6, "FRAME\n", 6);
        r.frames_written = i + 1;
        r.bytes_written = payload_[i] + planar_[i];
    }
    r.status = frame_status_;
    r.message = frame_message_;
    return r;
}

}  // namespace mmr
