// C ABI of libmmrecode_gpu.so: the v1 symbols of mmrecode.h (same semantics
// as crates/capi/src/lib.rs) and the additive batch API of mmrecode_gpu.h.
#include <cuda_runtime.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "../../include/mmrecode.h"
#include "../../include/mmrecode_gpu.h"
#include "encode.h"
#include "encode_gpu.h"
#include "engine.h"
#include "last_error.h"
#include "runtime.h"
#include "stream.h"

using mmr::Engine;
using mmr::Item;
using mmr::with_prefix;

namespace {

const char kVersion[] = "0.0.1+gb300";

// lib.rs:46-48: the last diagnostic is thread-local.
thread_local std::string g_last_error;

mmr_status finish(mmr_status st, const std::string &msg) {
    g_last_error = st == MMR_STATUS_OK ? std::string() : msg;
    return st;
}

mmr_status invalid_argument(const std::string &m) { return finish(MMR_STATUS_INVALID_ARGUMENT, "invalid argument: " + m); }

// Engines for the v1 single-packet calls: each concurrent caller borrows one.
std::mutex g_pool_mutex;
std::vector<Engine *> g_pool;

Engine *acquire_engine(std::string &err) {
    {
        std::lock_guard<std::mutex> lock(g_pool_mutex);
        if (!g_pool.empty()) {
            Engine *e = g_pool.back();
            g_pool.pop_back();
            return e;
        }
    }
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        err = "no CUDA device is available to the GPU decoder";
        return nullptr;
    }
    try {
        return new Engine(0);
    } catch (const std::exception &e) {
        err = std::string("could not initialise the GPU decoder: ") + e.what();
        return nullptr;
    }
}

void release_engine(Engine *e) {
    std::lock_guard<std::mutex> lock(g_pool_mutex);
    g_pool.push_back(e);
}

void reset_frame(mmr_video_frame *f) {
    memset(f, 0, sizeof(*f));
    f->struct_size = sizeof(mmr_video_frame);
}

void free_frame_planes(mmr_video_frame *f) {
    size_t n = f->plane_count < MMR_MAX_PLANES ? f->plane_count : MMR_MAX_PLANES;
    for (size_t i = 0; i < n; i++) free(f->planes[i].data);
}

// Host planes for a packet whose headers give its geometry, set as the item's
// planar outputs (one malloc'd buffer per plane, as mmr_video_frame_free expects);
// planes stay null when the headers fail (the decode then reports why). False
// when the host is out of memory.
bool alloc_planes(const mmr::Probe &pr, Item &it, uint8_t *planes[3]) {
    planes[0] = planes[1] = planes[2] = nullptr;
    if (pr.status != MMR_STATUS_OK || pr.format == 0 || pr.plane_count > 3) return true;
    for (size_t c = 0; c < pr.plane_count; c++) {
        size_t bytes = pr.plane_width[c] * pr.plane_height[c];
        planes[c] = (uint8_t *)malloc(bytes ? bytes : 1);
        if (!planes[c]) {
            for (size_t k = 0; k < c; k++) free(planes[k]);
            planes[0] = planes[1] = planes[2] = nullptr;
            return false;
        }
        it.plane_out[c] = planes[c];
    }
    it.out_capacity = pr.planar_bytes;
    return true;
}

// Hands the decoded planes to the caller's frame (which owns them from here on).
void fill_frame(const Item &it, uint8_t *const planes[3], mmr_video_frame *out) {
    out->format = it.format;
    out->range = it.range;
    out->width = it.width;
    out->height = it.height;
    out->plane_count = it.plane_count;
    for (size_t c = 0; c < it.plane_count && c < MMR_MAX_PLANES; c++) {
        out->planes[c].data = planes[c];
        out->planes[c].width = it.plane_width[c];
        out->planes[c].height = it.plane_height[c];
        out->planes[c].stride = it.plane_width[c];
        out->planes[c].data_len = it.plane_width[c] * it.plane_height[c];
    }
}

// The v1 convention for a caller's frame (lib.rs:604-611): non-null, its
// struct_size this library's (else INVALID_ARGUMENT and the frame is untouched).
mmr_status check_frame(mmr_video_frame *out) {
    if (!out) return invalid_argument("out_frame is null");
    if (out->struct_size != sizeof(mmr_video_frame)) {
        char m[128];
        snprintf(m, sizeof m, "out_frame struct_size is %zu, expected %zu", out->struct_size, sizeof(mmr_video_frame));
        return invalid_argument(m);
    }
    return MMR_STATUS_OK;
}

// mjpeg_decode_impl / dv_decode_impl (lib.rs:594-642) on the GPU.
mmr_status decode_one(uint32_t codec, const uint8_t *data, size_t len, mmr_video_frame *out) {
    if (mmr_status st = check_frame(out)) return st;
    reset_frame(out);
    if (len > 0 && !data) return invalid_argument("data is null while length is nonzero");
    mmr::Probe pr = mmr::probe_packet(codec, data, len);
    Item it;
    it.data = data;
    it.len = len;
    it.codec = codec;
    it.output = mmr::kOutPlanar;
    uint8_t *planes[3];
    if (!alloc_planes(pr, it, planes)) return finish(MMR_STATUS_INTERNAL_ERROR, "out of host memory");
    std::string err;
    Engine *engine = acquire_engine(err);
    if (!engine) {
        for (auto p : planes) free(p);
        return finish(MMR_STATUS_INTERNAL_ERROR, err);
    }
    engine->decode(&it, 1);
    release_engine(engine);
    if (it.status != MMR_STATUS_OK) {
        for (auto p : planes) free(p);
        return finish(it.status, with_prefix(it.status, it.message));
    }
    fill_frame(it, planes, out);
    return finish(MMR_STATUS_OK, "");
}

// video_frame_from_view + validate_plane_storage (lib.rs:1061-1127).
mmr_status frame_from_view(const mmr_video_frame_view *v, mmr::FrameIn &f) {
    if (v->plane_count > MMR_MAX_PLANES) {
        char m[96];
        snprintf(m, sizeof m, "plane_count %zu exceeds %u", v->plane_count, MMR_MAX_PLANES);
        return invalid_argument(m);
    }
    if (v->format < 1 || v->format > 5) {
        char m[96];
        snprintf(m, sizeof m, "unknown pixel format %u", v->format);
        return invalid_argument(m);
    }
    if (v->range > 2) {
        char m[96];
        snprintf(m, sizeof m, "unknown color range %u", v->range);
        return invalid_argument(m);
    }
    size_t expected = v->format == MMR_PIXEL_FORMAT_GRAY8 ? 1 : 3;
    if (v->plane_count != expected) {
        char m[96];
        snprintf(m, sizeof m, "pixel format requires %zu planes, received %zu", expected, v->plane_count);
        return invalid_argument(m);
    }
    f.format = v->format;
    f.range = v->range;
    f.width = v->width;
    f.height = v->height;
    f.plane_count = v->plane_count;
    for (size_t i = 0; i < v->plane_count; i++) {
        const mmr_plane_view &p = v->planes[i];
        if (p.data_len > 0 && !p.data) return invalid_argument("plane data is null while length is nonzero");
        size_t rows = p.height ? p.height - 1 : 0;
        unsigned __int128 required = (unsigned __int128)rows * p.stride + p.width;
        if (required > p.data_len) {
            char m[128];
            snprintf(m, sizeof m, "plane %zu needs %llu bytes but data_len is %zu", i, (unsigned long long)required,
                     p.data_len);
            return invalid_argument(m);
        }
        f.planes[i] = {p.data, p.data_len, p.stride, p.width, p.height};
    }
    return MMR_STATUS_OK;
}

mmr_status check_buffer(mmr_buffer *b) {
    if (b->struct_size != sizeof(mmr_buffer)) {
        char m[128];
        snprintf(m, sizeof m, "out_buffer struct_size is %zu, expected %zu", b->struct_size, sizeof(mmr_buffer));
        return invalid_argument(m);
    }
    return MMR_STATUS_OK;
}

void reset_buffer(mmr_buffer *b) {
    b->struct_size = sizeof(mmr_buffer);
    b->data = nullptr;
    b->len = 0;
}

mmr_status emit_buffer(const mmr::EncodeResult &r, mmr_buffer *out) {
    if (r.status != MMR_STATUS_OK) return finish(r.status, with_prefix(r.status, r.message));
    out->data = (uint8_t *)malloc(r.data.size() ? r.data.size() : 1);
    if (!out->data) return finish(MMR_STATUS_INTERNAL_ERROR, "out of host memory");
    memcpy(out->data, r.data.data(), r.data.size());
    out->len = r.data.size();
    return finish(MMR_STATUS_OK, "");
}

template <typename F>
mmr_status encode_entry(const mmr_video_frame_view *frame, mmr_buffer *out, F &&encode) {
    if (!frame) return invalid_argument("frame is null");
    if (!out) return invalid_argument("out_buffer is null");
    if (frame->struct_size != sizeof(mmr_video_frame_view)) {
        char m[128];
        snprintf(m, sizeof m, "frame struct_size is %zu, expected %zu", frame->struct_size, sizeof(mmr_video_frame_view));
        return invalid_argument(m);
    }
    if (check_buffer(out) != MMR_STATUS_OK) return MMR_STATUS_INVALID_ARGUMENT;
    reset_buffer(out);
    mmr::FrameIn f;
    memset(&f, 0, sizeof(f));
    mmr_status st = frame_from_view(frame, f);
    if (st != MMR_STATUS_OK) return st;
    return emit_buffer(encode(f), out);
}

mmr_status outside_scope(const char *what) {
    return finish(MMR_STATUS_UNSUPPORTED, std::string("unsupported: ") + what +
                                              " is outside this library, which implements the MJPEG and DV25 paths");
}

}  // namespace

namespace mmr {

void set_last_error(int32_t status, const char *message) {
    if (status == MMR_STATUS_OK) g_last_error.clear();
    else g_last_error.assign(message);
}

}  // namespace mmr

struct mmr_gpu_context {
    mmr::EnginePool *pool;
    double last_ms;
    uint32_t last_launches;
    mmr::EngineTimes times;
    mmr::GpuJpegEncoder *encoder = nullptr;  // created by the first encode batch
    std::mutex encoder_mu;
};

struct mmr_gpu_server {
    mmr::Server *server;
};

struct mmr_gpu_stream {
    mmr::Stream *stream;
};

namespace {

// One packet of a decoder session, from send_packet until receive_frame hands
// its frame over: the packet copy and the output planes stay put (the entry is
// heap-held) while the server's engine reads and writes them.
struct SessionEntry {
    std::vector<uint8_t> packet;
    uint8_t *planes[3] = {nullptr, nullptr, nullptr};
    void *dev = nullptr;  // device output of a session that delivers device frames
    size_t dev_bytes = 0;
    uint64_t tag = 0;
    uint64_t ticket = 0;
    bool done = false;  // result holds the outcome (the server has forgotten the ticket)
    Item result;
};

// The server the sessions of the process share (device 0), created with the
// first packet and kept until the process ends, like the v1 engine pool.
std::mutex g_session_server_mu;
mmr::Server *g_session_server = nullptr;

mmr::Server *session_server(std::string &err) {
    std::lock_guard<std::mutex> lock(g_session_server_mu);
    if (g_session_server) return g_session_server;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        err = "no CUDA device is available to the GPU decoder";
        return nullptr;
    }
    try {
        mmr::ServerConfig c;
        c.device = 0;
        c.engines = 4;
        c.max_batch = 16;
        c.memory_budget = 0;
        g_session_server = new mmr::Server(c);
    } catch (const std::exception &e) {
        err = std::string("could not initialise the GPU decoder: ") + e.what();
        return nullptr;
    }
    return g_session_server;
}

// Device buffers of the sessions' device frames (device 0): released frames keep
// their buffers here, up to kDevKeepBytes, for later frames of about the same size,
// so that steady decoding allocates nothing.
std::mutex g_devbuf_mu;
std::multimap<size_t, void *> g_devbuf_free;  // capacity -> buffer
size_t g_devbuf_free_bytes = 0;
constexpr size_t kDevKeepBytes = size_t(1) << 30;

// Runs f with device 0 current on this thread, then restores the caller's device.
template <class F>
cudaError_t on_device0(F &&f) {
    int prev = 0;
    cudaError_t e = cudaGetDevice(&prev);
    if (e != cudaSuccess) return e;
    if ((e = cudaSetDevice(0)) != cudaSuccess) return e;
    e = f();
    cudaSetDevice(prev);
    return e;
}

// A buffer of at least `need` bytes (at most 1.5x that when reused); null when
// the device is out of memory.
void *devbuf_take(size_t need, size_t *capacity) {
    {
        std::lock_guard<std::mutex> lock(g_devbuf_mu);
        auto it = g_devbuf_free.lower_bound(need);
        if (it != g_devbuf_free.end() && it->first <= need + need / 2) {
            void *p = it->second;
            *capacity = it->first;
            g_devbuf_free_bytes -= it->first;
            g_devbuf_free.erase(it);
            return p;
        }
    }
    void *p = nullptr;
    if (on_device0([&] { return cudaMalloc(&p, need); }) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    *capacity = need;
    return p;
}

void devbuf_give(void *p, size_t capacity) {
    if (!p) return;
    {
        std::lock_guard<std::mutex> lock(g_devbuf_mu);
        if (g_devbuf_free_bytes + capacity <= kDevKeepBytes) {
            g_devbuf_free.emplace(capacity, p);
            g_devbuf_free_bytes += capacity;
            return;
        }
    }
    on_device0([&] { return cudaFree(p); });
}

}  // namespace

// Decoder trait state (mjpeg/src/codec.rs:16-19, dv/src/codec.rs:16-19): the
// configured flag and the queue of frames, here of packets on their way to frames.
struct mmr_gpu_decoder {
    uint32_t codec;
    bool configured = false;
    bool device_frames = false;  // MMR_SESSION_DEVICE_FRAMES
    std::deque<std::unique_ptr<SessionEntry>> queue;
    mmr::Server *server = nullptr;  // set by the first packet

    const char *kind() const { return codec == MMR_CODEC_DV ? "DV" : "Motion JPEG"; }

    // Waits until the entry's decode is over and keeps its outcome.
    void settle(SessionEntry &e) {
        if (e.done) return;
        server->wait(e.ticket, -1, &e.result, nullptr);
        e.done = true;
    }

    // Drops every queued packet (after its decode is over) with its planes.
    void clear() {
        for (auto &e : queue) {
            settle(*e);
            for (auto p : e->planes) free(p);
            devbuf_give(e->dev, e->dev_bytes);
        }
        queue.clear();
    }
};

namespace {

// The reference's InvalidState texts (mjpeg/src/codec.rs:39-71, dv/src/codec.rs:33-65).
mmr_status unconfigured(const mmr_gpu_decoder *d, const char *what) {
    return finish(MMR_STATUS_INVALID_STATE,
                  std::string("invalid state: ") + d->kind() + " decoder must be configured before " + what);
}

}  // namespace

namespace {

bool to_item(const mmr_gpu_item &g, Item &it, const char **err) {
    if (g.struct_size != sizeof(mmr_gpu_item)) {
        *err = "item struct_size mismatch";
        return false;
    }
    if (g.len > 0 && !g.data) {
        *err = "item data is null while length is nonzero";
        return false;
    }
    it.data = static_cast<const uint8_t *>(g.data);
    it.dev_data = static_cast<const uint8_t *>(g.device_data);
    it.len = g.len;
    it.codec = g.codec;
    it.output = g.output;
    it.flags = (g.flags & MMR_ITEM_CONCEAL) ? (uint32_t)mmr::kFlagConceal : 0u;
    it.out = static_cast<uint8_t *>(g.out);
    it.out_capacity = g.out_capacity;
    it.out_on_device = (g.flags & MMR_ITEM_OUT_DEVICE) != 0;
    return true;
}

void from_item(const Item &it, mmr_gpu_item &g) {
    g.status = it.status;
    g.format = it.format;
    g.range = it.range;
    g.width = it.width;
    g.height = it.height;
    g.plane_count = it.plane_count;
    for (int c = 0; c < 3; c++) {
        g.plane_offset[c] = it.plane_offset[c];
        g.plane_width[c] = it.plane_width[c];
        g.plane_height[c] = it.plane_height[c];
    }
    g.out_bytes = it.out_bytes;
    g.concealed_segments = (uint32_t)it.concealed.size();
    std::string m = it.status == MMR_STATUS_OK ? std::string() : with_prefix(it.status, it.message);
    snprintf(g.message, sizeof g.message, "%s", m.c_str());
}

}  // namespace

extern "C" {

MMR_API uint32_t mmr_abi_version(void) { return MMR_ABI_VERSION; }

MMR_API const char *mmr_version(void) { return kVersion; }

MMR_API size_t mmr_last_error_message(char *buffer, size_t capacity) {
    size_t required = g_last_error.size() + 1;
    if (buffer && capacity > 0) {
        size_t copied = g_last_error.size() < capacity - 1 ? g_last_error.size() : capacity - 1;
        memcpy(buffer, g_last_error.data(), copied);
        buffer[copied] = 0;
    }
    return required;
}

MMR_API mmr_status mmr_mjpeg_decode(const uint8_t *data, size_t len, mmr_video_frame *out_frame) {
    try {
        return decode_one(mmr::kCodecMjpeg, data, len, out_frame);
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API mmr_status mmr_dv_decode(const uint8_t *data, size_t len, mmr_video_frame *out_frame) {
    try {
        return decode_one(mmr::kCodecDv, data, len, out_frame);
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API mmr_status mmr_mpeg2_picture_count(const uint8_t *, size_t, size_t *out_count) {
    if (out_count) *out_count = 0;
    return outside_scope("MPEG-2 video");
}

MMR_API mmr_status mmr_mpeg2_decode_picture(const uint8_t *, size_t, size_t, mmr_video_frame *out_frame) {
    if (out_frame && out_frame->struct_size == sizeof(mmr_video_frame)) reset_frame(out_frame);
    return outside_scope("MPEG-2 video");
}

MMR_API void mmr_video_frame_free(mmr_video_frame *frame) {
    if (!frame) return;
    free_frame_planes(frame);
    reset_frame(frame);
}

MMR_API mmr_status mmr_mjpeg_encode(const mmr_video_frame_view *frame, uint8_t quality, mmr_buffer *out_buffer) {
    try {
        return encode_entry(frame, out_buffer, [&](const mmr::FrameIn &f) {
            mmr::JpegEncodeOptions o;
            o.quality = quality;
            return mmr::encode_jpeg(f, o);
        });
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API mmr_status mmr_dv_encode(const mmr_video_frame_view *frame, mmr_buffer *out_buffer) {
    try {
        return encode_entry(frame, out_buffer, [&](const mmr::FrameIn &f) { return mmr::encode_dv(f, mmr::kDvMode88); });
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API mmr_status mmr_mpeg2_encode(const mmr_video_frame_view *, size_t, const mmr_mpeg2_encode_options *,
                                    mmr_buffer *out_buffer) {
    if (out_buffer && out_buffer->struct_size == sizeof(mmr_buffer)) reset_buffer(out_buffer);
    return outside_scope("MPEG-2 video");
}

MMR_API mmr_status mmr_mpegts_mux_mpeg2(const uint8_t *, size_t, mmr_buffer *out_buffer) {
    if (out_buffer && out_buffer->struct_size == sizeof(mmr_buffer)) reset_buffer(out_buffer);
    return outside_scope("MPEG-TS");
}

MMR_API mmr_status mmr_mpegts_mux_mpeg2_mp2(const uint8_t *, size_t, const uint8_t *, size_t, mmr_buffer *out_buffer) {
    if (out_buffer && out_buffer->struct_size == sizeof(mmr_buffer)) reset_buffer(out_buffer);
    return outside_scope("MPEG-TS");
}

MMR_API mmr_status mmr_mpegts_demux_mpeg2(const uint8_t *, size_t, mmr_buffer *out_buffer) {
    if (out_buffer && out_buffer->struct_size == sizeof(mmr_buffer)) reset_buffer(out_buffer);
    return outside_scope("MPEG-TS");
}

MMR_API mmr_status mmr_mpegts_demux_mp2(const uint8_t *, size_t, mmr_buffer *out_buffer) {
    if (out_buffer && out_buffer->struct_size == sizeof(mmr_buffer)) reset_buffer(out_buffer);
    return outside_scope("MPEG-TS");
}

MMR_API void mmr_buffer_free(mmr_buffer *buffer) {
    if (!buffer) return;
    free(buffer->data);
    reset_buffer(buffer);
}

// ------------------------------------------------------------ GPU API ---

MMR_API mmr_status mmr_gpu_context_create(const mmr_gpu_config *config, mmr_gpu_context **out_context) {
    if (!out_context) return invalid_argument("out_context is null");
    *out_context = nullptr;
    int device = 0, engines = 4;
    if (config) {
        if (config->struct_size != sizeof(mmr_gpu_config)) return invalid_argument("config struct_size mismatch");
        device = config->device;
        if (config->engines) engines = (int)std::min<uint32_t>(config->engines, 16);
    }
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
        cudaGetLastError();
        return finish(MMR_STATUS_INTERNAL_ERROR, "no usable CUDA device for the GPU decoder");
    }
    try {
        mmr::EnginePool *pool = new mmr::EnginePool(device, engines);
        mmr_gpu_context *c = new mmr_gpu_context;
        c->pool = pool;
        c->last_ms = 0.0;
        c->last_launches = 0;
        *out_context = c;
        return finish(MMR_STATUS_OK, "");
    } catch (const std::exception &e) {
        return finish(MMR_STATUS_INTERNAL_ERROR, std::string("could not initialise the GPU decoder: ") + e.what());
    }
}

MMR_API void mmr_gpu_context_destroy(mmr_gpu_context *context) {
    if (!context) return;
    delete context->encoder;
    delete context->pool;
    delete context;
}

MMR_API mmr_status mmr_gpu_probe(uint32_t codec, const uint8_t *data, size_t len, mmr_gpu_frame_info *info) {
    if (!info) return invalid_argument("info is null");
    if (info->struct_size != sizeof(mmr_gpu_frame_info)) return invalid_argument("info struct_size mismatch");
    if (len > 0 && !data) return invalid_argument("data is null while length is nonzero");
    mmr::Probe p = mmr::probe_packet(codec, data, len);
    memset(info, 0, sizeof(*info));
    info->struct_size = sizeof(*info);
    info->status = p.status;
    info->format = p.format;
    info->range = p.range;
    info->width = p.width;
    info->height = p.height;
    info->plane_count = p.plane_count;
    for (int c = 0; c < 3; c++) {
        info->plane_width[c] = p.plane_width[c];
        info->plane_height[c] = p.plane_height[c];
    }
    info->planar_bytes = p.planar_bytes;
    info->rgb_bytes = p.rgb_bytes;
    return finish(MMR_STATUS_OK, "");
}

MMR_API mmr_status mmr_gpu_decode_batch(mmr_gpu_context *context, mmr_gpu_item *items, size_t count) {
    if (!context) return invalid_argument("context is null");
    if (count && !items) return invalid_argument("items is null");
    try {
        std::vector<Item> v(count);
        const char *err = nullptr;
        for (size_t i = 0; i < count; i++)
            if (!to_item(items[i], v[i], &err)) return invalid_argument(err);
        mmr::EngineTimes t;
        int32_t st = context->pool->decode(v.data(), count, &t);
        context->last_ms = t.device_ms;
        context->last_launches = context->pool->last_launches();
        context->times = t;
        for (size_t i = 0; i < count; i++) from_item(v[i], items[i]);
        if (st != mmr::kOk) return finish(MMR_STATUS_INTERNAL_ERROR, "CUDA device failure during batch decode");
        return finish(MMR_STATUS_OK, "");
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API double mmr_gpu_last_batch_ms(const mmr_gpu_context *context) { return context ? context->last_ms : 0.0; }

MMR_API uint32_t mmr_gpu_last_batch_launches(const mmr_gpu_context *context) {
    return context ? context->last_launches : 0;
}

MMR_API mmr_status mmr_gpu_autotune(mmr_gpu_context *context, mmr_gpu_item *items, size_t count,
                                    mmr_gpu_tune_entry *report, size_t capacity, size_t *report_count) {
    if (!context) return invalid_argument("context is null");
    if (count && !items) return invalid_argument("items is null");
    try {
        std::vector<Item> v(count);
        const char *err = nullptr;
        for (size_t i = 0; i < count; i++)
            if (!to_item(items[i], v[i], &err)) return invalid_argument(err);
        const std::vector<mmr::TuneResult> r = context->pool->autotune(v.data(), count);
        for (size_t k = 0; k < r.size() && report && k < capacity; k++) {
            mmr_gpu_tune_entry &o = report[k];
            memset(&o, 0, sizeof(o));
            o.frame_class = r[k].frame_class;
            o.kind = r[k].kind;
            o.frames = r[k].frames;
            if (r[k].kind == 0) {
                o.slice_bits = r[k].slice_bits;
                for (int c = 0; c < 4; c++) o.entropy_ms[c] = r[k].ms[c];
            } else {
                o.strip_mcus = r[k].strip_mcus;
                for (int c = 0; c < 2; c++) o.transform_ms[c] = r[k].ms[c];
            }
        }
        if (report_count) *report_count = r.size();
        return finish(MMR_STATUS_OK, "");
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

namespace {

// A tuning table from the caller's entries; nullptr (with the message) when one is invalid.
const char *to_table(const mmr_gpu_tune_entry *entries, size_t count, std::vector<mmr::TuneResult> &table) {
    table.assign(count, mmr::TuneResult());
    for (size_t k = 0; k < count; k++) {
        const mmr_gpu_tune_entry &e = entries[k];
        if (e.kind > 1) return "tune entry kind must be 0 (slice size) or 1 (strip)";
        if (e.kind == 0 && (e.slice_bits < 128 || e.slice_bits % 32 || e.slice_bits > (1u << 20)))
            return "slice bits must be a multiple of 32 in 128..1048576";
        table[k].kind = e.kind;
        table[k].frame_class = e.frame_class;
        table[k].slice_bits = e.slice_bits;
        table[k].strip_mcus = e.strip_mcus;
    }
    return nullptr;
}

}  // namespace

MMR_API mmr_status mmr_gpu_set_tuning(mmr_gpu_context *context, const mmr_gpu_tune_entry *entries, size_t count) {
    if (!context) return invalid_argument("context is null");
    if (count && !entries) return invalid_argument("entries is null");
    std::vector<mmr::TuneResult> table;
    if (const char *err = to_table(entries, count, table)) return invalid_argument(err);
    try {
        context->pool->set_tuning(table);
        return finish(MMR_STATUS_OK, "");
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API mmr_status mmr_gpu_set_graphs(mmr_gpu_context *context, int enable) {
    if (!context) return invalid_argument("context is null");
    context->pool->set_graphs(enable != 0);
    return finish(MMR_STATUS_OK, "");
}

MMR_API mmr_status mmr_gpu_set_slice_bits(mmr_gpu_context *context, uint32_t bits) {
    if (!context) return invalid_argument("context is null");
    if (!context->pool->set_slice_bits(bits)) return invalid_argument("slice bits must be 0 or a multiple of 32 in 128..1048576");
    return finish(MMR_STATUS_OK, "");
}

MMR_API mmr_status mmr_gpu_last_batch_stats(const mmr_gpu_context *context, mmr_gpu_batch_stats *stats) {
    if (!context || !stats) return invalid_argument("context or stats is null");
    if (stats->struct_size != sizeof(mmr_gpu_batch_stats)) return invalid_argument("stats struct_size mismatch");
    const mmr::EngineTimes &t = context->times;
    stats->total_ms = t.device_ms;
    stats->upload_ms = t.upload_ms;
    stats->scan_ms = t.scan_ms;
    stats->entropy_ms = t.entropy_ms;
    stats->idct_ms = t.idct_ms;
    stats->dv_ms = t.dv_ms;
    stats->rgb_ms = t.rgb_ms;
    stats->download_ms = t.download_ms;
    stats->input_bytes = t.input_bytes;
    stats->output_bytes = t.output_bytes;
    stats->jpeg_blocks = t.jpeg_blocks;
    stats->dv_blocks = t.dv_blocks;
    stats->rgb_pixels = t.rgb_pixels;
    stats->idct_exact_samples = t.idct_exact_samples;
    stats->launches = context->last_launches;
    stats->slice_spec_ms = t.slice_spec_ms;
    stats->slice_sync_ms = t.slice_sync_ms;
    stats->slice_decode_ms = t.slice_decode_ms;
    stats->graph_replays = t.graph_replays;
    stats->slices = t.slices;
    stats->slices_redone = t.slices_redone;
    stats->dv_segment_ms = t.dv_segment_ms;
    stats->dv_idct_ms = t.dv_idct_ms;
    stats->slices_redone_whole = t.slices_redone_whole;
    return finish(MMR_STATUS_OK, "");
}

MMR_API mmr_status mmr_mjpeg_encode_ex(const mmr_video_frame_view *frame, const mmr_jpeg_encode_options *options,
                                       mmr_buffer *out_buffer) {
    if (!options) return invalid_argument("options is null");
    if (options->struct_size != sizeof(mmr_jpeg_encode_options)) return invalid_argument("options struct_size mismatch");
    try {
        return encode_entry(frame, out_buffer, [&](const mmr::FrameIn &f) {
            mmr::JpegEncodeOptions o;
            o.quality = options->quality;
            o.annex_k = options->annex_k_huffman != 0;
            o.restart_interval = options->restart_interval;
            return mmr::encode_jpeg(f, o);
        });
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API mmr_status mmr_dv_encode_ex(const mmr_video_frame_view *frame, uint32_t mode_policy, mmr_buffer *out_buffer) {
    if (mode_policy > MMR_DV_MODE_ACTIVITY) return invalid_argument("unknown DV mode policy");
    try {
        return encode_entry(frame, out_buffer, [&](const mmr::FrameIn &f) { return mmr::encode_dv(f, mode_policy); });
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API mmr_status mmr_gpu_server_create(const mmr_gpu_server_config *config, mmr_gpu_server **out_server) {
    if (!out_server) return invalid_argument("out_server is null");
    *out_server = nullptr;
    if (!config) return invalid_argument("config is null");
    if (config->struct_size != sizeof(mmr_gpu_server_config)) return invalid_argument("config struct_size mismatch");
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || config->device < 0 || config->device >= count) {
        cudaGetLastError();
        return finish(MMR_STATUS_INTERNAL_ERROR, "no usable CUDA device for the GPU decoder");
    }
    try {
        mmr::ServerConfig c;
        c.device = config->device;
        c.engines = config->engines ? (int)std::min<uint32_t>(config->engines, 16) : 3;
        c.max_batch = config->max_batch ? config->max_batch : 64;
        c.memory_budget = config->memory_budget;
        *out_server = new mmr_gpu_server{new mmr::Server(c)};
        return finish(MMR_STATUS_OK, "");
    } catch (const std::exception &e) {
        return finish(MMR_STATUS_INTERNAL_ERROR, std::string("could not initialise the GPU server: ") + e.what());
    }
}

MMR_API void mmr_gpu_server_destroy(mmr_gpu_server *server) {
    if (!server) return;
    delete server->server;
    delete server;
}

MMR_API mmr_status mmr_gpu_server_submit(mmr_gpu_server *server, const mmr_gpu_item *item, uint64_t *ticket) {
    if (!server || !item || !ticket) return invalid_argument("server, item or ticket is null");
    try {
        Item it;
        const char *err = nullptr;
        if (!to_item(*item, it, &err)) return invalid_argument(err);
        if (server->server->submit(it, ticket) != mmr::kOk)
            return invalid_argument("request exceeds the server's device-memory budget per engine");
        return finish(MMR_STATUS_OK, "");
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API mmr_status mmr_gpu_server_wait(mmr_gpu_server *server, uint64_t ticket, int64_t timeout_ns,
                                       mmr_gpu_item *result, double *latency_ms) {
    if (!server || !result) return invalid_argument("server or result is null");
    if (result->struct_size != sizeof(mmr_gpu_item)) return invalid_argument("result struct_size mismatch");
    try {
        Item it;
        double lat = 0;
        if (!server->server->wait(ticket, timeout_ns, &it, &lat)) {
            if (!server->server->known(ticket)) return invalid_argument("unknown ticket");
            return finish(MMR_STATUS_INVALID_STATE, "request not complete before the timeout");
        }
        from_item(it, *result);
        if (latency_ms) *latency_ms = lat;
        return finish(MMR_STATUS_OK, "");
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API mmr_status mmr_gpu_server_stats_get(mmr_gpu_server *server, int reset, mmr_gpu_server_stats *stats) {
    if (!server || !stats) return invalid_argument("server or stats is null");
    if (stats->struct_size != sizeof(mmr_gpu_server_stats)) return invalid_argument("stats struct_size mismatch");
    const mmr::ServerStats s = server->server->stats(reset != 0);
    stats->submitted = s.submitted;
    stats->completed = s.completed;
    stats->failed = s.failed;
    stats->rejected = s.rejected;
    stats->batches = s.batches;
    stats->in_flight = s.in_flight;
    stats->queued = s.queued;
    stats->p50_ms = s.p50_ms;
    stats->p99_ms = s.p99_ms;
    stats->max_ms = s.max_ms;
    stats->mean_ms = s.mean_ms;
    stats->frames_per_s = s.frames_per_s;
    stats->window_s = s.window_s;
    stats->peak_budget_bytes = s.peak_budget_bytes;
    return finish(MMR_STATUS_OK, "");
}

MMR_API mmr_status mmr_gpu_server_replay(mmr_gpu_server *server, mmr_gpu_item *items, size_t count,
                                         const int64_t *arrival_ns, double *latency_ms, int64_t *max_lag_ns) {
    if (!server) return invalid_argument("server is null");
    if (count && (!items || !arrival_ns || !latency_ms)) return invalid_argument("items, arrival_ns or latency_ms is null");
    try {
        std::vector<Item> v(count);
        const char *err = nullptr;
        for (size_t i = 0; i < count; i++) {
            if (!to_item(items[i], v[i], &err)) return invalid_argument(err);
            if (i && arrival_ns[i] < arrival_ns[i - 1]) return invalid_argument("arrival times must not decrease");
        }
        server->server->replay(v.data(), count, arrival_ns, latency_ms, max_lag_ns);
        for (size_t i = 0; i < count; i++) from_item(v[i], items[i]);
        return finish(MMR_STATUS_OK, "");
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API mmr_status mmr_gpu_server_set_tuning(mmr_gpu_server *server, const mmr_gpu_tune_entry *entries,
                                             size_t count) {
    if (!server) return invalid_argument("server is null");
    if (count && !entries) return invalid_argument("entries is null");
    std::vector<mmr::TuneResult> table;
    if (const char *err = to_table(entries, count, table)) return invalid_argument(err);
    try {
        server->server->set_tuning(table);
        return finish(MMR_STATUS_OK, "");
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API mmr_status mmr_gpu_decoder_create(uint32_t codec, mmr_gpu_decoder **out_decoder) {
    if (!out_decoder) return invalid_argument("out_decoder is null");
    *out_decoder = nullptr;
    if (codec != MMR_CODEC_MJPEG && codec != MMR_CODEC_DV) return invalid_argument("unknown codec");
    mmr_gpu_decoder *d = new (std::nothrow) mmr_gpu_decoder();
    if (!d) return finish(MMR_STATUS_INTERNAL_ERROR, "out of host memory");
    d->codec = codec;
    *out_decoder = d;
    return finish(MMR_STATUS_OK, "");
}

MMR_API void mmr_gpu_decoder_destroy(mmr_gpu_decoder *decoder) {
    if (!decoder) return;
    decoder->clear();
    delete decoder;
}

// configure (mjpeg/src/codec.rs:22-37, dv/src/codec.rs:22-31).
MMR_API mmr_status mmr_gpu_decoder_configure(mmr_gpu_decoder *decoder, const char *codec_id, const char *media_type) {
    if (!decoder || !codec_id || !media_type) return invalid_argument("decoder, codec_id or media_type is null");
    const bool video = strcmp(media_type, "video") == 0;
    if (decoder->codec == MMR_CODEC_DV) {
        if (strcmp(codec_id, "video/dv") != 0 || !video)
            return finish(MMR_STATUS_INVALID_DATA, "invalid data: DV decoder requires a video/dv video descriptor");
    } else {
        if (strcmp(codec_id, "video/mjpeg") != 0)
            return finish(MMR_STATUS_INVALID_DATA,
                          std::string("invalid data: expected video/mjpeg, received ") + codec_id);
        if (!video)
            return finish(MMR_STATUS_INVALID_DATA,
                          "invalid data: Motion JPEG decoder requires a video stream descriptor");
    }
    try {
        decoder->clear();
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
    decoder->configured = true;
    return finish(MMR_STATUS_OK, "");
}

// send_packet (mjpeg/src/codec.rs:39-53, dv/src/codec.rs:33-47), queued instead of
// decoded before returning.
MMR_API mmr_status mmr_gpu_decoder_send_packet(mmr_gpu_decoder *decoder, const uint8_t *data, size_t len,
                                               uint64_t user_tag) {
    if (!decoder) return invalid_argument("decoder is null");
    if (!decoder->configured) return unconfigured(decoder, "receiving packets");
    if (len > 0 && !data) return invalid_argument("data is null while length is nonzero");
    try {
        if (!decoder->server) {
            std::string err;
            decoder->server = session_server(err);
            if (!decoder->server) return finish(MMR_STATUS_INTERNAL_ERROR, err);
        }
        auto e = std::make_unique<SessionEntry>();
        e->packet.assign(data, data + len);
        e->tag = user_tag;
        Item it;
        it.data = e->packet.data();
        it.len = len;
        it.codec = decoder->codec;
        it.output = mmr::kOutPlanar;
        mmr::Probe pr = mmr::probe_packet(decoder->codec, it.data, len);
        if (decoder->device_frames) {
            if (pr.status == MMR_STATUS_OK && pr.format != 0 && pr.planar_bytes) {
                e->dev = devbuf_take(pr.planar_bytes, &e->dev_bytes);
                if (!e->dev) return finish(MMR_STATUS_INTERNAL_ERROR, "out of device memory");
                it.out = static_cast<uint8_t *>(e->dev);
                it.out_capacity = e->dev_bytes;
                it.out_on_device = true;
            }
        } else if (!alloc_planes(pr, it, e->planes)) {
            return finish(MMR_STATUS_INTERNAL_ERROR, "out of host memory");
        }
        if (decoder->server->submit(it, &e->ticket) != mmr::kOk) {  // only a memory budget refuses; this one has none
            for (auto p : e->planes) free(p);
            devbuf_give(e->dev, e->dev_bytes);
            return finish(MMR_STATUS_INTERNAL_ERROR, "the GPU decoder refused the packet");
        }
        decoder->queue.push_back(std::move(e));
        return finish(MMR_STATUS_OK, "");
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

// receive_frame (mjpeg/src/codec.rs:55-62, dv/src/codec.rs:49-56).
MMR_API mmr_status mmr_gpu_decoder_receive_frame(mmr_gpu_decoder *decoder, int64_t wait_ns,
                                                 mmr_video_frame *out_frame, uint64_t *out_user_tag,
                                                 int *out_has_frame) {
    if (!decoder || !out_has_frame) return invalid_argument("decoder or out_has_frame is null");
    *out_has_frame = 0;
    if (!decoder->configured) return unconfigured(decoder, "receiving frames");
    if (mmr_status st = check_frame(out_frame)) return st;
    reset_frame(out_frame);
    if (decoder->device_frames)
        return finish(MMR_STATUS_INVALID_STATE,
                      "invalid state: the session delivers device frames (mmr_gpu_decoder_receive_device_frame)");
    if (decoder->queue.empty()) return finish(MMR_STATUS_OK, "");
    try {
        SessionEntry &e = *decoder->queue.front();
        if (!e.done) {
            if (!decoder->server->wait(e.ticket, wait_ns, &e.result, nullptr)) return finish(MMR_STATUS_OK, "");
            e.done = true;
        }
        std::unique_ptr<SessionEntry> owned = std::move(decoder->queue.front());
        decoder->queue.pop_front();
        if (out_user_tag) *out_user_tag = owned->tag;
        const Item &it = owned->result;
        if (it.status != MMR_STATUS_OK) {
            for (auto p : owned->planes) free(p);
            return finish(it.status, with_prefix(it.status, it.message));
        }
        fill_frame(it, owned->planes, out_frame);
        *out_has_frame = 1;
        return finish(MMR_STATUS_OK, "");
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

// flush (mjpeg/src/codec.rs:64-71, dv/src/codec.rs:58-65): the reference has no
// delayed frames; here it waits until every queued packet is decoded.
MMR_API mmr_status mmr_gpu_decoder_flush(mmr_gpu_decoder *decoder) {
    if (!decoder) return invalid_argument("decoder is null");
    if (!decoder->configured) return unconfigured(decoder, "flushing");
    try {
        for (auto &e : decoder->queue) decoder->settle(*e);
        return finish(MMR_STATUS_OK, "");
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API mmr_status mmr_gpu_decoder_set_output(mmr_gpu_decoder *decoder, uint32_t where) {
    if (!decoder) return invalid_argument("decoder is null");
    if (where != MMR_SESSION_HOST_FRAMES && where != MMR_SESSION_DEVICE_FRAMES)
        return invalid_argument("unknown session output");
    if (!decoder->queue.empty())
        return finish(MMR_STATUS_INVALID_STATE, "invalid state: the session output changes only with no packet queued");
    decoder->device_frames = where == MMR_SESSION_DEVICE_FRAMES;
    return finish(MMR_STATUS_OK, "");
}

MMR_API mmr_status mmr_gpu_decoder_receive_device_frame(mmr_gpu_decoder *decoder, int64_t wait_ns,
                                                        mmr_gpu_device_frame *out_frame, uint64_t *out_user_tag,
                                                        int *out_has_frame) {
    if (!decoder || !out_has_frame) return invalid_argument("decoder or out_has_frame is null");
    *out_has_frame = 0;
    if (!decoder->configured) return unconfigured(decoder, "receiving frames");
    if (!out_frame) return invalid_argument("out_frame is null");
    if (out_frame->struct_size != sizeof(mmr_gpu_device_frame)) return invalid_argument("out_frame struct_size mismatch");
    memset(out_frame, 0, sizeof(*out_frame));
    out_frame->struct_size = sizeof(mmr_gpu_device_frame);
    if (!decoder->device_frames)
        return finish(MMR_STATUS_INVALID_STATE,
                      "invalid state: the session delivers host frames (mmr_gpu_decoder_receive_frame)");
    if (decoder->queue.empty()) return finish(MMR_STATUS_OK, "");
    try {
        SessionEntry &e = *decoder->queue.front();
        if (!e.done) {
            if (!decoder->server->wait(e.ticket, wait_ns, &e.result, nullptr)) return finish(MMR_STATUS_OK, "");
            e.done = true;
        }
        std::unique_ptr<SessionEntry> owned = std::move(decoder->queue.front());
        decoder->queue.pop_front();
        if (out_user_tag) *out_user_tag = owned->tag;
        const Item &it = owned->result;
        if (it.status != MMR_STATUS_OK) {
            devbuf_give(owned->dev, owned->dev_bytes);
            return finish(it.status, with_prefix(it.status, it.message));
        }
        out_frame->format = it.format;
        out_frame->range = it.range;
        out_frame->width = it.width;
        out_frame->height = it.height;
        out_frame->plane_count = it.plane_count;
        for (size_t c = 0; c < it.plane_count && c < MMR_MAX_PLANES; c++) {
            out_frame->planes[c] = static_cast<const uint8_t *>(owned->dev) + it.plane_offset[c];
            out_frame->plane_width[c] = it.plane_width[c];
            out_frame->plane_height[c] = it.plane_height[c];
        }
        out_frame->buffer = owned->dev;
        out_frame->buffer_bytes = owned->dev_bytes;
        *out_has_frame = 1;
        return finish(MMR_STATUS_OK, "");
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API void mmr_gpu_device_frame_release(mmr_gpu_device_frame *frame) {
    if (!frame || frame->struct_size != sizeof(mmr_gpu_device_frame)) return;
    devbuf_give(frame->buffer, frame->buffer_bytes);
    memset(frame, 0, sizeof(*frame));
    frame->struct_size = sizeof(mmr_gpu_device_frame);
}

MMR_API mmr_status mmr_gpu_server_set_slice_bits(mmr_gpu_server *server, uint32_t bits) {
    if (!server) return invalid_argument("server is null");
    if (!server->server->set_slice_bits(bits)) return invalid_argument("slice bits must be 0 or a multiple of 32 in 128..1048576");
    return finish(MMR_STATUS_OK, "");
}

MMR_API mmr_status mmr_gpu_stream_open(mmr_gpu_context *context, const uint8_t *data, size_t len,
                                       const char *input_name, mmr_gpu_stream **out_stream,
                                       mmr_gpu_stream_info *info) {
    if (!out_stream) return invalid_argument("out_stream is null");
    *out_stream = nullptr;
    if (!context) return invalid_argument("context is null");
    if (len > 0 && !data) return invalid_argument("data is null while length is nonzero");
    if (info && info->struct_size != sizeof(mmr_gpu_stream_info)) return invalid_argument("info struct_size mismatch");
    try {
        mmr::Stream *s = new mmr::Stream(*context->pool, data, len, input_name ? input_name : "input");
        if (info) {
            memset(info, 0, sizeof(*info));
            info->struct_size = sizeof(*info);
            info->kind = s->kind();
            info->frame_status = s->frame_status();
            info->frame_count = s->frame_count();
            info->y4m_bytes = s->y4m_bytes();
            info->candidates = s->candidates();
            info->upload_ms = s->upload_ms();
            info->scan_ms = s->scan_ms();
            snprintf(info->message, sizeof info->message, "%s", s->frame_message().c_str());
        }
        *out_stream = new mmr_gpu_stream{s};
        return finish(MMR_STATUS_OK, "");
    } catch (const std::exception &e) {
        return finish(MMR_STATUS_INTERNAL_ERROR, std::string("CUDA device failure: ") + e.what());
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API mmr_status mmr_gpu_stream_frame(const mmr_gpu_stream *stream, size_t index, uint64_t *offset,
                                        uint64_t *length) {
    if (!stream) return invalid_argument("stream is null");
    if (!offset || !length) return invalid_argument("offset or length is null");
    if (index >= stream->stream->frame_count()) return invalid_argument("frame index out of range");
    *offset = stream->stream->frame_offset(index);
    *length = stream->stream->frame_length(index);
    return finish(MMR_STATUS_OK, "");
}

MMR_API mmr_status mmr_gpu_stream_decode_y4m(mmr_gpu_stream *stream, uint8_t *out, size_t capacity,
                                             mmr_gpu_stream_result *result) {
    if (!stream) return invalid_argument("stream is null");
    if (!result) return invalid_argument("result is null");
    if (result->struct_size != sizeof(mmr_gpu_stream_result)) return invalid_argument("result struct_size mismatch");
    if (stream->stream->frame_count() && (!out || capacity < stream->stream->y4m_bytes()))
        return invalid_argument("output buffer is smaller than the stream's Y4M bytes");
    try {
        const mmr::StreamResult r = stream->stream->decode_y4m(out, capacity);
        memset(result, 0, sizeof(*result));
        result->struct_size = sizeof(*result);
        result->status = r.status;
        result->frames_written = r.frames_written;
        result->bytes_written = r.bytes_written;
        snprintf(result->message, sizeof result->message, "%s", r.message.c_str());
        if (r.status == MMR_STATUS_INTERNAL_ERROR) return finish(MMR_STATUS_INTERNAL_ERROR, r.message);
        return finish(MMR_STATUS_OK, "");
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API void mmr_gpu_stream_close(mmr_gpu_stream *stream) {
    if (!stream) return;
    delete stream->stream;
    delete stream;
}

MMR_API size_t mmr_gpu_jpeg_encode_bound(mmr_pixel_format format, size_t width, size_t height,
                                         uint16_t restart_interval) {
    return mmr::jpeg_encode_bound(format, width, height, restart_interval);
}

MMR_API mmr_status mmr_gpu_jpeg_encode_batch(mmr_gpu_context *context, const mmr_jpeg_encode_options *options,
                                             mmr_gpu_encode_item *items, size_t count) {
    if (!context) return invalid_argument("context is null");
    if (!options) return invalid_argument("options is null");
    if (options->struct_size != sizeof(mmr_jpeg_encode_options)) return invalid_argument("options struct_size mismatch");
    if (count && !items) return invalid_argument("items is null");
    try {
        for (size_t i = 0; i < count; i++)
            if (items[i].struct_size != sizeof(mmr_gpu_encode_item)) return invalid_argument("item struct_size mismatch");
        std::vector<mmr::EncodeItem> work;
        std::vector<size_t> index;
        for (size_t i = 0; i < count; i++) {
            mmr_gpu_encode_item &g = items[i];
            g.out_len = 0;
            g.message[0] = 0;
            mmr::EncodeItem it;
            memset(&it.frame, 0, sizeof(it.frame));
            if (g.frame.struct_size != sizeof(mmr_video_frame_view)) {
                g.status = MMR_STATUS_INVALID_ARGUMENT;
                snprintf(g.message, sizeof g.message, "invalid argument: frame struct_size is %zu, expected %zu",
                         g.frame.struct_size, sizeof(mmr_video_frame_view));
                continue;
            }
            const mmr_status st = frame_from_view(&g.frame, it.frame);  // the ABI's view checks (lib.rs:1061-1127)
            if (st != MMR_STATUS_OK) {
                g.status = st;
                snprintf(g.message, sizeof g.message, "%s", g_last_error.c_str());
                continue;
            }
            it.in_on_device = (g.flags & MMR_ITEM_IN_DEVICE) != 0;
            it.out_on_device = (g.flags & MMR_ITEM_OUT_DEVICE) != 0;
            it.out = g.out;
            it.out_capacity = g.out_capacity;
            work.push_back(it);
            index.push_back(i);
        }
        mmr::JpegEncodeOptions o;
        o.quality = options->quality;
        o.annex_k = options->annex_k_huffman != 0;
        o.restart_interval = options->restart_interval;
        int32_t st = mmr::kOk;
        {
            std::lock_guard<std::mutex> g(context->encoder_mu);
            if (!context->encoder) context->encoder = new mmr::GpuJpegEncoder(context->pool->device());
            st = context->encoder->encode(work.data(), work.size(), o);
        }
        for (size_t k = 0; k < work.size(); k++) {
            mmr_gpu_encode_item &g = items[index[k]];
            g.status = work[k].status;
            g.out_len = work[k].out_len;
            const std::string m = work[k].status == MMR_STATUS_OK ? std::string() : with_prefix(work[k].status, work[k].message);
            snprintf(g.message, sizeof g.message, "%s", m.c_str());
        }
        if (st != mmr::kOk) return finish(MMR_STATUS_INTERNAL_ERROR, "CUDA device failure during encode");
        return finish(MMR_STATUS_OK, "");
    } catch (const std::exception &e) {
        return finish(MMR_STATUS_INTERNAL_ERROR, std::string("could not run the GPU encoder: ") + e.what());
    } catch (...) {
        return finish(MMR_STATUS_INTERNAL_ERROR, "panic contained at MMRecode C API boundary");
    }
}

MMR_API mmr_status mmr_gpu_last_encode_stats(const mmr_gpu_context *context, mmr_gpu_encode_stats *stats) {
    if (!context) return invalid_argument("context is null");
    if (!stats) return invalid_argument("stats is null");
    if (stats->struct_size != sizeof(mmr_gpu_encode_stats)) return invalid_argument("stats struct_size mismatch");
    const mmr::EncodeStats t = context->encoder ? context->encoder->last_stats() : mmr::EncodeStats();
    stats->device_ms = t.device_ms;
    stats->blocks = t.blocks;
    stats->exact_coefficients = t.exact_coefficients;
    stats->bytes_out = t.bytes_out;
    return finish(MMR_STATUS_OK, "");
}

}  // extern "C"
