// DV25 decode that allocates nothing (mmr_dv_decode_static in mmrecode_gpu.h).
//
// Meant for callers that must not allocate memory while decoding: a real-time
// capture or playback thread that cannot afford cudaMalloc's implicit device
// synchronisation, a host application whose memory is budgeted up front, or
// an embedding runtime that forbids allocations outside its own arena. Every
// device byte this path uses lives in one file-scope array, g_dv_scratch,
// sized for one DV25 frame of either system (kDvStaticScratchBytes, 2.25 MiB);
// every GPU that loads the library holds that array until the process exits.
// The caller passes the packet and the output buffer in host memory.
//
// The first call on a device sets that device up (looks up the array's device
// address with cudaGetSymbolAddress and writes the VLC lookup table into it),
// so that first call should come before any stream capture. All calls share
// the array and it keeps the last call's contents: each call clears what must
// start at zero, and calls that overlap on the GPU (from several threads on the
// same device) race on it -- serialise them.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <mutex>
#include <string>

#include "../../include/mmrecode_gpu.h"
#include "dv_vlc.h"
#include "exact_fixed.h"
#include "engine.h"
#include "last_error.h"
#include "kernels.h"
#include "plan.h"
#include "tables.h"

namespace mmr {
namespace {

constexpr size_t kDvStaticScratchBytes = 2304u * 1024u;  // 2.25 MiB
constexpr size_t kDvMaxInput = 144000;                   // one 625/50 frame
constexpr size_t kDvMaxPlanar = 720 * 576 + 2 * 360 * 288;
constexpr uint32_t kDvMaxSegments = 12 * 27;
constexpr uint32_t kDvMaxDif = 12 * 150;
constexpr size_t kVlcMaxEntries = kDvVlcMaxEntries;

static __device__ __align__(256) uint8_t g_dv_scratch[kDvStaticScratchBytes];

constexpr size_t a256(size_t v) { return (v + 255) / 256 * 256; }
// Layout of g_dv_scratch (byte offsets).
constexpr size_t kOffIn = 0;
constexpr size_t kOffOut = kOffIn + a256(kDvMaxInput);
constexpr size_t kOffFlags = kOffOut + a256(kDvMaxPlanar);
constexpr size_t kOffSegErr = kOffFlags + a256(kDvMaxDif);
constexpr size_t kOffModes = kOffSegErr + a256(kDvMaxSegments);
constexpr size_t kOffCoef = kOffModes + a256(kDvMaxSegments * 30);
constexpr size_t kOffVlc = kOffCoef + a256((size_t)kDvMaxSegments * 30 * 128);
constexpr size_t kOffFix = kOffVlc + a256(kVlcMaxEntries * 4);  // DV fixed-point weights (exact_fixed.h)
constexpr size_t kOffMeta = kOffFix + a256(2 * kFixEntries * sizeof(long long));
constexpr size_t kMetaBytes = 1024;
static_assert(kOffMeta + kMetaBytes <= kDvStaticScratchBytes, "DV static scratch layout exceeds the array");

struct Meta {  // per-call plan and state (lives at kOffMeta)
    DvFrame frame;
    DvState state;
    uint32_t item_ok;
    uint32_t seg_first[2];
    uint32_t dif_first[2];
};
static_assert(sizeof(Meta) <= kMetaBytes, "DV static metadata exceeds its region");

// The VLC lookup table (dv_vlc.h) and the fixed-point transform weights
// (exact_fixed.h), filled into static host arrays (no heap use) and copied into
// the scratch at set-up.
uint32_t g_vlc_host[kVlcMaxEntries];
long long g_fix_host[2 * kFixEntries];

std::mutex g_setup_mutex;
uint8_t *g_scratch_ptr[64] = {};  // device address of g_dv_scratch, per device

// Once per device, with that device current: looks up the array's device
// address and writes the VLC table into it. Later calls only confirm the
// address (a device reset reloads the module, possibly elsewhere); `redo`
// forces the table to be written again (the caller saw it cleared).
cudaError_t setup(int device, uint8_t **ptr, bool redo = false) {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_dv_scratch);
    if (e != cudaSuccess) return e;
    if (g_scratch_ptr[device] == (uint8_t *)p && !redo) {
        *ptr = g_scratch_ptr[device];
        return cudaSuccess;
    }
    size_t entries = fill_dv_vlc(g_vlc_host, kVlcMaxEntries);
    if (entries == 0) return cudaErrorInvalidValue;
    e = cudaMemcpy((uint8_t *)p + kOffVlc, g_vlc_host, entries * 4, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    build_dv_fixed(g_fix_host, g_fix_host + kFixEntries);
    e = cudaMemcpy((uint8_t *)p + kOffFix, g_fix_host, sizeof(g_fix_host), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return e;
    g_scratch_ptr[device] = (uint8_t *)p;
    *ptr = (uint8_t *)p;
    return cudaSuccess;
}

mmr_status fail(mmr_gpu_frame_info *info, mmr_status st, const char *m) {
    set_last_error(st, m);
    if (info) info->status = st;
    return st;
}

}  // namespace
}  // namespace mmr

using namespace mmr;

namespace {

// One decode of the validated packet with the set-up array at s. *table_word
// receives the first VLC table entry as the device held it during the call
// (never 0 once set up: it decodes the two-bit code 00).
mmr_status run_static(const uint8_t *data, size_t len, uint8_t *out, const Probe &pr, uint8_t *s, uint32_t *table_word,
                      mmr_gpu_frame_info *info);

}  // namespace

extern "C" MMR_API mmr_status mmr_dv_decode_static(const uint8_t *data, size_t len, uint8_t *out, size_t out_capacity,
                                                   mmr_gpu_frame_info *info) {
    char msg[200];
    if (!info || info->struct_size != sizeof(mmr_gpu_frame_info))
        return fail(nullptr, MMR_STATUS_INVALID_ARGUMENT, "invalid argument: info is null or its struct_size is wrong");
    size_t keep = info->struct_size;
    memset(info, 0, sizeof(*info));
    info->struct_size = keep;
    if (len > 0 && !data)
        return fail(info, MMR_STATUS_INVALID_ARGUMENT, "invalid argument: data is null while length is nonzero");
    if (len > kDvMaxInput) {
        snprintf(msg, sizeof msg, "invalid argument: packet of %zu bytes exceeds the %zu-byte frame the static scratch holds",
                 len, kDvMaxInput);
        return fail(info, MMR_STATUS_INVALID_ARGUMENT, msg);
    }
    // detect_profile (crates/codecs/dv/src/profile.rs:87-127)
    Probe pr = probe_packet(kCodecDv, data, len);
    if (pr.status != kOk) {
        snprintf(msg, sizeof msg, "invalid data: %s", render_message(pr.diag, data, len, 0, 0).c_str());
        return fail(info, pr.status, msg);
    }
    if (!out || out_capacity < pr.planar_bytes) {
        snprintf(msg, sizeof msg, "invalid argument: output buffer needs %zu bytes", pr.planar_bytes);
        return fail(info, MMR_STATUS_INVALID_ARGUMENT, msg);
    }
    int device = 0;
    uint8_t *s = nullptr;
    cudaError_t e = cudaGetDevice(&device);
    if (e == cudaSuccess) e = setup(device, &s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        snprintf(msg, sizeof msg, "CUDA device unavailable: %s", cudaGetErrorString(e));
        return fail(info, MMR_STATUS_INTERNAL_ERROR, msg);
    }
    uint32_t word = 0;
    mmr_status st = run_static(data, len, out, pr, s, &word, info);
    if (st != MMR_STATUS_INTERNAL_ERROR && word == 0) {
        // the table was cleared under us (the device was reset): set up again and redo the call
        e = setup(device, &s, true);
        if (e != cudaSuccess) {
            cudaGetLastError();
            snprintf(msg, sizeof msg, "CUDA device unavailable: %s", cudaGetErrorString(e));
            return fail(info, MMR_STATUS_INTERNAL_ERROR, msg);
        }
        st = run_static(data, len, out, pr, s, &word, info);
    }
    return st;
}

namespace {

mmr_status run_static(const uint8_t *data, size_t len, uint8_t *out, const Probe &pr, uint8_t *s, uint32_t *table_word,
                      mmr_gpu_frame_info *info) {
    char msg[200];
    cudaError_t e = cudaSuccess;
    bool pal = pr.format == kYuv420;
    uint32_t seqs = pal ? 12 : 10;
    Meta meta;
    memset(&meta, 0, sizeof(meta));
    DvFrame &F = meta.frame;
    F.in = s + kOffIn;
    F.planes = s + kOffOut;
    F.pal = pal;
    F.sequences = seqs;
    F.width = 720;
    F.height = pal ? 576 : 480;
    F.cw = pal ? 360 : 180;
    F.ch = pal ? 288 : 480;
    F.conceal = 0;
    F.item = 0;
    meta.state.bad_segment = 0xffffffffu;
    meta.item_ok = 1;
    meta.seg_first[1] = seqs * 27;
    meta.dif_first[1] = seqs * 150;
    Meta *dm = reinterpret_cast<Meta *>(s + kOffMeta);
    DvLaunch L;
    memset(&L, 0, sizeof(L));
    L.frames = &dm->frame;
    L.states = &dm->state;
    L.n_frames = 1;
    L.seg_first = dm->seg_first;
    L.n_segments = seqs * 27;
    L.dif_first = dm->dif_first;
    L.n_dif = seqs * 150;
    L.flags = s + kOffFlags;
    L.seg_err = s + kOffSegErr;
    L.coef = reinterpret_cast<int16_t *>(s + kOffCoef);
    L.modes = s + kOffModes;
    L.vlc = reinterpret_cast<const uint32_t *>(s + kOffVlc);
    L.fixw = reinterpret_cast<const long long *>(s + kOffFix);
    L.n_blocks = (uint64_t)seqs * 27 * 30;
    L.item_ok = &dm->item_ok;
    // the calling thread's default stream: no creation, no allocation, and no
    // implicit synchronisation with the application's other (blocking) streams
    cudaStream_t st = cudaStreamPerThread;
    e = cudaMemcpyAsync(s + kOffIn, data, len, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dm, &meta, sizeof(meta), cudaMemcpyHostToDevice, st);
    // (the segment decoder writes every coefficient of every block)
    if (e == cudaSuccess) {
        launch_dv_decode(L, st);
        launch_dv_idct(L, st);
        e = cudaGetLastError();
    }
    Meta back;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&back, dm, sizeof(back), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, s + kOffOut, pr.planar_bytes, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(table_word, s + kOffVlc, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        cudaGetLastError();
        snprintf(msg, sizeof msg, "CUDA device failure: %s", cudaGetErrorString(e));
        return fail(info, MMR_STATUS_INTERNAL_ERROR, msg);
    }
    if (back.state.bad_segment != 0xffffffffu) {
        Diag d = back.state.diag;
        snprintf(msg, sizeof msg, "invalid data: %s", render_message(d, nullptr, 0, 0, 0).c_str());
        return fail(info, d.status, msg);
    }
    info->status = MMR_STATUS_OK;
    info->format = pr.format;
    info->range = pr.range;
    info->width = pr.width;
    info->height = pr.height;
    info->plane_count = 3;
    for (int c = 0; c < 3; c++) {
        info->plane_width[c] = pr.plane_width[c];
        info->plane_height[c] = pr.plane_height[c];
    }
    info->planar_bytes = pr.planar_bytes;
    info->rgb_bytes = pr.rgb_bytes;
    set_last_error(MMR_STATUS_OK, "");
    return MMR_STATUS_OK;
}

}  // namespace
