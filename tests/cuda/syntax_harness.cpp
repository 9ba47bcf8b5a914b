// Host-only harness for the marker parser shared by the host and the device
// (mmrecode_gb300/csrc/jpeg_syntax.h): the prefix up to the first SOS, the first
// scan's end found sequentially, then the tail, as the engine runs them.
#include <stddef.h>
#include <stdint.h>

#include "jpeg_syntax.h"

struct ParseOut {
    int32_t status;   // of the first parse error, 0 if none
    uint32_t kind;
    uint32_t offset;
    uint32_t width, height, ncomp, dri, scan_count, data_offset, ended_at_eoi;
};

extern "C" int mmr_test_parse_jpeg(const uint8_t *in, size_t len, ParseOut *out) {
    mmr::JpegHeader h;
    mmr::jpeg_parse_prefix(in, len, &h);
    if (h.err.kind == mmr::kDiagNone && h.prefix_done && h.have_sos) {
        size_t term = 0;
        mmr::Diag e{};
        if (mmr::jpeg_find_first_scan_end(in, len, &h, &term, &e)) mmr::jpeg_parse_tail(in, len, term, &h);
        else h.err = e;
    }
    out->status = h.err.kind == mmr::kDiagNone ? 0 : h.err.status;
    out->kind = h.err.kind;
    out->offset = h.err.offset;
    out->width = h.width;
    out->height = h.height;
    out->ncomp = h.ncomp;
    out->dri = h.dri;
    out->scan_count = h.scan_count;
    out->data_offset = h.data_offset;
    out->ended_at_eoi = h.ended_at_eoi;
    return 0;
}
