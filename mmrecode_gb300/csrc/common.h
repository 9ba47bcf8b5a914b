// Shared host/device definitions for the GB300 MJPEG / DV25 decode library.
#pragma once

#include <stddef.h>
#include <stdint.h>

#if defined(__CUDACC__)
#define MMR_HD __host__ __device__ __forceinline__
#define MMR_D __device__ __forceinline__
#else
#define MMR_HD inline
#define MMR_D inline
#endif

namespace mmr {

// Status codes of the C ABI (crates/capi/src/lib.rs:26-32).
enum Status : int32_t {
    kOk = 0,
    kInvalidArgument = 1,
    kInvalidData = 2,
    kUnsupported = 3,
    kInvalidState = 4,
    kIoError = 5,
    kInternal = 100,
};

// Pixel formats and ranges (crates/capi/src/lib.rs:34-42).
enum PixelFormat : uint32_t { kGray8 = 1, kYuv420 = 2, kYuv422 = 3, kYuv444 = 4, kYuv411 = 5 };
enum ColorRange : uint32_t { kRangeUnspecified = 0, kRangeFull = 1, kRangeLimited = 2 };

// Output layouts of the batch API.
enum OutputKind : uint32_t { kOutPlanar = 0, kOutRgb24 = 1 };

// One diagnostic, produced on either side and rendered to text on the host.
// `kind` selects the reference's message; offset/aux/aux2 carry its arguments.
struct Diag {
    int32_t status;
    uint16_t kind;
    uint16_t pad;
    uint32_t offset;
    uint32_t aux;
    uint32_t aux2;
};

// Every failure the reference decode path can report, keyed to its source.
enum DiagKind : uint16_t {
    kDiagNone = 0,
    // crates/codecs/mjpeg/src/parser.rs
    kJExpectFF,           // :95  "expected JPEG marker prefix 0xff"
    kJTruncMarker,        // :104 "truncated marker"
    kJStuffedOutside,     // :106 "stuffed 0xff byte outside entropy-coded data"
    kJExpectSoi,          // :20  "expected SOI as the first marker"
    kJTruncLength,        // :112 "truncated segment length"
    kJBadLength,          // :50  "segment length must include its two length bytes"
    kJTruncPayload,       // :56  "truncated {marker} payload" (aux = marker code)
    kJSofShort,           // :151
    kJSofNoComp,          // :155
    kJSofSize,            // :159 (aux = count, aux2 = payload bytes)
    kJSofPrecision,       // :168
    kJSofWidth,           // :174
    kJSofSampling,        // :186
    kJSofTq,              // :191
    kJDqtPrecision,       // :215
    kJDqtId,              // :219
    kJDqtTrunc,           // :230
    kJDqtEmpty,           // :248
    kJDhtClass,           // :260
    kJDhtId,              // :264
    kJDhtTruncCounts,     // :272
    kJDhtTruncSymbols,    // :279
    kJDhtEmpty,           // :293
    kJDriSize,            // :127
    kJSosEmpty,           // :299
    kJSosNoComp,          // :303
    kJSosSize,            // :307 (aux = count, aux2 = payload bytes)
    kJSosSelector,        // :320
    kJJfifShort,          // :343
    kJJfifThumb,          // :349
    kJScanTruncMarker,    // :393 "truncated marker in entropy-coded data"
    kJScanNoTerminator,   // :413 "entropy-coded scan has no terminating marker"
    // crates/codecs/mjpeg/src/decoder.rs prologue
    kJNoSof,              // :142 "JPEG has no baseline SOF0 frame header"
    kJScanCount,          // :198 (aux = scan count) Unsupported
    kJDnlHeight,          // :225 Unsupported
    kJPartialScan,        // :230 Unsupported
    kJNotBaseline,        // :240 Unsupported
    kJScanSelect,         // :250 (aux = component id)
    kJHuffInconsistent,   // entropy.rs:25 (aux = table id)
    kJHuffOversub,        // entropy.rs:38 (aux = table id, aux2 = length)
    kJMissingQuant,       // :421 (aux = component id, aux2 = table)
    kJQuant16,            // :428 Unsupported
    kJMissingDc,          // :478 (aux = table)
    kJMissingAc,          // :486 (aux = table)
    kJPanic,              // :470 `.expect` in make_scan_decoders -> C ABI status 100
    // entropy decode (entropy.rs, decoder.rs:495-548); offset = source byte offset
    kJEndOfData,          // entropy.rs:147 "unexpected end of entropy-coded data"
    kJTruncEntropyMarker, // entropy.rs:156 "truncated entropy marker"
    kJMarkerInData,       // entropy.rs:161 (aux = marker code)
    kJNoHuffCode,         // entropy.rs:69
    kJDcCategory,         // decoder.rs:505
    kJAcZeroSize,         // decoder.rs:527
    kJZrlOverrun,         // decoder.rs:531
    kJAcCategory,         // decoder.rs:536
    kJAcRun,              // decoder.rs:540
    kJDcPredOverflow,     // decoder.rs:510
    kJDcDeqOverflow,      // decoder.rs:514
    kJExpectRst,          // entropy.rs:116 "expected restart marker at MCU boundary"
    kJTruncRst,           // entropy.rs:125 "truncated restart marker"
    kJRstMismatch,        // entropy.rs:129 (aux = expected, aux2 = code)
    kJExtendTooLong,      // entropy.rs:173 (unreachable after category checks)
    // decoder.rs:98-126 into_video_frame
    kJFormatComponents,   // Unsupported
    kJFormatChroma,       // Unsupported
    // crates/codecs/dv
    kDvShortHeader,       // profile.rs:113 (aux = len)
    kDvNotHeader,         // profile.rs:118
    kDvLength,            // profile.rs:93 (aux = expected, aux2 = len)
    kDvDamagedId,         // decoder.rs:168 (aux = slot, aux2 = sequence)
    kDvIncomplete,        // decoder.rs:181 (aux = slot, aux2 = sequence)
    kDvBadVlc,            // decoder.rs:278 (unreachable: the VLC code is complete)
    // library / environment
    kOutputCapacity,      // caller's output buffer is too small
    kDeviceError,         // CUDA failure
    kUnknownCodec,
};

MMR_HD int32_t diag_status(uint16_t kind) {
    switch (kind) {
    case kDiagNone:
        return kOk;
    case kJScanCount:
    case kJDnlHeight:
    case kJPartialScan:
    case kJNotBaseline:
    case kJQuant16:
    case kJFormatComponents:
    case kJFormatChroma:
        return kUnsupported;
    case kJPanic:
    case kDeviceError:
        return kInternal;
    case kOutputCapacity:
    case kUnknownCodec:
        return kInvalidArgument;
    default:
        return kInvalidData;
    }
}

// 0x80 in each byte of x that is zero, else 0 (exact: (x & 0x7f) + 0x7f never
// carries out of its byte).
MMR_HD uint32_t zero_bytes(uint32_t x) { return ~(((x & 0x7f7f7f7fu) + 0x7f7f7f7fu) | x | 0x7f7f7f7fu); }

// Nonzero iff some byte of w is 0xFF (the borrow test for a zero byte of ~w,
// exact as a test for any).
MMR_HD uint32_t any_ff(uint32_t w) { return (~w - 0x01010101u) & w & 0x80808080u; }

MMR_HD Diag make_diag(uint16_t kind, uint32_t offset = 0, uint32_t aux = 0, uint32_t aux2 = 0) {
    Diag d;
    d.status = diag_status(kind);
    d.kind = kind;
    d.pad = 0;
    d.offset = offset;
    d.aux = aux;
    d.aux2 = aux2;
    return d;
}

}  // namespace mmr
