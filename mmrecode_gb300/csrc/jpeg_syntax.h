// JPEG marker/segment parsing shared by host and device code.
//
// Restates crates/codecs/mjpeg/src/parser.rs (parse_jpeg and its segment
// parsers) and the table-collection half of decoder.rs, split in two:
//   parse_prefix()  SOI .. first SOS header (inclusive): everything the decode
//                   needs -- frame header, tables, restart interval, the start
//                   of the entropy-coded data;
//   parse_tail()    from the marker that ends the first scan to EOI: only its
//                   errors and colour-model facts can change the result.
// The entropy-coded bytes between them are scanned on the GPU (marker scan
// kernel), which reports the terminating marker's offset and code.
// Nothing here allocates; tables are referenced by their offset in the input.
#pragma once

#include "common.h"

namespace mmr {

struct JpegHeader {
    Diag err;  // first parse error in source order (kind == kDiagNone if none)
    // first SOF0 of the image
    uint8_t have_sof;
    uint8_t have_sos;
    uint8_t jfif;           // a JFIF APP0 was seen anywhere
    uint8_t prefix_done;    // parse_prefix reached the first SOS or EOI
    uint16_t width, height;
    uint16_t ncomp;         // SOF0 component count
    uint16_t sos_ncomp;
    uint32_t sof_comp_off;  // input offset of SOF0's 3-byte component records
    // first SOS
    uint32_t sos_marker_off;
    uint32_t sos_comp_off;  // input offset of SOS's 2-byte component records
    uint8_t ss, se, ah, al;
    uint32_t data_offset;   // first entropy-coded byte
    uint32_t scan_count;    // entropy scans in the whole image
    int32_t adobe;          // transform byte of the first "Adobe" APP14, -1 if none
    // tables defined before the first SOS (DecodeTables::collect, decoder.rs:264-299)
    uint16_t dri;
    uint8_t q_present[4];
    uint8_t q_sixteen[4];
    uint32_t q_off[4];      // offset of the 64 values (zigzag order)
    uint8_t h_present[8];   // index class*4 + id
    uint32_t h_off[8];      // offset of the 16 code counts; symbols follow
    uint16_t h_nsym[8];
    Diag huff_err;          // first HuffmanDecoder::new failure, in collect order
    uint8_t ended_at_eoi;   // prefix parse met EOI before any SOS
};

namespace jpeg_detail {

MMR_HD uint16_t be16(const uint8_t *p) { return (uint16_t)((p[0] << 8) | p[1]); }

MMR_HD bool has_length(uint8_t code) {
    if (code == 0x01) return false;
    if (code >= 0xd0 && code <= 0xd7) return false;
    if (code == 0xd8 || code == 0xd9) return false;
    return true;
}

// parser.rs:93-110
MMR_HD bool read_marker(const uint8_t *in, size_t len, size_t position, size_t *moff, uint8_t *code, size_t *after,
                        Diag *err) {
    if (position >= len || in[position] != 0xff) {
        *err = make_diag(kJExpectFF, (uint32_t)position);
        return false;
    }
    size_t code_offset = position + 1;
    while (code_offset < len && in[code_offset] == 0xff) code_offset++;
    if (code_offset >= len) {
        *err = make_diag(kJTruncMarker, (uint32_t)code_offset);
        return false;
    }
    uint8_t c = in[code_offset];
    if (c == 0x00) {
        *err = make_diag(kJStuffedOutside, (uint32_t)code_offset);
        return false;
    }
    *moff = position;
    *code = c;
    *after = code_offset + 1;
    return true;
}

// HuffmanDecoder::new validity (entropy.rs:18-55): counts must be non-empty and
// not oversubscribe any code length.
MMR_HD bool huffman_table_ok(const uint8_t *counts, uint8_t id, Diag *err) {
    uint32_t nsym = 0;
    for (int i = 0; i < 16; i++) nsym += counts[i];
    if (nsym == 0) {
        *err = make_diag(kJHuffInconsistent, 0, id);
        return false;
    }
    uint32_t code = 0;
    for (int li = 0; li < 16; li++) {
        uint32_t length = (uint32_t)li + 1;
        if (code + counts[li] > (1u << length)) {
            *err = make_diag(kJHuffOversub, 0, id, length);
            return false;
        }
        code += counts[li];
        code <<= 1;
    }
    return true;
}

// parse_segment_data (parser.rs:119-147) for one segment. `before_sos` selects
// whether table definitions are recorded for decoding.
MMR_HD bool parse_segment(const uint8_t *in, uint8_t code, size_t base, size_t n, bool before_sos, JpegHeader *h,
                          Diag *err) {
    const uint8_t *p = in + base;
    if (code == 0xc0) {  // parse_frame_header, parser.rs:149-204
        if (n < 6) return *err = make_diag(kJSofShort, (uint32_t)base), false;
        uint32_t count = p[5];
        if (count == 0) return *err = make_diag(kJSofNoComp, (uint32_t)(base + 5)), false;
        if (n != 6 + 3 * (size_t)count) return *err = make_diag(kJSofSize, (uint32_t)(base + 5), count, (uint32_t)n), false;
        if (p[0] != 8) return *err = make_diag(kJSofPrecision, (uint32_t)base), false;
        uint16_t height = be16(p + 1), width = be16(p + 3);
        if (width == 0) return *err = make_diag(kJSofWidth, (uint32_t)(base + 3)), false;
        for (uint32_t i = 0; i < count; i++) {
            size_t o = 6 + (size_t)i * 3;
            uint8_t hs = p[o + 1] >> 4, vs = p[o + 1] & 0x0f;
            if (!(hs >= 1 && hs <= 4) || !(vs >= 1 && vs <= 4))
                return *err = make_diag(kJSofSampling, (uint32_t)(base + o + 1)), false;
            if (p[o + 2] > 3) return *err = make_diag(kJSofTq, (uint32_t)(base + o + 2)), false;
        }
        if (!h->have_sof) {
            h->have_sof = 1;
            h->width = width;
            h->height = height;
            h->ncomp = (uint16_t)count;
            h->sof_comp_off = (uint32_t)(base + 6);
        }
        return true;
    }
    if (code == 0xdb) {  // parse_quantization_tables, parser.rs:206-250
        size_t position = 0;
        int count = 0;
        while (position < n) {
            uint8_t spec = p[position];
            position += 1;
            uint8_t prec = spec >> 4;
            if (prec > 1) return *err = make_diag(kJDqtPrecision, (uint32_t)(base + position - 1)), false;
            uint8_t id = spec & 0x0f;
            if (id > 3) return *err = make_diag(kJDqtId, (uint32_t)(base + position - 1)), false;
            size_t table_bytes = prec ? 128 : 64;
            if (n - position < table_bytes) return *err = make_diag(kJDqtTrunc, (uint32_t)(base + position)), false;
            if (before_sos) {
                h->q_present[id] = 1;
                h->q_sixteen[id] = prec;
                h->q_off[id] = (uint32_t)(base + position);
            }
            position += table_bytes;
            count++;
        }
        if (count == 0) return *err = make_diag(kJDqtEmpty, (uint32_t)base), false;
        return true;
    }
    if (code == 0xc4) {  // parse_huffman_tables, parser.rs:252-295
        size_t position = 0;
        int count = 0;
        while (position < n) {
            uint8_t spec = p[position];
            position += 1;
            uint8_t cls = spec >> 4;
            if (cls > 1) return *err = make_diag(kJDhtClass, (uint32_t)(base + position - 1)), false;
            uint8_t id = spec & 0x0f;
            if (id > 3) return *err = make_diag(kJDhtId, (uint32_t)(base + position - 1)), false;
            if (position + 16 > n) return *err = make_diag(kJDhtTruncCounts, (uint32_t)(base + position)), false;
            const uint8_t *counts = p + position;
            size_t nsym = 0;
            for (int i = 0; i < 16; i++) nsym += counts[i];
            if (position + 16 + nsym > n) return *err = make_diag(kJDhtTruncSymbols, (uint32_t)(base + position + 16)), false;
            if (before_sos) {
                // DecodeTables::collect builds every table in order and stops at the first
                // invalid one; remember that one, and the latest definition per slot.
                if (h->huff_err.kind == kDiagNone) {
                    Diag he;
                    if (!huffman_table_ok(counts, id, &he)) h->huff_err = he;
                }
                int slot = cls * 4 + id;
                h->h_present[slot] = 1;
                h->h_off[slot] = (uint32_t)(base + position);
                h->h_nsym[slot] = (uint16_t)nsym;
            }
            position += 16 + nsym;
            count++;
        }
        if (count == 0) return *err = make_diag(kJDhtEmpty, (uint32_t)base), false;
        return true;
    }
    if (code == 0xdd) {  // DRI, parser.rs:125-133
        if (n != 2) return *err = make_diag(kJDriSize, (uint32_t)base), false;
        if (before_sos) h->dri = be16(p);
        return true;
    }
    if (code == 0xda) {  // parse_scan_header, parser.rs:297-339
        if (n == 0) return *err = make_diag(kJSosEmpty, (uint32_t)base), false;
        uint32_t count = p[0];
        if (count == 0) return *err = make_diag(kJSosNoComp, (uint32_t)base), false;
        if (n != 1 + 2 * (size_t)count + 3) return *err = make_diag(kJSosSize, (uint32_t)base, count, (uint32_t)n), false;
        for (uint32_t i = 0; i < count; i++) {
            size_t o = 1 + (size_t)i * 2;
            uint8_t sel = p[o + 1];
            if ((sel >> 4) > 3 || (sel & 0x0f) > 3) return *err = make_diag(kJSosSelector, (uint32_t)(base + o + 1)), false;
        }
        if (!h->have_sos) {
            size_t tail = 1 + 2 * (size_t)count;
            h->have_sos = 1;
            h->sos_ncomp = (uint16_t)count;
            h->sos_comp_off = (uint32_t)(base + 1);
            h->ss = p[tail];
            h->se = p[tail + 1];
            h->ah = p[tail + 2] >> 4;
            h->al = p[tail + 2] & 0x0f;
        }
        return true;
    }
    if (code == 0xe0 && n >= 5 && p[0] == 'J' && p[1] == 'F' && p[2] == 'I' && p[3] == 'F' && p[4] == 0) {
        // parse_jfif, parser.rs:341-371
        if (n < 14) return *err = make_diag(kJJfifShort, (uint32_t)base), false;
        size_t thumb = 3 * (size_t)p[12] * (size_t)p[13];
        if (n != 14 + thumb) return *err = make_diag(kJJfifThumb, (uint32_t)(base + 12)), false;
        h->jfif = 1;
        return true;
    }
    if (code == 0xee && h->adobe < 0 && n >= 12 && p[0] == 'A' && p[1] == 'd' && p[2] == 'o' && p[3] == 'b' &&
        p[4] == 'e') {
        // infer_color_model's first "Adobe" APP14 (decoder.rs:173-184)
        h->adobe = p[11];
    }
    return true;
}

// scan_entropy_data (parser.rs:373-414) run sequentially; used by parse_tail for
// any further scan and by hosts that must find the first scan's end themselves.
MMR_HD bool scan_entropy(const uint8_t *in, size_t len, size_t data_offset, size_t *moff, uint8_t *mcode,
                         size_t *after, Diag *err) {
    size_t position = data_offset;
    while (position < len) {
        if (in[position] != 0xff) {
            position += 1;
            continue;
        }
        size_t marker_offset = position;
        position += 1;
        while (position < len && in[position] == 0xff) position += 1;
        if (position >= len) return *err = make_diag(kJScanTruncMarker, (uint32_t)position), false;
        uint8_t code = in[position];
        position += 1;
        if (code == 0x00 || (code >= 0xd0 && code <= 0xd7)) continue;
        *moff = marker_offset;
        *mcode = code;
        *after = position;
        return true;
    }
    return *err = make_diag(kJScanNoTerminator, (uint32_t)len), false;
}

// The marker loop of parse_jpeg (parser.rs:30-80) from `position` (or from a
// pending marker). Stops after the first SOS header when stop_at_sos is set.
MMR_HD void marker_loop(const uint8_t *in, size_t len, size_t position, bool pending, size_t p_off, uint8_t p_code,
                        size_t p_after, bool stop_at_sos, JpegHeader *h) {
    for (;;) {
        size_t offset, after;
        uint8_t code;
        if (pending) {
            offset = p_off;
            code = p_code;
            after = p_after;
            pending = false;
        } else if (!read_marker(in, len, position, &offset, &code, &after, &h->err)) {
            return;
        }
        position = after;
        if (code == 0xd9) {
            if (stop_at_sos) h->ended_at_eoi = 1;
            return;
        }
        if (!has_length(code)) continue;
        if (position + 2 > len) {
            h->err = make_diag(kJTruncLength, (uint32_t)position);
            return;
        }
        uint16_t length = be16(in + position);
        if (length < 2) {
            h->err = make_diag(kJBadLength, (uint32_t)position);
            return;
        }
        size_t payload_offset = position + 2;
        size_t payload_length = (size_t)length - 2;
        size_t payload_end = payload_offset + payload_length;
        if (payload_end > len) {
            h->err = make_diag(kJTruncPayload, (uint32_t)payload_offset, code);
            return;
        }
        bool before_sos = !h->have_sos;
        if (!parse_segment(in, code, payload_offset, payload_length, before_sos, h, &h->err)) return;
        position = payload_end;
        if (code == 0xda) {
            h->scan_count += 1;
            if (stop_at_sos && before_sos) {
                h->sos_marker_off = (uint32_t)offset;
                h->data_offset = (uint32_t)position;
                return;
            }
            if (!scan_entropy(in, len, position, &p_off, &p_code, &p_after, &h->err)) return;
            position = p_after;
            pending = true;
        }
    }
}

}  // namespace jpeg_detail

MMR_HD void jpeg_header_init(JpegHeader *h) {
    uint8_t *b = (uint8_t *)h;
    for (size_t i = 0; i < sizeof(JpegHeader); i++) b[i] = 0;
    h->adobe = -1;
}

// SOI .. end of the first SOS header (or EOI, or the first error).
MMR_HD void jpeg_parse_prefix(const uint8_t *in, size_t len, JpegHeader *h) {
    using namespace jpeg_detail;
    jpeg_header_init(h);
    size_t soi_off, pos;
    uint8_t soi;
    if (!read_marker(in, len, 0, &soi_off, &soi, &pos, &h->err)) return;
    if (soi != 0xd8 || soi_off != 0) {
        h->err = make_diag(kJExpectSoi, (uint32_t)soi_off);
        return;
    }
    marker_loop(in, len, pos, false, 0, 0, 0, true, h);
    h->prefix_done = h->err.kind == kDiagNone;
}

// Continues parse_jpeg from the marker that terminated the first scan: the
// marker's FF run starts at term_off. Records errors, later scans and
// colour-model facts; table definitions found here do not affect decoding.
MMR_HD void jpeg_parse_tail(const uint8_t *in, size_t len, size_t term_off, JpegHeader *h) {
    using namespace jpeg_detail;
    size_t q = term_off + 1;
    while (q < len && in[q] == 0xff) q++;
    // The marker scan guarantees a code byte exists here.
    marker_loop(in, len, 0, true, term_off, in[q], q + 1, false, h);
}

// Host fallback for images whose first SOF0 follows the first SOS: finds the
// first scan's end sequentially. Returns false (with h->err set) on failure.
MMR_HD bool jpeg_find_first_scan_end(const uint8_t *in, size_t len, const JpegHeader *h, size_t *term_off,
                                     Diag *err) {
    size_t moff, after;
    uint8_t code;
    if (!jpeg_detail::scan_entropy(in, len, h->data_offset, &moff, &code, &after, err)) return false;
    *term_off = moff;
    return true;
}

}  // namespace mmr
