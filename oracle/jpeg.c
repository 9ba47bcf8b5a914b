/*
 * Oracle restatement of the MMRecode baseline JPEG decoder.
 * TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Follows, statement for statement:
 *   crates/codecs/mjpeg/src/parser.rs     (parse_jpeg and segment parsers)
 *   crates/codecs/mjpeg/src/entropy.rs    (HuffmanDecoder, EntropyReader, receive_extend)
 *   crates/codecs/mjpeg/src/decoder.rs    (decode_jpeg, reconstruct, decode_block, ...)
 *   crates/codecs/mjpeg/src/transform.rs  (inverse_dct, IDCT_MATRIX)
 *   crates/codecs/mjpeg/src/tables.rs     (ZIGZAG_TO_NATURAL)
 */
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

static void set_err(orc_result *res, int status, const char *fmt, ...) {
    if (!res) return;
    res->status = status;
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(res->message, sizeof(res->message), fmt, ap);
    va_end(ap);
}

/* parser.rs:416-422: "JPEG at byte 0x%08x: msg" */
static int jpeg_invalid(orc_result *res, size_t offset, const char *msg) {
    set_err(res, ORC_INVALID_DATA, "JPEG at byte 0x%08zx: %s", offset, msg);
    return ORC_INVALID_DATA;
}

/* ------------------------------------------------------------------ */
/* syntax.rs:34-110 Marker                                              */
/* ------------------------------------------------------------------ */

static const char *marker_name(uint8_t code) {
    static const char *rst[8] = {"RST0", "RST1", "RST2", "RST3", "RST4", "RST5", "RST6", "RST7"};
    if (code == 0x01) return "TEM";
    if (code == 0xc0) return "SOF0";
    if (code == 0xc4) return "DHT";
    if (code >= 0xd0 && code <= 0xd7) return rst[code - 0xd0];
    if (code == 0xd8) return "SOI";
    if (code == 0xd9) return "EOI";
    if (code == 0xda) return "SOS";
    if (code == 0xdb) return "DQT";
    if (code == 0xdc) return "DNL";
    if (code == 0xdd) return "DRI";
    if (code >= 0xe0 && code <= 0xef) return "APP";
    if (code == 0xfe) return "COM";
    return "UNKNOWN";
}

static int marker_has_length(uint8_t code) {
    if (code == 0x01) return 0;
    if (code >= 0xd0 && code <= 0xd7) return 0;
    if (code == 0xd8 || code == 0xd9) return 0;
    return 1;
}

/* ------------------------------------------------------------------ */
/* Parsed representation (syntax.rs:114-325)                          */
/* ------------------------------------------------------------------ */

enum seg_kind {
    SEG_EMPTY, SEG_FRAME, SEG_DQT, SEG_DHT, SEG_DRI, SEG_SOS, SEG_JFIF, SEG_APP, SEG_COM, SEG_UNKNOWN
};

typedef struct { uint8_t id, h, v, tq; } fcomp_t;
typedef struct { uint8_t precision; uint16_t height, width; int ncomp; fcomp_t comp[256]; } frame_t;
typedef struct { uint8_t id; int sixteen; uint16_t values[64]; } qtable_t;
typedef struct { int ac; uint8_t id; uint8_t counts[16]; int nsym; uint8_t symbols[16 * 255]; } htable_t;
typedef struct { uint8_t sel, td, ta; } scomp_t;
typedef struct { int ncomp; scomp_t comp[256]; uint8_t ss, se, ah, al; } scan_t;

typedef struct {
    size_t offset;
    uint8_t code;
    int kind;
    /* payload-derived data */
    int first, count;    /* index range into the typed arrays */
    uint16_t dri;
    const uint8_t *app_data;
    size_t app_len;
} seg_t;

typedef struct {
    size_t data_offset, data_length;
    size_t nrst;
    size_t *rst_offsets;
    uint8_t *rst_numbers;
} escan_t;

typedef struct {
    seg_t *segs; size_t nseg, capseg;
    frame_t *frames; size_t nframe, capframe;
    qtable_t *qt; size_t nqt, capqt;
    htable_t *ht; size_t nht, capht;
    scan_t *scans; size_t nscan_hdr, capscan;
    escan_t *escans; size_t nescan, capescan;
    size_t trailing_len;
} image_t;

#define GROW(arr, n, cap)                                                        \
    do {                                                                         \
        if ((n) == (cap)) {                                                      \
            (cap) = (cap) ? (cap) * 2 : 8;                                       \
            (arr) = realloc((arr), (cap) * sizeof(*(arr)));                     \
        }                                                                        \
    } while (0)

static void image_free(image_t *im) {
    free(im->segs);
    free(im->frames);
    free(im->qt);
    free(im->ht);
    free(im->scans);
    for (size_t i = 0; i < im->nescan; i++) {
        free(im->escans[i].rst_offsets);
        free(im->escans[i].rst_numbers);
    }
    free(im->escans);
    memset(im, 0, sizeof(*im));
}

static seg_t *push_seg(image_t *im, size_t offset, uint8_t code, int kind) {
    GROW(im->segs, im->nseg, im->capseg);
    seg_t *s = &im->segs[im->nseg++];
    memset(s, 0, sizeof(*s));
    s->offset = offset;
    s->code = code;
    s->kind = kind;
    return s;
}

/* parser.rs:93-110 read_marker */
static int read_marker(const uint8_t *in, size_t len, size_t position, size_t *moff,
                       uint8_t *code, size_t *after, orc_result *res) {
    if (position >= len || in[position] != 0xff)
        return jpeg_invalid(res, position, "expected JPEG marker prefix 0xff");
    size_t offset = position;
    size_t code_offset = position + 1;
    while (code_offset < len && in[code_offset] == 0xff) code_offset++;
    if (code_offset >= len) return jpeg_invalid(res, code_offset, "truncated marker");
    uint8_t c = in[code_offset];
    if (c == 0x00)
        return jpeg_invalid(res, code_offset, "stuffed 0xff byte outside entropy-coded data");
    *moff = offset;
    *code = c;
    *after = code_offset + 1;
    return ORC_OK;
}

/* parser.rs:149-204 parse_frame_header */
static int parse_frame_header(image_t *im, const uint8_t *p, size_t n, size_t base, seg_t *seg,
                              orc_result *res) {
    if (n < 6) return jpeg_invalid(res, base, "SOF0 payload is too short");
    size_t count = p[5];
    if (count == 0) return jpeg_invalid(res, base + 5, "SOF0 must declare at least one component");
    size_t expected = 6 + 3 * count;
    if (n != expected) {
        char msg[128];
        snprintf(msg, sizeof msg, "SOF0 declares %zu components but has %zu bytes", count, n);
        return jpeg_invalid(res, base + 5, msg);
    }
    if (p[0] != 8) return jpeg_invalid(res, base, "baseline SOF0 sample precision must be 8 bits");
    uint16_t height = (uint16_t)((p[1] << 8) | p[2]);
    uint16_t width = (uint16_t)((p[3] << 8) | p[4]);
    if (width == 0) return jpeg_invalid(res, base + 3, "SOF0 width must be non-zero");
    frame_t f;
    f.precision = p[0];
    f.height = height;
    f.width = width;
    f.ncomp = (int)count;
    for (size_t i = 0; i < count; i++) {
        size_t o = 6 + i * 3;
        uint8_t s = p[o + 1];
        uint8_t h = s >> 4, v = s & 0x0f;
        if (!(h >= 1 && h <= 4) || !(v >= 1 && v <= 4))
            return jpeg_invalid(res, base + o + 1, "sampling factors must be between 1 and 4");
        if (p[o + 2] > 3)
            return jpeg_invalid(res, base + o + 2, "quantization table selector must be 0 through 3");
        f.comp[i].id = p[o];
        f.comp[i].h = h;
        f.comp[i].v = v;
        f.comp[i].tq = p[o + 2];
    }
    GROW(im->frames, im->nframe, im->capframe);
    seg->first = (int)im->nframe;
    seg->count = 1;
    im->frames[im->nframe++] = f;
    return ORC_OK;
}

/* parser.rs:206-250 parse_quantization_tables */
static int parse_dqt(image_t *im, const uint8_t *p, size_t n, size_t base, seg_t *seg,
                     orc_result *res) {
    size_t position = 0;
    int first = (int)im->nqt, count = 0;
    while (position < n) {
        uint8_t spec = p[position];
        position += 1;
        int sixteen;
        if ((spec >> 4) == 0) sixteen = 0;
        else if ((spec >> 4) == 1) sixteen = 1;
        else return jpeg_invalid(res, base + position - 1, "DQT precision must be 0 or 1");
        uint8_t id = spec & 0x0f;
        if (id > 3) return jpeg_invalid(res, base + position - 1, "DQT table identifier must be 0 through 3");
        size_t bpv = sixteen ? 2 : 1;
        size_t table_bytes = 64 * bpv;
        size_t avail = n > position ? n - position : 0;
        if (avail < table_bytes) return jpeg_invalid(res, base + position, "truncated DQT values");
        qtable_t t;
        t.id = id;
        t.sixteen = sixteen;
        for (int i = 0; i < 64; i++) {
            if (bpv == 1) {
                t.values[i] = p[position];
                position += 1;
            } else {
                t.values[i] = (uint16_t)((p[position] << 8) | p[position + 1]);
                position += 2;
            }
        }
        GROW(im->qt, im->nqt, im->capqt);
        im->qt[im->nqt++] = t;
        count++;
    }
    if (count == 0) return jpeg_invalid(res, base, "DQT must contain at least one table");
    seg->first = first;
    seg->count = count;
    return ORC_OK;
}

/* parser.rs:252-295 parse_huffman_tables */
static int parse_dht(image_t *im, const uint8_t *p, size_t n, size_t base, seg_t *seg,
                     orc_result *res) {
    size_t position = 0;
    int first = (int)im->nht, count = 0;
    while (position < n) {
        uint8_t spec = p[position];
        position += 1;
        int ac;
        if ((spec >> 4) == 0) ac = 0;
        else if ((spec >> 4) == 1) ac = 1;
        else return jpeg_invalid(res, base + position - 1, "DHT class must be 0 or 1");
        uint8_t id = spec & 0x0f;
        if (id > 3) return jpeg_invalid(res, base + position - 1, "DHT table identifier must be 0 through 3");
        if (position + 16 > n) return jpeg_invalid(res, base + position, "truncated DHT code counts");
        htable_t t;
        t.ac = ac;
        t.id = id;
        memcpy(t.counts, p + position, 16);
        position += 16;
        size_t nsym = 0;
        for (int i = 0; i < 16; i++) nsym += t.counts[i];
        if (position + nsym > n) return jpeg_invalid(res, base + position, "truncated DHT symbols");
        /* 16 counts of at most 255 each bound the table to 4080 symbols. */
        t.nsym = (int)nsym;
        memcpy(t.symbols, p + position, nsym);
        position += nsym;
        GROW(im->ht, im->nht, im->capht);
        im->ht[im->nht++] = t;
        count++;
    }
    if (count == 0) return jpeg_invalid(res, base, "DHT must contain at least one table");
    seg->first = first;
    seg->count = count;
    return ORC_OK;
}

/* parser.rs:297-339 parse_scan_header */
static int parse_sos(image_t *im, const uint8_t *p, size_t n, size_t base, seg_t *seg,
                     orc_result *res) {
    if (n == 0) return jpeg_invalid(res, base, "SOS payload is empty");
    size_t count = p[0];
    if (count == 0) return jpeg_invalid(res, base, "SOS must select at least one component");
    size_t expected = 1 + 2 * count + 3;
    if (n != expected) {
        char msg[128];
        snprintf(msg, sizeof msg, "SOS declares %zu components but has %zu bytes", count, n);
        return jpeg_invalid(res, base, msg);
    }
    scan_t s;
    s.ncomp = (int)count;
    for (size_t i = 0; i < count; i++) {
        size_t o = 1 + i * 2;
        uint8_t sel = p[o + 1];
        if ((sel >> 4) > 3 || (sel & 0x0f) > 3)
            return jpeg_invalid(res, base + o + 1, "Huffman table selectors must be 0 through 3");
        s.comp[i].sel = p[o];
        s.comp[i].td = sel >> 4;
        s.comp[i].ta = sel & 0x0f;
    }
    size_t tail = 1 + 2 * count;
    s.ss = p[tail];
    s.se = p[tail + 1];
    s.ah = p[tail + 2] >> 4;
    s.al = p[tail + 2] & 0x0f;
    GROW(im->scans, im->nscan_hdr, im->capscan);
    seg->first = (int)im->nscan_hdr;
    seg->count = 1;
    im->scans[im->nscan_hdr++] = s;
    return ORC_OK;
}

/* parser.rs:341-371 parse_jfif */
static int parse_jfif(const uint8_t *p, size_t n, size_t base, orc_result *res) {
    if (n < 14) return jpeg_invalid(res, base, "JFIF APP0 payload is too short");
    size_t thumb = 3 * (size_t)p[12] * (size_t)p[13];
    if (n != 14 + thumb)
        return jpeg_invalid(res, base + 12, "JFIF thumbnail dimensions do not match payload size");
    return ORC_OK;
}

/* parser.rs:119-147 parse_segment_data */
static int parse_segment_data(image_t *im, uint8_t code, const uint8_t *p, size_t n, size_t base,
                              seg_t *seg, orc_result *res) {
    switch (code) {
    case 0xc0:
        seg->kind = SEG_FRAME;
        return parse_frame_header(im, p, n, base, seg, res);
    case 0xdb:
        seg->kind = SEG_DQT;
        return parse_dqt(im, p, n, base, seg, res);
    case 0xc4:
        seg->kind = SEG_DHT;
        return parse_dht(im, p, n, base, seg, res);
    case 0xdd:
        seg->kind = SEG_DRI;
        if (n != 2) return jpeg_invalid(res, base, "DRI payload must contain exactly two bytes");
        seg->dri = (uint16_t)((p[0] << 8) | p[1]);
        return ORC_OK;
    case 0xda:
        seg->kind = SEG_SOS;
        return parse_sos(im, p, n, base, seg, res);
    default:
        break;
    }
    if (code == 0xe0 && n >= 5 && memcmp(p, "JFIF\0", 5) == 0) {
        seg->kind = SEG_JFIF;
        return parse_jfif(p, n, base, res);
    }
    if (code >= 0xe0 && code <= 0xef) {
        seg->kind = SEG_APP;
        seg->app_data = p;
        seg->app_len = n;
        return ORC_OK;
    }
    seg->kind = code == 0xfe ? SEG_COM : SEG_UNKNOWN;
    return ORC_OK;
}

/* parser.rs:373-414 scan_entropy_data */
static int scan_entropy_data(image_t *im, const uint8_t *in, size_t len, size_t data_offset,
                             size_t *moff, uint8_t *mcode, size_t *after, orc_result *res) {
    size_t position = data_offset;
    escan_t sc;
    memset(&sc, 0, sizeof sc);
    size_t cap = 0;
    while (position < len) {
        if (in[position] != 0xff) {
            position += 1;
            continue;
        }
        size_t marker_offset = position;
        position += 1;
        while (position < len && in[position] == 0xff) position += 1;
        if (position >= len) {
            free(sc.rst_offsets);
            free(sc.rst_numbers);
            return jpeg_invalid(res, position, "truncated marker in entropy-coded data");
        }
        uint8_t code = in[position];
        position += 1;
        if (code == 0x00) continue;
        if (code >= 0xd0 && code <= 0xd7) {
            if (sc.nrst == cap) {
                cap = cap ? cap * 2 : 16;
                sc.rst_offsets = realloc(sc.rst_offsets, cap * sizeof(size_t));
                sc.rst_numbers = realloc(sc.rst_numbers, cap);
            }
            sc.rst_offsets[sc.nrst] = marker_offset;
            sc.rst_numbers[sc.nrst] = code - 0xd0;
            sc.nrst++;
            continue;
        }
        sc.data_offset = data_offset;
        sc.data_length = marker_offset - data_offset;
        GROW(im->escans, im->nescan, im->capescan);
        im->escans[im->nescan++] = sc;
        *moff = marker_offset;
        *mcode = code;
        *after = position;
        return ORC_OK;
    }
    free(sc.rst_offsets);
    free(sc.rst_numbers);
    return jpeg_invalid(res, len, "entropy-coded scan has no terminating marker");
}

/* parser.rs:18-81 parse_jpeg */
static int parse_jpeg(const uint8_t *in, size_t len, image_t *im, orc_result *res) {
    memset(im, 0, sizeof(*im));
    size_t soi_offset, position;
    uint8_t soi;
    int st = read_marker(in, len, 0, &soi_offset, &soi, &position, res);
    if (st) return st;
    if (soi != 0xd8 || soi_offset != 0) return jpeg_invalid(res, soi_offset, "expected SOI as the first marker");
    push_seg(im, soi_offset, soi, SEG_EMPTY);
    int have_pending = 0;
    size_t p_off = 0, p_after = 0;
    uint8_t p_code = 0;
    for (;;) {
        size_t offset, after;
        uint8_t code;
        if (have_pending) {
            offset = p_off;
            code = p_code;
            after = p_after;
            have_pending = 0;
        } else {
            st = read_marker(in, len, position, &offset, &code, &after, res);
            if (st) return st;
        }
        position = after;
        if (code == 0xd9) {
            push_seg(im, offset, code, SEG_EMPTY);
            im->trailing_len = len - position;
            return ORC_OK;
        }
        if (!marker_has_length(code)) {
            push_seg(im, offset, code, SEG_EMPTY);
            continue;
        }
        if (position + 2 > len) return jpeg_invalid(res, position, "truncated segment length");
        uint16_t length = (uint16_t)((in[position] << 8) | in[position + 1]);
        if (length < 2) return jpeg_invalid(res, position, "segment length must include its two length bytes");
        size_t payload_offset = position + 2;
        size_t payload_length = (size_t)length - 2;
        size_t payload_end = payload_offset + payload_length;
        if (payload_end > len) {
            char msg[64];
            snprintf(msg, sizeof msg, "truncated %s payload", marker_name(code));
            return jpeg_invalid(res, payload_offset, msg);
        }
        seg_t tmp;
        memset(&tmp, 0, sizeof tmp);
        st = parse_segment_data(im, code, in + payload_offset, payload_length, payload_offset, &tmp, res);
        if (st) return st;
        seg_t *s = push_seg(im, offset, code, tmp.kind);
        s->first = tmp.first;
        s->count = tmp.count;
        s->dri = tmp.dri;
        s->app_data = tmp.app_data;
        s->app_len = tmp.app_len;
        position = payload_end;
        if (code == 0xda) {
            st = scan_entropy_data(im, in, len, position, &p_off, &p_code, &p_after, res);
            if (st) return st;
            position = p_after;
            have_pending = 1;
        }
    }
}

/* ------------------------------------------------------------------ */
/* entropy.rs                                                           */
/* ------------------------------------------------------------------ */

typedef struct { uint16_t bits; uint8_t length; uint8_t symbol; } hcode_t;
typedef struct { hcode_t codes[4096]; int ncodes; int valid; } hdec_t;

/* entropy.rs:18-55 HuffmanDecoder::new */
static int huffman_new(const htable_t *t, hdec_t *d, orc_result *res) {
    size_t nsym = 0;
    for (int i = 0; i < 16; i++) nsym += t->counts[i];
    if (nsym == 0 || nsym != (size_t)t->nsym) {
        set_err(res, ORC_INVALID_DATA, "JPEG Huffman table %u has inconsistent symbol counts", t->id);
        return ORC_INVALID_DATA;
    }
    uint32_t code = 0;
    int si = 0;
    d->ncodes = 0;
    for (int li = 0; li < 16; li++) {
        uint8_t length = (uint8_t)(li + 1);
        uint32_t limit = 1u << length;
        uint32_t count = t->counts[li];
        if (code + count > limit) {
            set_err(res, ORC_INVALID_DATA, "JPEG Huffman table %u is oversubscribed at length %u", t->id, length);
            return ORC_INVALID_DATA;
        }
        for (uint32_t c = 0; c < count; c++) {
            d->codes[d->ncodes].bits = (uint16_t)code;
            d->codes[d->ncodes].length = length;
            d->codes[d->ncodes].symbol = t->symbols[si];
            d->ncodes++;
            si++;
            code++;
        }
        code <<= 1;
    }
    d->valid = 1;
    return ORC_OK;
}

/* entropy.rs:74-91 EntropyReader */
typedef struct {
    const uint8_t *data;
    size_t len;
    size_t base_offset;
    size_t position;
    uint8_t current_byte;
    uint8_t bits_remaining;
} reader_t;

static int reader_error(reader_t *r, orc_result *res, const char *msg) {
    set_err(res, ORC_INVALID_DATA, "JPEG entropy at byte 0x%08zx: %s", r->base_offset + r->position, msg);
    return ORC_INVALID_DATA;
}

/* entropy.rs:143-165 read_data_byte */
static int read_data_byte(reader_t *r, uint8_t *out, orc_result *res) {
    if (r->position >= r->len) return reader_error(r, res, "unexpected end of entropy-coded data");
    uint8_t byte = r->data[r->position];
    r->position += 1;
    if (byte != 0xff) {
        *out = byte;
        return ORC_OK;
    }
    while (r->position < r->len && r->data[r->position] == 0xff) r->position += 1;
    if (r->position >= r->len) return reader_error(r, res, "truncated entropy marker");
    uint8_t code = r->data[r->position];
    r->position += 1;
    if (code == 0x00) {
        *out = 0xff;
        return ORC_OK;
    }
    char msg[64];
    snprintf(msg, sizeof msg, "unexpected marker 0xff%02x inside coded block", code);
    return reader_error(r, res, msg);
}

/* entropy.rs:93-101 read_bit */
static int read_bit(reader_t *r, uint8_t *bit, orc_result *res) {
    if (r->bits_remaining == 0) {
        int st = read_data_byte(r, &r->current_byte, res);
        if (st) return st;
        r->bits_remaining = 8;
    }
    r->bits_remaining -= 1;
    *bit = (r->current_byte >> r->bits_remaining) & 1;
    return ORC_OK;
}

/* entropy.rs:103-109 read_bits */
static int read_bits(reader_t *r, uint8_t count, uint16_t *value, orc_result *res) {
    uint16_t v = 0;
    for (uint8_t i = 0; i < count; i++) {
        uint8_t b;
        int st = read_bit(r, &b, res);
        if (st) return st;
        v = (uint16_t)((v << 1) | b);
    }
    *value = v;
    return ORC_OK;
}

/* entropy.rs:111-134 consume_restart */
static int consume_restart(reader_t *r, uint8_t expected, orc_result *res) {
    r->bits_remaining = 0;
    size_t marker_offset = r->base_offset + r->position;
    if (r->position >= r->len || r->data[r->position] != 0xff)
        return reader_error(r, res, "expected restart marker at MCU boundary");
    r->position += 1;
    while (r->position < r->len && r->data[r->position] == 0xff) r->position += 1;
    if (r->position >= r->len) return reader_error(r, res, "truncated restart marker");
    uint8_t code = r->data[r->position];
    r->position += 1;
    if (code != (uint8_t)(0xd0 + expected)) {
        set_err(res, ORC_INVALID_DATA, "JPEG at byte 0x%08zx: expected RST%u, found marker 0x%02x",
                marker_offset, expected, code);
        return ORC_INVALID_DATA;
    }
    return ORC_OK;
}

/* entropy.rs:57-70 HuffmanDecoder::decode */
static int huffman_decode(const hdec_t *d, reader_t *r, uint8_t *symbol, orc_result *res) {
    uint16_t bits = 0;
    for (uint8_t length = 1; length <= 16; length++) {
        uint8_t b;
        int st = read_bit(r, &b, res);
        if (st) return st;
        bits = (uint16_t)((bits << 1) | b);
        for (int i = 0; i < d->ncodes; i++) {
            if (d->codes[i].length == length && d->codes[i].bits == bits) {
                *symbol = d->codes[i].symbol;
                return ORC_OK;
            }
        }
    }
    return reader_error(r, res, "no Huffman code matches the next 16 bits");
}

/* entropy.rs:168-182 receive_extend */
static int receive_extend(reader_t *r, uint8_t size, int32_t *out, orc_result *res) {
    if (size == 0) {
        *out = 0;
        return ORC_OK;
    }
    if (size > 15) return reader_error(r, res, "coefficient magnitude contains more than 15 bits");
    uint16_t v;
    int st = read_bits(r, size, &v, res);
    if (st) return st;
    int32_t bits = v;
    int32_t threshold = 1 << (size - 1);
    *out = bits < threshold ? bits + 1 - (1 << size) : bits;
    return ORC_OK;
}

/* ------------------------------------------------------------------ */
/* tables.rs / transform.rs                                             */
/* ------------------------------------------------------------------ */

/* tables.rs:1-5 */
static const int ZIGZAG_TO_NATURAL[64] = {
    0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,  12, 19, 26, 33, 40, 48,
    41, 34, 27, 20, 13, 6,  7,  14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23,
    30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

/* transform.rs:2-84: the reference's literal f64 matrix, decimal digits as written there
 * (also used by the encoder restatement, encode.c). */
const double ORC_IDCT_MATRIX[8][8] = {
    {0.3535533905932738, 0.4903926402016152, 0.4619397662556434, 0.4157348061512726,
     0.3535533905932738, 0.2777851165098011, 0.1913417161825449, 0.09754516100806417},
    {0.3535533905932738, 0.4157348061512726, 0.1913417161825449, -0.0975451610080641,
     -0.3535533905932737, -0.4903926402016152, -0.4619397662556434, -0.2777851165098011},
    {0.3535533905932738, 0.2777851165098011, -0.1913417161825448, -0.4903926402016152,
     -0.3535533905932738, 0.09754516100806415, 0.4619397662556433, 0.4157348061512727},
    {0.3535533905932738, 0.09754516100806417, -0.4619397662556434, -0.2777851165098011,
     0.3535533905932737, 0.4157348061512727, -0.191341716182545, -0.4903926402016152},
    {0.3535533905932738, -0.0975451610080641, -0.4619397662556434, 0.2777851165098009,
     0.3535533905932738, -0.4157348061512726, -0.1913417161825449, 0.4903926402016152},
    {0.3535533905932738, -0.277785116509801, -0.1913417161825452, 0.4903926402016152,
     -0.3535533905932733, -0.0975451610080640, 0.4619397662556437, -0.415734806151272},
    {0.3535533905932738, -0.4157348061512727, 0.191341716182545, 0.0975451610080640,
     -0.3535533905932736, 0.4903926402016153, -0.4619397662556435, 0.2777851165098008},
    {0.3535533905932738, -0.4903926402016152, 0.4619397662556433, -0.415734806151272,
     0.3535533905932732, -0.2777851165098008, 0.1913417161825431, -0.0975451610080625},
};

/* f64::round then clamp(0,255) then `as u8` */
static uint8_t round_clamp_u8(double v) {
    double r = round(v);
    if (r < 0.0) r = 0.0;
    if (r > 255.0) r = 255.0;
    return (uint8_t)r;
}

/* transform.rs:86-109 inverse_dct */
void orc_jpeg_idct(const int32_t coefficients[64], uint8_t out[64]) {
    double temporary[64];
    for (int i = 0; i < 64; i++) temporary[i] = 0.0;
    for (int v = 0; v < 8; v++)
        for (int x = 0; x < 8; x++)
            for (int u = 0; u < 8; u++)
                temporary[v * 8 + x] += ORC_IDCT_MATRIX[x][u] * (double)coefficients[v * 8 + u];
    for (int y = 0; y < 8; y++)
        for (int x = 0; x < 8; x++) {
            double sum = 0.0;
            for (int v = 0; v < 8; v++) sum += ORC_IDCT_MATRIX[y][v] * temporary[v * 8 + x];
            out[y * 8 + x] = round_clamp_u8(sum + 128.0);
        }
}

void orc_jpeg_idct_many(const int32_t *coefficients, size_t n, uint8_t *out) {
    for (size_t b = 0; b < n; b++) orc_jpeg_idct(coefficients + 64 * b, out + 64 * b);
}

/* ------------------------------------------------------------------ */
/* decoder.rs                                                           */
/* ------------------------------------------------------------------ */

static const frame_t *image_frame_header(const image_t *im) {
    for (size_t i = 0; i < im->nseg; i++)
        if (im->segs[i].kind == SEG_FRAME) return &im->frames[im->segs[i].first];
    return NULL;
}

static int image_has_jfif(const image_t *im) {
    for (size_t i = 0; i < im->nseg; i++)
        if (im->segs[i].kind == SEG_JFIF) return 1;
    return 0;
}

enum { CM_GRAY = 0, CM_YCBCR = 1, CM_RGB = 2, CM_CMYK = 3, CM_YCCK = 4, CM_UNKNOWN = 5 };

/* decoder.rs:169-194 infer_color_model */
static int infer_color_model(const image_t *im, const frame_t *f) {
    if (f->ncomp == 1) return CM_GRAY;
    int adobe = -1;
    for (size_t i = 0; i < im->nseg; i++) {
        const seg_t *s = &im->segs[i];
        if (s->kind == SEG_APP && s->code == 0xee && s->app_len >= 12 && memcmp(s->app_data, "Adobe", 5) == 0) {
            adobe = s->app_data[11];
            break;
        }
    }
    if (f->ncomp == 3 && adobe == 0) return CM_RGB;
    if (f->ncomp == 3 && adobe == 1) return CM_YCBCR;
    if (f->ncomp == 4 && adobe == 0) return CM_CMYK;
    if (f->ncomp == 4 && adobe == 2) return CM_YCCK;
    if (f->ncomp == 3 && adobe == -1 && image_has_jfif(im)) return CM_YCBCR;
    return CM_UNKNOWN;
}

/* decoder.rs:196-221 single_scan */
static int single_scan(const image_t *im, const scan_t **scan, size_t *scan_offset, orc_result *res) {
    if (im->nescan != 1) {
        set_err(res, ORC_UNSUPPORTED, "baseline decoder currently requires exactly one scan, found %zu", im->nescan);
        return ORC_UNSUPPORTED;
    }
    int found = 0;
    for (size_t i = 0; i < im->nseg; i++) {
        if (im->segs[i].kind != SEG_SOS) continue;
        if (found) {
            set_err(res, ORC_UNSUPPORTED, "baseline decoder currently supports only one SOS header");
            return ORC_UNSUPPORTED;
        }
        *scan = &im->scans[im->segs[i].first];
        *scan_offset = im->segs[i].offset;
        found = 1;
    }
    if (!found) {
        set_err(res, ORC_INVALID_DATA, "JPEG has entropy data without an SOS header");
        return ORC_INVALID_DATA;
    }
    return ORC_OK;
}

/* decoder.rs:223-255 validate_baseline_subset */
static int validate_baseline_subset(const frame_t *f, const scan_t *s, orc_result *res) {
    if (f->height == 0) {
        set_err(res, ORC_UNSUPPORTED, "JPEG height supplied by a DNL marker is not supported yet");
        return ORC_UNSUPPORTED;
    }
    if (s->ncomp != f->ncomp) {
        set_err(res, ORC_UNSUPPORTED, "non-interleaved or partial-component JPEG scans are not supported yet");
        return ORC_UNSUPPORTED;
    }
    if (s->ss != 0 || s->se != 63 || s->ah != 0 || s->al != 0) {
        set_err(res, ORC_UNSUPPORTED, "scan parameters are not baseline sequential");
        return ORC_UNSUPPORTED;
    }
    for (int c = 0; c < f->ncomp; c++) {
        int occ = 0;
        for (int k = 0; k < s->ncomp; k++)
            if (s->comp[k].sel == f->comp[c].id) occ++;
        if (occ != 1) {
            set_err(res, ORC_INVALID_DATA, "JPEG scan must select frame component %u exactly once", f->comp[c].id);
            return ORC_INVALID_DATA;
        }
    }
    return ORC_OK;
}

typedef struct {
    const qtable_t *quant[4];
    hdec_t *dc[4];
    hdec_t *ac[4];
    uint16_t restart_interval;
} tables_t;

static void tables_free(tables_t *t) {
    for (int i = 0; i < 4; i++) {
        free(t->dc[i]);
        free(t->ac[i]);
    }
}

/* decoder.rs:264-299 DecodeTables::collect */
static int collect_tables(const image_t *im, size_t scan_offset, tables_t *t, orc_result *res) {
    memset(t, 0, sizeof(*t));
    for (size_t i = 0; i < im->nseg; i++) {
        const seg_t *s = &im->segs[i];
        if (!(s->offset < scan_offset)) break;
        if (s->kind == SEG_DQT) {
            for (int k = 0; k < s->count; k++) {
                const qtable_t *q = &im->qt[s->first + k];
                t->quant[q->id] = q;
            }
        } else if (s->kind == SEG_DHT) {
            for (int k = 0; k < s->count; k++) {
                const htable_t *h = &im->ht[s->first + k];
                hdec_t *d = malloc(sizeof(hdec_t));
                int st = huffman_new(h, d, res);
                if (st) {
                    free(d);
                    return st;
                }
                hdec_t **dst = h->ac ? &t->ac[h->id] : &t->dc[h->id];
                free(*dst);
                *dst = d;
            }
        } else if (s->kind == SEG_DRI) {
            t->restart_interval = s->dri;
        }
    }
    return ORC_OK;
}

typedef struct {
    uint8_t id, h, v;
    size_t width, height;
    uint8_t *samples;
    const qtable_t *quant;
    int32_t dc_prediction;
} cstate_t;

/* decoder.rs:495-548 decode_block */
static int decode_block(reader_t *r, const hdec_t *dcd, const hdec_t *acd, const qtable_t *q,
                        int32_t *dc_prediction, int32_t coefficients[64], orc_result *res) {
    for (int i = 0; i < 64; i++) coefficients[i] = 0;
    uint8_t dc_size;
    int st = huffman_decode(dcd, r, &dc_size, res);
    if (st) return st;
    if (dc_size > 11) return reader_error(r, res, "baseline DC coefficient category exceeds 11");
    int32_t difference;
    st = receive_extend(r, dc_size, &difference, res);
    if (st) return st;
    int64_t pred = (int64_t)*dc_prediction + difference;
    if (pred > INT32_MAX || pred < INT32_MIN) return reader_error(r, res, "DC prediction overflow");
    *dc_prediction = (int32_t)pred;
    int64_t dcq = (int64_t)*dc_prediction * (int64_t)q->values[0];
    if (dcq > INT32_MAX || dcq < INT32_MIN) return reader_error(r, res, "dequantized DC coefficient overflow");
    coefficients[0] = (int32_t)dcq;

    int zigzag_index = 1;
    while (zigzag_index < 64) {
        uint8_t symbol;
        st = huffman_decode(acd, r, &symbol, res);
        if (st) return st;
        int run = symbol >> 4;
        uint8_t size = symbol & 0x0f;
        if (size == 0) {
            if (run == 0) break;
            if (run != 15) return reader_error(r, res, "invalid zero-size AC Huffman symbol");
            zigzag_index += 16;
            if (zigzag_index > 64) return reader_error(r, res, "AC zero run exceeds the end of the block");
            continue;
        }
        if (size > 10) return reader_error(r, res, "baseline AC coefficient category exceeds 10");
        zigzag_index += run;
        if (zigzag_index >= 64) return reader_error(r, res, "AC coefficient run exceeds the end of the block");
        int32_t value;
        st = receive_extend(r, size, &value, res);
        if (st) return st;
        int64_t deq = (int64_t)value * (int64_t)q->values[zigzag_index];
        if (deq > INT32_MAX || deq < INT32_MIN) return reader_error(r, res, "dequantized AC coefficient overflow");
        coefficients[ZIGZAG_TO_NATURAL[zigzag_index]] = (int32_t)deq;
        zigzag_index += 1;
    }
    return ORC_OK;
}

/* decoder.rs:550-565 write_block */
static void write_block(cstate_t *p, size_t x, size_t y, const uint8_t block[64]) {
    for (size_t by = 0; by < 8; by++) {
        size_t dy = y + by;
        if (dy >= p->height) break;
        for (size_t bx = 0; bx < 8; bx++) {
            size_t dx = x + bx;
            if (dx >= p->width) break;
            p->samples[dy * p->width + dx] = block[by * 8 + bx];
        }
    }
}

/* decoder.rs:313-410 reconstruct (+ make_component_states :412-458, make_scan_decoders :460-493) */
static int reconstruct(const frame_t *f, const scan_t *s, const uint8_t *entropy, size_t elen,
                       size_t eoff, const tables_t *t, cstate_t **out_states, orc_result *res) {
    size_t width = f->width, height = f->height;
    uint8_t hmax = 0, vmax = 0;
    for (int c = 0; c < f->ncomp; c++) {
        if (f->comp[c].h > hmax) hmax = f->comp[c].h;
        if (f->comp[c].v > vmax) vmax = f->comp[c].v;
    }
    cstate_t *st = calloc((size_t)f->ncomp, sizeof(cstate_t));
    *out_states = st;
    for (int c = 0; c < f->ncomp; c++) {
        const fcomp_t *fc = &f->comp[c];
        const qtable_t *q = t->quant[fc->tq];
        if (!q) {
            set_err(res, ORC_INVALID_DATA, "JPEG component %u references missing quantization table %u", fc->id, fc->tq);
            return ORC_INVALID_DATA;
        }
        if (q->sixteen) {
            set_err(res, ORC_UNSUPPORTED, "16-bit quantization tables are not allowed in baseline JPEG");
            return ORC_UNSUPPORTED;
        }
        st[c].id = fc->id;
        st[c].h = fc->h;
        st[c].v = fc->v;
        st[c].width = (width * fc->h + hmax - 1) / hmax;
        st[c].height = (height * fc->v + vmax - 1) / vmax;
        st[c].samples = calloc(st[c].width * st[c].height > 0 ? st[c].width * st[c].height : 1, 1);
        st[c].quant = q;
        st[c].dc_prediction = 0;
    }
    int ndec = s->ncomp;
    int comp_index[256];
    const hdec_t *dcd[256];
    const hdec_t *acd[256];
    for (int k = 0; k < ndec; k++) {
        int idx = -1;
        for (int c = 0; c < f->ncomp; c++)
            if (f->comp[c].id == s->comp[k].sel) {
                idx = c;
                break;
            }
        if (idx < 0) {
            /* decoder.rs:470-474: `.expect(...)` panics when a scan selector names no frame
             * component (possible only with duplicate frame component ids); the C ABI
             * contains the panic (capi/src/lib.rs:572-588). */
            set_err(res, ORC_INTERNAL, "panic contained at MMRecode C API boundary");
            return ORC_INTERNAL;
        }
        comp_index[k] = idx;
        dcd[k] = t->dc[s->comp[k].td];
        if (!dcd[k]) {
            set_err(res, ORC_INVALID_DATA, "JPEG scan references missing DC Huffman table %u", s->comp[k].td);
            return ORC_INVALID_DATA;
        }
        acd[k] = t->ac[s->comp[k].ta];
        if (!acd[k]) {
            set_err(res, ORC_INVALID_DATA, "JPEG scan references missing AC Huffman table %u", s->comp[k].ta);
            return ORC_INVALID_DATA;
        }
    }
    int interleaved = f->ncomp > 1;
    size_t mcu_w = interleaved ? (size_t)hmax * 8 : 8;
    size_t mcu_h = interleaved ? (size_t)vmax * 8 : 8;
    size_t mcu_cols = (width + mcu_w - 1) / mcu_w;
    size_t mcu_rows = (height + mcu_h - 1) / mcu_h;
    reader_t r = {entropy, elen, eoff, 0, 0, 0};
    uint8_t restart_number = 0;
    int32_t coefficients[64];
    uint8_t samples[64];
    for (size_t mcu = 0; mcu < mcu_cols * mcu_rows; mcu++) {
        if (mcu > 0 && t->restart_interval != 0 && mcu % t->restart_interval == 0) {
            int e = consume_restart(&r, restart_number, res);
            if (e) return e;
            restart_number = (restart_number + 1) & 7;
            for (int c = 0; c < f->ncomp; c++) st[c].dc_prediction = 0;
        }
        size_t mx = mcu % mcu_cols, my = mcu / mcu_cols;
        for (int k = 0; k < ndec; k++) {
            cstate_t *cs = &st[comp_index[k]];
            size_t brows = interleaved ? cs->v : 1;
            size_t bcols = interleaved ? cs->h : 1;
            for (size_t by = 0; by < brows; by++)
                for (size_t bx = 0; bx < bcols; bx++) {
                    int e = decode_block(&r, dcd[k], acd[k], cs->quant, &cs->dc_prediction, coefficients, res);
                    if (e) return e;
                    orc_jpeg_idct(coefficients, samples);
                    write_block(cs, (mx * bcols + bx) * 8, (my * brows + by) * 8, samples);
                }
        }
    }
    return ORC_OK;
}

int orc_jpeg_parse(const uint8_t *data, size_t len, orc_jpeg_info *info, orc_result *res) {
    res->status = ORC_OK;
    res->message[0] = 0;
    memset(info, 0, sizeof(*info));
    image_t im;
    int st = parse_jpeg(data, len, &im, res);
    if (st) {
        image_free(&im);
        return st;
    }
    const frame_t *f = image_frame_header(&im);
    if (f) {
        info->width = f->width;
        info->height = f->height;
        info->component_count = (size_t)f->ncomp;
    }
    info->scan_count = im.nescan;
    if (im.nescan) {
        info->data_offset = im.escans[0].data_offset;
        info->data_length = im.escans[0].data_length;
        info->restart_count = im.escans[0].nrst;
        for (size_t i = 0; i < im.escans[0].nrst && i < 64; i++) {
            info->restart_offsets[i] = im.escans[0].rst_offsets[i];
            info->restart_numbers[i] = im.escans[0].rst_numbers[i];
        }
    }
    info->segment_count = im.nseg;
    info->last_marker = im.nseg ? im.segs[im.nseg - 1].code : 0;
    info->trailing_length = im.trailing_len;
    image_free(&im);
    return ORC_OK;
}

/* decoder.rs:140-167 decode_jpeg, followed by into_video_frame (:69-126) */
int orc_jpeg_decode(const uint8_t *data, size_t len, orc_frame *out, int *color_model, orc_result *res) {
    res->status = ORC_OK;
    res->message[0] = 0;
    memset(out, 0, sizeof(*out));
    if (color_model) *color_model = -1;
    image_t im;
    int st = parse_jpeg(data, len, &im, res);
    if (st) {
        image_free(&im);
        return st;
    }
    const frame_t *f = image_frame_header(&im);
    if (!f) {
        image_free(&im);
        set_err(res, ORC_INVALID_DATA, "JPEG has no baseline SOF0 frame header");
        return ORC_INVALID_DATA;
    }
    const scan_t *scan = NULL;
    size_t scan_offset = 0;
    st = single_scan(&im, &scan, &scan_offset, res);
    if (!st) st = validate_baseline_subset(f, scan, res);
    if (st) {
        image_free(&im);
        return st;
    }
    int cm = infer_color_model(&im, f);
    if (color_model) *color_model = cm;
    const escan_t *es = &im.escans[0];
    tables_t tables;
    st = collect_tables(&im, scan_offset, &tables, res);
    cstate_t *states = NULL;
    if (!st) st = reconstruct(f, scan, data + es->data_offset, es->data_length, es->data_offset, &tables, &states, res);
    tables_free(&tables);
    if (st) {
        if (states)
            for (int c = 0; c < f->ncomp; c++) free(states[c].samples);
        free(states);
        image_free(&im);
        return st;
    }
    /* into_video_frame / standard_pixel_format */
    size_t W = f->width, H = f->height;
    int fmt = 0;
    if (cm == CM_GRAY && f->ncomp == 1 && states[0].width == W && states[0].height == H) {
        fmt = ORC_FMT_GRAY8;
    } else if (cm != CM_YCBCR || f->ncomp != 3 || states[0].width != W || states[0].height != H ||
               states[1].width != states[2].width || states[1].height != states[2].height) {
        set_err(res, ORC_UNSUPPORTED, "JPEG components do not map directly to a shared planar pixel format");
        st = ORC_UNSUPPORTED;
    } else {
        size_t cw = states[1].width, ch = states[1].height;
        if (cw == W && ch == H) fmt = ORC_FMT_YUV444P8;
        else if (cw == (W + 1) / 2 && ch == H) fmt = ORC_FMT_YUV422P8;
        else if (cw == (W + 1) / 2 && ch == (H + 1) / 2) fmt = ORC_FMT_YUV420P8;
        else {
            set_err(res, ORC_UNSUPPORTED, "JPEG chroma sampling is not 4:2:0, 4:2:2, or 4:4:4");
            st = ORC_UNSUPPORTED;
        }
    }
    if (st) {
        for (int c = 0; c < f->ncomp; c++) free(states[c].samples);
        free(states);
        image_free(&im);
        return st;
    }
    out->format = (uint32_t)fmt;
    out->range = ORC_RANGE_FULL;
    out->width = W;
    out->height = H;
    out->plane_count = (size_t)f->ncomp;
    for (int c = 0; c < f->ncomp; c++) {
        out->planes[c].data = states[c].samples;
        out->planes[c].width = states[c].width;
        out->planes[c].height = states[c].height;
    }
    free(states);
    image_free(&im);
    return ORC_OK;
}

void orc_frame_free(orc_frame *frame) {
    if (!frame) return;
    for (size_t i = 0; i < frame->plane_count && i < 3; i++) free(frame->planes[i].data);
    memset(frame, 0, sizeof(*frame));
}
