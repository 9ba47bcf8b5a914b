/*
 * CPU oracle, encoder side: the reference's constrained baseline JPEG encoder
 * (crates/codecs/mjpeg/src/encoder.rs) restated in C, plus a coefficient-level
 * writer.
 *
 * TEST INFRASTRUCTURE ONLY. It generates test and benchmark input without the
 * product library (the reference arm of the benchmark must not load it), and it
 * writes crafted streams whose quantised coefficients the tests choose (the
 * adversarial transform blocks). Nothing in the product library links, includes
 * or calls this code.
 *
 * Options beyond the reference encoder, used to generate the benchmark shapes:
 * the standard Annex K Huffman tables (ITU-T T.81 K.3, data of the standard)
 * and a restart interval (DRI + RSTn markers, T.81 B.2.4.4 / F.1.2.3). With
 * annex_k = 0 and restart_interval = 0 the bytes are the reference encoder's.
 *
 * Compiled with -ffp-contract=off (forward_dct_quantize is a binary64
 * multiply/add sequence that Rust never contracts).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

/* tables.rs:1-5 */
static const int ZZ[64] = {0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,
                           12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6,  7,  14, 21, 28,
                           35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
                           58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};

/* tables.rs:7-17 LUMA_QUANTIZATION / CHROMA_QUANTIZATION (natural order) */
static const uint8_t LUMA_Q[64] = {16, 11, 10, 16, 24,  40,  51,  61,  12, 12, 14, 19, 26,  58,  60,  55,
                                   14, 13, 16, 24, 40,  57,  69,  56,  14, 17, 22, 29, 51,  87,  80,  62,
                                   18, 22, 37, 56, 68,  109, 103, 77,  24, 35, 55, 64, 81,  104, 113, 92,
                                   49, 64, 78, 87, 103, 121, 120, 101, 72, 92, 95, 98, 112, 100, 103, 99};
static const uint8_t CHROMA_Q[64] = {17, 18, 24, 47, 99, 99, 99, 99, 18, 21, 26, 66, 99, 99, 99, 99,
                                     24, 26, 56, 99, 99, 99, 99, 99, 47, 66, 99, 99, 99, 99, 99, 99,
                                     99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99,
                                     99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99, 99};

#define M ORC_IDCT_MATRIX

/* ITU-T T.81 Annex K.3 typical tables: code counts per length 1..16, then symbols. */
static const uint8_t K_DC_LUMA_BITS[16] = {0, 1, 5, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0};
static const uint8_t K_DC_CHROMA_BITS[16] = {0, 3, 1, 1, 1, 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0};
static const uint8_t K_DC_VALS[12] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11};
static const uint8_t K_AC_LUMA_BITS[16] = {0, 2, 1, 3, 3, 2, 4, 3, 5, 5, 4, 4, 0, 0, 1, 0x7d};
static const uint8_t K_AC_LUMA_VALS[162] = {
    0x01, 0x02, 0x03, 0x00, 0x04, 0x11, 0x05, 0x12, 0x21, 0x31, 0x41, 0x06, 0x13, 0x51, 0x61, 0x07, 0x22, 0x71,
    0x14, 0x32, 0x81, 0x91, 0xa1, 0x08, 0x23, 0x42, 0xb1, 0xc1, 0x15, 0x52, 0xd1, 0xf0, 0x24, 0x33, 0x62, 0x72,
    0x82, 0x09, 0x0a, 0x16, 0x17, 0x18, 0x19, 0x1a, 0x25, 0x26, 0x27, 0x28, 0x29, 0x2a, 0x34, 0x35, 0x36, 0x37,
    0x38, 0x39, 0x3a, 0x43, 0x44, 0x45, 0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58, 0x59,
    0x5a, 0x63, 0x64, 0x65, 0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a, 0x83,
    0x84, 0x85, 0x86, 0x87, 0x88, 0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99, 0x9a, 0xa2, 0xa3,
    0xa4, 0xa5, 0xa6, 0xa7, 0xa8, 0xa9, 0xaa, 0xb2, 0xb3, 0xb4, 0xb5, 0xb6, 0xb7, 0xb8, 0xb9, 0xba, 0xc2, 0xc3,
    0xc4, 0xc5, 0xc6, 0xc7, 0xc8, 0xc9, 0xca, 0xd2, 0xd3, 0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda, 0xe1, 0xe2,
    0xe3, 0xe4, 0xe5, 0xe6, 0xe7, 0xe8, 0xe9, 0xea, 0xf1, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};
static const uint8_t K_AC_CHROMA_BITS[16] = {0, 2, 1, 2, 4, 4, 3, 4, 7, 5, 4, 4, 0, 1, 2, 0x77};
static const uint8_t K_AC_CHROMA_VALS[162] = {
    0x00, 0x01, 0x02, 0x03, 0x11, 0x04, 0x05, 0x21, 0x31, 0x06, 0x12, 0x41, 0x51, 0x07, 0x61, 0x71, 0x13, 0x22,
    0x32, 0x81, 0x08, 0x14, 0x42, 0x91, 0xa1, 0xb1, 0xc1, 0x09, 0x23, 0x33, 0x52, 0xf0, 0x15, 0x62, 0x72, 0xd1,
    0x0a, 0x16, 0x24, 0x34, 0xe1, 0x25, 0xf1, 0x17, 0x18, 0x19, 0x1a, 0x26, 0x27, 0x28, 0x29, 0x2a, 0x35, 0x36,
    0x37, 0x38, 0x39, 0x3a, 0x43, 0x44, 0x45, 0x46, 0x47, 0x48, 0x49, 0x4a, 0x53, 0x54, 0x55, 0x56, 0x57, 0x58,
    0x59, 0x5a, 0x63, 0x64, 0x65, 0x66, 0x67, 0x68, 0x69, 0x6a, 0x73, 0x74, 0x75, 0x76, 0x77, 0x78, 0x79, 0x7a,
    0x82, 0x83, 0x84, 0x85, 0x86, 0x87, 0x88, 0x89, 0x8a, 0x92, 0x93, 0x94, 0x95, 0x96, 0x97, 0x98, 0x99, 0x9a,
    0xa2, 0xa3, 0xa4, 0xa5, 0xa6, 0xa7, 0xa8, 0xa9, 0xaa, 0xb2, 0xb3, 0xb4, 0xb5, 0xb6, 0xb7, 0xb8, 0xb9, 0xba,
    0xc2, 0xc3, 0xc4, 0xc5, 0xc6, 0xc7, 0xc8, 0xc9, 0xca, 0xd2, 0xd3, 0xd4, 0xd5, 0xd6, 0xd7, 0xd8, 0xd9, 0xda,
    0xe2, 0xe3, 0xe4, 0xe5, 0xe6, 0xe7, 0xe8, 0xe9, 0xea, 0xf2, 0xf3, 0xf4, 0xf5, 0xf6, 0xf7, 0xf8, 0xf9, 0xfa};

typedef struct {
    uint8_t cls, id;
    uint8_t counts[16];
    uint8_t symbols[256];
    size_t nsym;
} htab_t;

typedef struct {
    uint16_t bits;
    uint8_t length;
    uint8_t present;
} hcode_t;

/* encoder.rs:230-256 simple_dc_table / simple_ac_table */
static void simple_tables(htab_t *dc, htab_t *ac) {
    memset(dc, 0, sizeof *dc);
    memset(ac, 0, sizeof *ac);
    dc->cls = 0;
    dc->counts[3] = 12;
    for (int s = 0; s <= 11; s++) dc->symbols[dc->nsym++] = (uint8_t)s;
    ac->cls = 1;
    ac->counts[7] = 162;
    ac->symbols[ac->nsym++] = 0x00;
    ac->symbols[ac->nsym++] = 0xf0;
    for (int run = 0; run <= 15; run++)
        for (int size = 1; size <= 10; size++) ac->symbols[ac->nsym++] = (uint8_t)((run << 4) | size);
}

static void annex_table(htab_t *t, uint8_t cls, uint8_t id, const uint8_t *bits, const uint8_t *vals, size_t n) {
    memset(t, 0, sizeof *t);
    t->cls = cls;
    t->id = id;
    memcpy(t->counts, bits, 16);
    memcpy(t->symbols, vals, n);
    t->nsym = n;
}

/* encoder.rs:427-473 HuffmanEncoder::new */
static int huffman_codes(const htab_t *t, hcode_t codes[256]) {
    memset(codes, 0, 256 * sizeof(hcode_t));
    uint32_t code = 0;
    size_t si = 0;
    for (int li = 0; li < 16; li++) {
        const uint32_t length = (uint32_t)li + 1;
        if (code + t->counts[li] > (1u << length)) return 0;
        for (int k = 0; k < t->counts[li]; k++) {
            if (si >= t->nsym) return 0;
            codes[t->symbols[si]].bits = (uint16_t)code;
            codes[t->symbols[si]].length = (uint8_t)length;
            codes[t->symbols[si]].present = 1;
            si++;
            code++;
        }
        code <<= 1;
    }
    return si == t->nsym;
}

/* encoder.rs:219-228 scale_quantization */
static void scale_quantization(const uint8_t base[64], uint32_t quality, uint8_t out[64]) {
    const uint32_t scale = quality < 50 ? 5000 / quality : 200 - quality * 2;
    for (int i = 0; i < 64; i++) {
        uint32_t v = ((uint32_t)base[i] * scale + 50) / 100;
        out[i] = (uint8_t)(v < 1 ? 1 : v > 255 ? 255 : v);
    }
}

/* transform.rs:111-134 forward_dct_quantize */
void orc_jpeg_fdct_quantize(const uint8_t samples[64], const uint8_t quantization[64], int32_t out[64]) {
    double t[64];
    for (int i = 0; i < 64; i++) t[i] = 0.0;
    for (int y = 0; y < 8; y++)
        for (int u = 0; u < 8; u++)
            for (int x = 0; x < 8; x++) t[y * 8 + u] += M[x][u] * ((double)samples[y * 8 + x] - 128.0);
    for (int v = 0; v < 8; v++)
        for (int u = 0; u < 8; u++) {
            double value = 0.0;
            for (int y = 0; y < 8; y++) value += M[y][v] * t[y * 8 + u];
            /* f64::round (half away from zero), then `as i32` (saturating) */
            double r = round(value / (double)quantization[v * 8 + u]);
            out[v * 8 + u] = r >= 2147483647.0 ? 2147483647 : r <= -2147483648.0 ? (-2147483647 - 1) : (int32_t)r;
        }
}

void orc_jpeg_fdct_quantize_many(const uint8_t *samples, const uint8_t *quantization, size_t n, int32_t *out) {
    for (size_t b = 0; b < n; b++) orc_jpeg_fdct_quantize(samples + 64 * b, quantization + 64 * b, out + 64 * b);
}

/* ------------------------------------------------------------- writer --- */

/* encoder.rs:495-543 EntropyWriter: MSB-first bits, 0x00 stuffed after 0xFF,
 * the last byte padded with 1 bits. */
typedef struct {
    uint8_t *out;
    size_t cap, len;
    uint8_t cur, nbits;
    int overflow;
} writer_t;

static void put_byte(writer_t *w, uint8_t b) {
    if (w->len < w->cap) w->out[w->len] = b;
    else w->overflow = 1;
    w->len++;
}

static void write_bits(writer_t *w, uint32_t value, int count) {
    for (int i = count - 1; i >= 0; i--) {
        w->cur = (uint8_t)((w->cur << 1) | ((value >> i) & 1));
        if (++w->nbits == 8) {
            put_byte(w, w->cur);
            if (w->cur == 0xff) put_byte(w, 0);
            w->cur = 0;
            w->nbits = 0;
        }
    }
}

static void pad_bits(writer_t *w) {
    while (w->nbits != 0) write_bits(w, 1, 1);
}

static void put_segment(writer_t *w, uint8_t marker, const uint8_t *p, size_t n) {
    put_byte(w, 0xff);
    put_byte(w, marker);
    put_byte(w, (uint8_t)((n + 2) >> 8));
    put_byte(w, (uint8_t)(n + 2));
    for (size_t i = 0; i < n; i++) put_byte(w, p[i]);
}

/* encoder.rs:474-479 magnitude_category */
static int category(int32_t v) {
    uint32_t m = v < 0 ? (uint32_t)(-(int64_t)v) : (uint32_t)v;
    int c = 0;
    while (m) {
        c++;
        m >>= 1;
    }
    return c;
}

static int fail(orc_result *res, int status, const char *msg) {
    if (res) {
        res->status = status;
        snprintf(res->message, sizeof res->message, "%s", msg);
    }
    return status;
}

/*
 * Writes a baseline JPEG whose quantised coefficients are given: levels holds
 * 64 int32 per block (natural order, DC absolute) for every block of the scan
 * in scan order (MCU by MCU; within an MCU component by component, block row,
 * block column: encoder.rs:346-390). The header follows the reference encoder
 * (JFIF, DQT, SOF0, DHT, [DRI], SOS) with L->qt as the quantisation tables. A
 * DC difference needs category <= 11 and an AC level category <= 10: other
 * values give ORC_INVALID_ARGUMENT. *len receives the byte count; when it
 * exceeds cap the output is truncated and ORC_INVALID_ARGUMENT returned.
 */
int orc_jpeg_write_levels(const orc_jpeg_layout *L, const int32_t *levels, size_t nblocks, uint8_t *out, size_t cap,
                          size_t *len, orc_result *res) {
    if (res) {
        res->status = ORC_OK;
        res->message[0] = 0;
    }
    const uint32_t nc = L->ncomp;
    if (nc < 1 || nc > 3 || L->width == 0 || L->height == 0 || L->width > 65535 || L->height > 65535)
        return fail(res, ORC_INVALID_ARGUMENT, "layout");
    uint32_t hmax = 1, vmax = 1;
    for (uint32_t c = 0; c < nc; c++) {
        if (L->h[c] > hmax) hmax = L->h[c];
        if (L->v[c] > vmax) vmax = L->v[c];
    }
    const size_t mcu_cols = (L->width + hmax * 8 - 1) / (hmax * 8), mcu_rows = (L->height + vmax * 8 - 1) / (vmax * 8);
    size_t per_mcu = 0;
    for (uint32_t c = 0; c < nc; c++) per_mcu += (size_t)L->h[c] * L->v[c];
    if (nblocks != mcu_cols * mcu_rows * per_mcu) return fail(res, ORC_INVALID_ARGUMENT, "block count");

    htab_t tabs[4];
    int ntab;
    if (L->annex_k) {
        annex_table(&tabs[0], 0, 0, K_DC_LUMA_BITS, K_DC_VALS, 12);
        annex_table(&tabs[1], 1, 0, K_AC_LUMA_BITS, K_AC_LUMA_VALS, 162);
        annex_table(&tabs[2], 0, 1, K_DC_CHROMA_BITS, K_DC_VALS, 12);
        annex_table(&tabs[3], 1, 1, K_AC_CHROMA_BITS, K_AC_CHROMA_VALS, 162);
        ntab = nc > 1 ? 4 : 2;
    } else {
        simple_tables(&tabs[0], &tabs[1]);
        ntab = 2;
    }
    hcode_t dc[2][256], ac[2][256];
    for (int t = 0; t < ntab; t++)
        if (!huffman_codes(&tabs[t], tabs[t].cls ? ac[tabs[t].id] : dc[tabs[t].id]))
            return fail(res, ORC_INVALID_DATA, "JPEG Huffman table is oversubscribed");

    writer_t w = {out, cap, 0, 0, 0, 0};
    put_byte(&w, 0xff);
    put_byte(&w, 0xd8);
    {
        static const uint8_t jfif[14] = {'J', 'F', 'I', 'F', 0, 1, 2, 0, 0, 1, 0, 1, 0, 0};
        put_segment(&w, 0xe0, jfif, 14);
    }
    {   /* encoder.rs:269-283: table 0, then table 1 when there are chroma components */
        uint8_t p[130];
        size_t n = 0;
        int ntq = 1;
        for (uint32_t c = 0; c < nc; c++)
            if (L->tq[c] + 1 > ntq) ntq = L->tq[c] + 1;
        for (int t = 0; t < ntq && t < 2; t++) {
            p[n++] = (uint8_t)t;
            for (int k = 0; k < 64; k++) p[n++] = L->qt[t][ZZ[k]];
        }
        put_segment(&w, 0xdb, p, n);
    }
    {   /* encoder.rs:285-310 */
        uint8_t p[16];
        size_t n = 0;
        p[n++] = 8;
        p[n++] = (uint8_t)(L->height >> 8);
        p[n++] = (uint8_t)L->height;
        p[n++] = (uint8_t)(L->width >> 8);
        p[n++] = (uint8_t)L->width;
        p[n++] = (uint8_t)nc;
        for (uint32_t c = 0; c < nc; c++) {
            p[n++] = (uint8_t)(c + 1);
            p[n++] = (uint8_t)((L->h[c] << 4) | L->v[c]);
            p[n++] = L->tq[c];
        }
        put_segment(&w, 0xc0, p, n);
    }
    {   /* encoder.rs:312-325 */
        uint8_t p[4 * (17 + 256)];
        size_t n = 0;
        for (int t = 0; t < ntab; t++) {
            p[n++] = (uint8_t)((tabs[t].cls << 4) | tabs[t].id);
            memcpy(p + n, tabs[t].counts, 16);
            n += 16;
            memcpy(p + n, tabs[t].symbols, tabs[t].nsym);
            n += tabs[t].nsym;
        }
        put_segment(&w, 0xc4, p, n);
    }
    if (L->restart_interval) {
        const uint8_t p[2] = {(uint8_t)(L->restart_interval >> 8), (uint8_t)L->restart_interval};
        put_segment(&w, 0xdd, p, 2);
    }
    uint8_t sel[3];
    for (uint32_t c = 0; c < nc; c++) sel[c] = L->annex_k ? (L->tq[c] ? 1 : 0) : 0;
    {   /* encoder.rs:327-335 */
        uint8_t p[10];
        size_t n = 0;
        p[n++] = (uint8_t)nc;
        for (uint32_t c = 0; c < nc; c++) {
            p[n++] = (uint8_t)(c + 1);
            p[n++] = (uint8_t)((sel[c] << 4) | sel[c]);
        }
        p[n++] = 0;
        p[n++] = 63;
        p[n++] = 0;
        put_segment(&w, 0xda, p, n);
    }
    /* encode_scan + encode_block (encoder.rs:346-425) */
    int32_t pred[3] = {0, 0, 0};
    size_t b = 0, mcu = 0;
    uint32_t rst = 0;
    for (size_t my = 0; my < mcu_rows; my++)
        for (size_t mx = 0; mx < mcu_cols; mx++, mcu++) {
            if (L->restart_interval && mcu > 0 && mcu % L->restart_interval == 0) {
                pad_bits(&w);
                put_byte(&w, 0xff);
                put_byte(&w, (uint8_t)(0xd0 + (rst & 7)));
                rst++;
                pred[0] = pred[1] = pred[2] = 0;
            }
            for (uint32_t c = 0; c < nc; c++) {
                const hcode_t *dcc = dc[sel[c]], *acc = ac[sel[c]];
                for (uint32_t k = 0; k < (uint32_t)L->h[c] * L->v[c]; k++, b++) {
                    const int32_t *co = levels + 64 * b;
                    const int64_t diff64 = (int64_t)co[0] - pred[c];
                    pred[c] = co[0];
                    if (diff64 < -2047 || diff64 > 2047) return fail(res, ORC_INVALID_ARGUMENT, "DC difference");
                    const int32_t diff = (int32_t)diff64;
                    const int dsz = category(diff);
                    if (!dcc[dsz].present) return fail(res, ORC_INVALID_DATA, "JPEG Huffman table has no DC symbol");
                    write_bits(&w, dcc[dsz].bits, dcc[dsz].length);
                    if (dsz) write_bits(&w, (uint32_t)(diff < 0 ? diff + (1 << dsz) - 1 : diff), dsz);
                    int run = 0;
                    for (int z = 1; z < 64; z++) {
                        const int32_t v = co[ZZ[z]];
                        if (v == 0) {
                            run++;
                            continue;
                        }
                        if (v < -1023 || v > 1023) return fail(res, ORC_INVALID_ARGUMENT, "AC level");
                        while (run >= 16) {
                            write_bits(&w, acc[0xf0].bits, acc[0xf0].length);
                            run -= 16;
                        }
                        const int sz = category(v);
                        const int sym = (run << 4) | sz;
                        if (!acc[sym].present) return fail(res, ORC_INVALID_DATA, "JPEG Huffman table has no AC symbol");
                        write_bits(&w, acc[sym].bits, acc[sym].length);
                        write_bits(&w, (uint32_t)(v < 0 ? v + (1 << sz) - 1 : v), sz);
                        run = 0;
                    }
                    if (run != 0) write_bits(&w, acc[0x00].bits, acc[0x00].length);
                }
            }
        }
    pad_bits(&w);
    put_byte(&w, 0xff);
    put_byte(&w, 0xd9);
    *len = w.len;
    if (w.overflow) return fail(res, ORC_INVALID_ARGUMENT, "output capacity");
    return ORC_OK;
}

/*
 * encode_jpeg (encoder.rs:44-87): validation of the frame layout, scaled
 * Annex K quantisers, read_block edge replication, forward_dct_quantize, AC
 * levels clamped to +-1023, then the scan. Planes are stride == width.
 */
int orc_jpeg_encode(const orc_frame *frame, int quality, int annex_k, int restart_interval, uint8_t *out, size_t cap,
                    size_t *len, orc_result *res) {
    orc_jpeg_layout L;
    memset(&L, 0, sizeof L);
    if (frame->width == 0 || frame->height == 0 || frame->width > 65535 || frame->height > 65535)
        return fail(res, ORC_INVALID_DATA, "JPEG frame dimensions must be between 1 and 65535");
    if (frame->range == ORC_RANGE_LIMITED)
        return fail(res, ORC_UNSUPPORTED, "limited-range input requires conversion to full-range JPEG samples");
    switch (frame->format) {
    case ORC_FMT_GRAY8: L.ncomp = 1; L.h[0] = L.v[0] = 1; break;
    case ORC_FMT_YUV420P8: L.ncomp = 3; L.h[0] = 2; L.v[0] = 2; break;
    case ORC_FMT_YUV422P8: L.ncomp = 3; L.h[0] = 2; L.v[0] = 1; break;
    case ORC_FMT_YUV444P8: L.ncomp = 3; L.h[0] = 1; L.v[0] = 1; break;
    default: return fail(res, ORC_UNSUPPORTED, "pixel format is not supported by JPEG");
    }
    for (uint32_t c = 1; c < L.ncomp; c++) {
        L.h[c] = L.v[c] = 1;
        L.tq[c] = 1;
    }
    const uint32_t hmax = L.h[0], vmax = L.v[0];
    if (frame->plane_count != L.ncomp) return fail(res, ORC_INVALID_DATA, "plane count");
    for (uint32_t c = 0; c < L.ncomp; c++) {
        const size_t w = (frame->width * L.h[c] + hmax - 1) / hmax, h = (frame->height * L.v[c] + vmax - 1) / vmax;
        if (frame->planes[c].width != w || frame->planes[c].height != h)
            return fail(res, ORC_INVALID_DATA, "JPEG input plane has inconsistent dimensions, stride, or storage");
    }
    if (quality < 1 || quality > 100) return fail(res, ORC_INVALID_DATA, "JPEG quality must be between 1 and 100");
    if (restart_interval < 0 || restart_interval > 65535) return fail(res, ORC_INVALID_ARGUMENT, "restart interval");
    L.width = (uint32_t)frame->width;
    L.height = (uint32_t)frame->height;
    L.annex_k = annex_k ? 1 : 0;
    L.restart_interval = (uint16_t)restart_interval;
    scale_quantization(LUMA_Q, (uint32_t)quality, L.qt[0]);
    scale_quantization(CHROMA_Q, (uint32_t)quality, L.qt[1]);

    const size_t mcu_cols = (frame->width + hmax * 8 - 1) / (hmax * 8),
                 mcu_rows = (frame->height + vmax * 8 - 1) / (vmax * 8);
    size_t per_mcu = 0;
    for (uint32_t c = 0; c < L.ncomp; c++) per_mcu += (size_t)L.h[c] * L.v[c];
    const size_t nblocks = mcu_cols * mcu_rows * per_mcu;
    int32_t *levels = (int32_t *)malloc(nblocks * 64 * sizeof(int32_t));
    if (!levels) return fail(res, ORC_INTERNAL, "out of memory");
    size_t b = 0;
    uint8_t block[64];
    for (size_t my = 0; my < mcu_rows; my++)
        for (size_t mx = 0; mx < mcu_cols; mx++)
            for (uint32_t c = 0; c < L.ncomp; c++) {
                const orc_plane *pl = &frame->planes[c];
                for (uint32_t by = 0; by < L.v[c]; by++)
                    for (uint32_t bx = 0; bx < L.h[c]; bx++, b++) {
                        const size_t x = (mx * L.h[c] + bx) * 8, y = (my * L.v[c] + by) * 8;
                        for (size_t yy = 0; yy < 8; yy++) {  /* encoder.rs:392-402 read_block */
                            const size_t sy = y + yy < pl->height ? y + yy : pl->height - 1;
                            for (size_t xx = 0; xx < 8; xx++) {
                                const size_t sx = x + xx < pl->width ? x + xx : pl->width - 1;
                                block[yy * 8 + xx] = pl->data[sy * pl->width + sx];
                            }
                        }
                        int32_t *co = levels + 64 * b;
                        orc_jpeg_fdct_quantize(block, L.qt[L.tq[c]], co);
                        for (int k = 1; k < 64; k++) co[k] = co[k] < -1023 ? -1023 : co[k] > 1023 ? 1023 : co[k];
                    }
            }
    const int st = orc_jpeg_write_levels(&L, levels, nblocks, out, cap, len, res);
    free(levels);
    return st;
}
