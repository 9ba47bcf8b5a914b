/*
 * Oracle restatement of the MMRecode DV25 video decoder.
 * TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Follows, statement for statement:
 *   crates/codecs/dv/src/profile.rs  (detect_profile)
 *   crates/codecs/dv/src/dif.rs      (parse_frame, expected_id)
 *   crates/codecs/dv/src/decoder.rs  (decode_video_with_options ... inverse_248)
 *   crates/codecs/dv/src/tables.rs   (ZIGZAG_248, QUANT_*, IWEIGHT_*, VLC_*)
 *
 * The reference keeps every bitstream as a Vec<u8> of single bits; so does this
 * restatement (bit vectors below), to stay line-for-line comparable.
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

/* ------------------------------------------------------------------ */
/* tables.rs                                                            */
/* ------------------------------------------------------------------ */

static const int ZIGZAG_248[64] = {
    0,  8,  1,  9,  16, 24, 2,  10, 17, 25, 32, 40, 48, 56, 33, 41, 18, 26, 3,  11, 4,  12,
    19, 27, 34, 42, 49, 57, 50, 58, 35, 43, 20, 28, 5,  13, 6,  14, 21, 29, 36, 44, 51, 59,
    52, 60, 37, 45, 22, 30, 7,  15, 23, 31, 38, 46, 53, 61, 54, 62, 39, 47, 55, 63};
static const int ZIGZAG_88[64] = {
    0,  1,  8,  16, 9,  2,  3,  10, 17, 24, 32, 25, 18, 11, 4,  5,  12, 19, 26, 33, 40, 48,
    41, 34, 27, 20, 13, 6,  7,  14, 21, 28, 35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23,
    30, 37, 44, 51, 58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63};
static const uint8_t QUANT_SHIFTS[22][4] = {
    {3, 3, 4, 4}, {3, 3, 4, 4}, {2, 3, 3, 4}, {2, 3, 3, 4}, {2, 2, 3, 3}, {2, 2, 3, 3},
    {1, 2, 2, 3}, {1, 2, 2, 3}, {1, 1, 2, 2}, {1, 1, 2, 2}, {0, 1, 1, 2}, {0, 1, 1, 2},
    {0, 0, 1, 1}, {0, 0, 1, 1}, {0, 0, 0, 1}, {0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0},
    {0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}, {0, 0, 0, 0}};
static const int QUANT_OFFSET[4] = {6, 3, 0, 1};
static const int32_t IWEIGHT_88[64] = {
    32768, 16705, 16705, 17734, 17032, 17734, 18205, 18081, 18081, 18205, 18725, 18562, 19195,
    18562, 18725, 19266, 19091, 19705, 19705, 19091, 19266, 21407, 19643, 20267, 20228, 20267,
    19643, 21407, 22725, 21826, 20853, 20806, 20806, 20853, 21826, 22725, 23170, 23170, 21407,
    21400, 21407, 23170, 23170, 24598, 23786, 22018, 22018, 23786, 24598, 25251, 24465, 22654,
    24465, 25251, 25972, 25172, 25172, 25972, 26722, 27969, 26722, 29692, 29692, 31521};
static const int32_t IWEIGHT_248[64] = {
    32768, 16384, 16705, 16705, 17734, 17734, 17734, 17734, 18081, 18081, 18725, 18725, 21407,
    21407, 19091, 19091, 19195, 19195, 18205, 18205, 18725, 18725, 19705, 19705, 20267, 20267,
    21826, 21826, 23170, 23170, 20806, 20806, 20267, 20267, 19266, 19266, 21407, 21407, 20853,
    20853, 21400, 21400, 23786, 23786, 24465, 24465, 22018, 22018, 23170, 23170, 22725, 22725,
    24598, 24598, 24465, 24465, 25172, 25172, 27969, 27969, 25972, 25972, 29692, 29692};

/* VLC_LEN / VLC_RUN / VLC_LEVEL (tables.rs:50-105), run-length encoded for brevity:
 * lengths are non-decreasing, so they are given as (length, count) pairs. */
static const uint16_t VLC_LEN_RLE[][2] = {{2, 1}, {3, 1}, {4, 4}, {5, 4}, {6, 4}, {7, 8}, {8, 16},
                                         {9, 16}, {10, 7}, {11, 8}, {12, 20}, {13, 64}, {15, 256}};
static const uint8_t VLC_RUN_HEAD[153] = {
    0, 0, 127, 1, 0, 0, 2, 1, 0, 0, 3, 4, 0, 0, 5, 6, 2, 1, 1, 0, 0, 0, 7, 8, 9, 10, 3, 4, 2, 1, 1,
    1, 0, 0, 0, 0, 0, 0, 11, 12, 13, 14, 5, 6, 3, 4, 2, 2, 1, 0, 0, 0, 0, 0, 5, 3, 3, 2, 1, 1, 1,
    0, 1, 6, 4, 3, 1, 1, 1, 2, 3, 4, 5, 7, 8, 9, 10, 7, 8, 4, 3, 2, 2, 2, 2, 2, 1, 1, 1, 0, 1, 2,
    3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26, 27,
    28, 29, 30, 31, 32, 33, 34, 35, 36, 37, 38, 39, 40, 41, 42, 43, 44, 45, 46, 47, 48, 49, 50, 51,
    52, 53, 54, 55, 56, 57, 58, 59, 60, 61, 62, 63};
static const uint8_t VLC_LEVEL_HEAD[153] = {
    1, 2, 0, 1, 3, 4, 1, 2, 5, 6, 1, 1, 7, 8, 1, 1, 2, 3, 4, 9, 10, 11, 1, 1, 1, 1, 2, 2, 3, 5, 6,
    7, 12, 13, 14, 15, 16, 17, 1, 1, 1, 1, 2, 2, 3, 3, 4, 5, 8, 18, 19, 20, 21, 22, 3, 4, 5, 6, 9,
    10, 11, 0, 0, 3, 4, 6, 12, 13, 14, 0, 0, 0, 0, 2, 2, 2, 2, 3, 3, 5, 7, 7, 8, 9, 10, 11, 15, 16,
    17, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
    0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0,
    0, 0};
/* The final 256 entries (length 15) are run 0 with levels 0..255. */

typedef struct { uint16_t code; uint8_t len; uint8_t run; int16_t level; } vlc_t;
static vlc_t VLC[746];
static int VLC_COUNT = 0;

/* decoder.rs:319-354 vlc_entries: canonical codes, sign bit appended, stable sort by len. */
static void build_vlc(void) {
    if (VLC_COUNT) return;
    uint8_t len_of[409], run_of[409];
    int16_t lvl_of[409];
    int n = 0;
    for (size_t i = 0; i < sizeof(VLC_LEN_RLE) / sizeof(VLC_LEN_RLE[0]); i++)
        for (int k = 0; k < VLC_LEN_RLE[i][1]; k++) len_of[n++] = (uint8_t)VLC_LEN_RLE[i][0];
    for (int i = 0; i < 409; i++) {
        if (i < 153) {
            run_of[i] = VLC_RUN_HEAD[i];
            lvl_of[i] = VLC_LEVEL_HEAD[i];
        } else {
            run_of[i] = 0;
            lvl_of[i] = (int16_t)(i - 153);
        }
    }
    vlc_t tmp[746];
    int m = 0;
    uint32_t canonical = 0;
    for (int i = 0; i < 409; i++) {
        uint8_t len = len_of[i];
        uint32_t code = canonical >> (32 - len);
        canonical += 1u << (32 - len);
        int16_t level = lvl_of[i];
        if (level == 0) {
            tmp[m++] = (vlc_t){(uint16_t)code, len, run_of[i], 0};
        } else {
            tmp[m++] = (vlc_t){(uint16_t)(code << 1), (uint8_t)(len + 1), run_of[i], level};
            tmp[m++] = (vlc_t){(uint16_t)((code << 1) | 1), (uint8_t)(len + 1), run_of[i], (int16_t)-level};
        }
    }
    /* stable sort by len */
    int k = 0;
    for (int L = 0; L <= 16; L++)
        for (int i = 0; i < m; i++)
            if (tmp[i].len == L) VLC[k++] = tmp[i];
    VLC_COUNT = k;
}

/* ------------------------------------------------------------------ */
/* bit vectors (decoder.rs:604-626)                                     */
/* ------------------------------------------------------------------ */

typedef struct { uint8_t *b; size_t n, cap; } bits_t;

static void bits_push(bits_t *v, uint8_t bit) {
    if (v->n == v->cap) {
        v->cap = v->cap ? v->cap * 2 : 64;
        v->b = realloc(v->b, v->cap);
    }
    v->b[v->n++] = bit;
}
static void bits_extend(bits_t *v, const uint8_t *src, size_t n) {
    for (size_t i = 0; i < n; i++) bits_push(v, src[i]);
}
static void bits_free(bits_t *v) {
    free(v->b);
    memset(v, 0, sizeof(*v));
}
static uint32_t bits_value(const uint8_t *bits, size_t n) {
    uint32_t v = 0;
    for (size_t i = 0; i < n; i++) v = (v << 1) | bits[i];
    return v;
}
static int32_t signed_bits(const uint8_t *bits, size_t n) {
    int32_t value = (int32_t)bits_value(bits, n);
    if (n > 0 && bits[0] == 1) return value - (1 << n);
    return value;
}

/* ------------------------------------------------------------------ */
/* profile.rs / dif.rs                                                  */
/* ------------------------------------------------------------------ */

typedef struct {
    int pal;          /* 0 = 525/60, 1 = 625/50 */
    size_t frame_size, dif_sequences, width, height;
    uint32_t format;
} profile_t;

/* profile.rs:87-127 */
static int detect_profile(const uint8_t *d, size_t len, profile_t *p, orc_result *res) {
    if (len < 4) {
        set_err(res, ORC_INVALID_DATA, "DV profile detection needs 4 header bytes, found %zu", len);
        return ORC_INVALID_DATA;
    }
    if ((d[0] >> 5) != 0) {
        set_err(res, ORC_INVALID_DATA, "first DIF block is not a header");
        return ORC_INVALID_DATA;
    }
    if ((d[3] & 0x80) == 0) *p = (profile_t){0, 120000, 10, 720, 480, ORC_FMT_YUV411P8};
    else *p = (profile_t){1, 144000, 12, 720, 576, ORC_FMT_YUV420P8};
    if (len != p->frame_size) {
        set_err(res, ORC_INVALID_DATA, "DV header identifies a %zu-byte frame, found %zu bytes", p->frame_size, len);
        return ORC_INVALID_DATA;
    }
    return ORC_OK;
}

/* dif.rs:235-253 expected_id: returns section (0..4) and number */
static void expected_id(size_t position, int *section, int *number) {
    if (position == 0) {
        *section = 0;
        *number = 0;
    } else if (position <= 2) {
        *section = 1;
        *number = (int)(position - 1);
    } else if (position <= 5) {
        *section = 2;
        *number = (int)(position - 3);
    } else {
        size_t av = position - 6;
        size_t within = av % 16;
        if (within == 0) {
            *section = 3;
            *number = (int)(av / 16);
        } else {
            *section = 4;
            *number = (int)((av - av / 16 - 1) & 0xff);
        }
    }
}

/* dif.rs:181-232 parse_frame: one flag per DIF block when it carries any issue */
static int parse_frame(const uint8_t *d, size_t len, profile_t *p, uint8_t **issue_flags, size_t *issue_count,
                       size_t *first_issue, orc_result *res) {
    int st = detect_profile(d, len, p, res);
    if (st) return st;
    size_t nblocks = p->dif_sequences * 150;
    uint8_t *flags = calloc(nblocks, 1);
    size_t count = 0;
    *first_issue = (size_t)-1;
    for (size_t index = 0; index < nblocks; index++) {
        const uint8_t *b = d + index * 80;
        int section = b[0] >> 5;
        int sequence = b[1] >> 4;
        int number = b[2];
        size_t phys_seq = index / 150, pos = index % 150;
        int es, en;
        expected_id(pos, &es, &en);
        int issues = 0;
        if (section != es) issues++;
        if ((size_t)sequence != phys_seq) issues++;
        if (number != en) issues++;
        if (issues) {
            flags[index] = 1;
            if (*first_issue == (size_t)-1) *first_issue = index * 80;
        }
        count += (size_t)issues;
    }
    *issue_flags = flags;
    *issue_count = count;
    return ORC_OK;
}

int orc_dv_issue_count(const uint8_t *data, size_t len, size_t *count, size_t *first_offset, orc_result *res) {
    res->status = ORC_OK;
    res->message[0] = 0;
    profile_t p;
    uint8_t *flags = NULL;
    int st = parse_frame(data, len, &p, &flags, count, first_offset, res);
    free(flags);
    return st;
}

/* ------------------------------------------------------------------ */
/* decoder.rs                                                           */
/* ------------------------------------------------------------------ */

static const size_t BLOCK_BITS[6] = {112, 112, 112, 112, 80, 80};

typedef struct {
    int32_t coefficients[64];
    size_t position;
    int dct_mode;
    size_t class_;
    size_t quantization;
    bits_t partial;
    int complete;
} dctblock_t;

/* decoder.rs:290-310 inverse_factor_for_encoding */
static int32_t inverse_factor(size_t quantization, size_t class_, int dct_mode, size_t position) {
    size_t q = quantization + (size_t)QUANT_OFFSET[class_];
    size_t area = position <= 5 ? 0 : position <= 20 ? 1 : position <= 42 ? 2 : 3;
    int32_t weight = dct_mode ? IWEIGHT_248[position] : IWEIGHT_88[position];
    size_t class_shift = class_ == 3;
    return weight << (QUANT_SHIFTS[q][area] + 1 + class_shift);
}

/* decoder.rs:312-317 decode_vlc */
static const vlc_t *decode_vlc(const uint8_t *bits, size_t n) {
    for (int i = 0; i < VLC_COUNT; i++) {
        size_t len = VLC[i].len;
        if (n >= len && bits_value(bits, len) == VLC[i].code) return &VLC[i];
    }
    return NULL;
}

/* decoder.rs:245-284 consume_ac: returns leftover bits in *out (caller frees) */
static int consume_ac(dctblock_t *block, const uint8_t *input, size_t n, bits_t *out, orc_result *res) {
    memset(out, 0, sizeof(*out));
    if (block->complete) {
        bits_extend(out, input, n);
        return ORC_OK;
    }
    bits_t bits = block->partial; /* std::mem::take */
    memset(&block->partial, 0, sizeof(block->partial));
    bits_extend(&bits, input, n);
    size_t cursor = 0;
    for (;;) {
        const uint8_t *remaining = bits.b + cursor;
        size_t rn = bits.n - cursor;
        const vlc_t *e = decode_vlc(remaining, rn);
        if (e) {
            cursor += e->len;
            block->position += (size_t)e->run + 1;
            if (block->position >= 64) {
                block->complete = 1;
                bits_extend(out, bits.b + cursor, bits.n - cursor);
                bits_free(&bits);
                return ORC_OK;
            }
            if (e->level != 0) {
                int32_t factor = inverse_factor(block->quantization, block->class_, block->dct_mode, block->position);
                int32_t level = ((int32_t)e->level * factor + 8192) >> 14;
                const int *scan = block->dct_mode ? ZIGZAG_248 : ZIGZAG_88;
                block->coefficients[scan[block->position]] = level;
            }
        } else if (rn < 16) {
            bits_extend(&block->partial, remaining, rn);
            bits_free(&bits);
            return ORC_OK;
        } else {
            bits_free(&bits);
            set_err(res, ORC_INVALID_DATA, "invalid DV variable-length coefficient code");
            return ORC_INVALID_DATA;
        }
    }
}

/* decoder.rs:235-243 consume_pool (also :225-233 for the segment level) */
static int consume_pool(dctblock_t *blocks, size_t nblocks, const uint8_t *pool, size_t n, bits_t *out,
                        orc_result *res) {
    bits_t remaining;
    memset(&remaining, 0, sizeof remaining);
    bits_extend(&remaining, pool, n);
    for (size_t i = 0; i < nblocks; i++) {
        if (!blocks[i].complete && remaining.n != 0) {
            bits_t next;
            int st = consume_ac(&blocks[i], remaining.b, remaining.n, &next, res);
            bits_free(&remaining);
            if (st) return st;
            remaining = next;
        }
    }
    *out = remaining;
    return ORC_OK;
}

/* decoder.rs:193-223 decode_macroblock */
static int decode_macroblock(const uint8_t *bytes, dctblock_t blocks[6], bits_t *overflow, orc_result *res) {
    size_t quantization = bytes[3] & 0x0f;
    uint8_t payload[608];
    for (int i = 0; i < 76; i++)
        for (int s = 7; s >= 0; s--) payload[i * 8 + (7 - s)] = (bytes[4 + i] >> s) & 1;
    size_t cursor = 0;
    bits_t mb_pool;
    memset(&mb_pool, 0, sizeof mb_pool);
    for (int b = 0; b < 6; b++) {
        const uint8_t *region = payload + cursor;
        cursor += BLOCK_BITS[b];
        dctblock_t *blk = &blocks[b];
        memset(blk, 0, sizeof(*blk));
        int32_t dc = signed_bits(region, 9);
        blk->dct_mode = region[9] != 0;
        blk->class_ = bits_value(region + 10, 2);
        blk->quantization = quantization;
        blk->coefficients[0] = dc * 4 + 1024;
        bits_t leftover;
        int st = consume_ac(blk, region + 12, BLOCK_BITS[b] - 12, &leftover, res);
        if (st) {
            bits_free(&mb_pool);
            return st;
        }
        if (blk->complete) bits_extend(&mb_pool, leftover.b, leftover.n);
        bits_free(&leftover);
    }
    int st = consume_pool(blocks, 6, mb_pool.b, mb_pool.n, overflow, res);
    bits_free(&mb_pool);
    return st;
}

/* decoder.rs:395-422 macroblock_coordinates */
static void macroblock_coordinates(const profile_t *p, size_t sequence, size_t slot, size_t xy[5][2]) {
    static const size_t OFF[5] = {2, 6, 8, 0, 4};
    static const size_t SHUF3[5] = {18, 9, 27, 0, 36};
    static const size_t L_START_SHUFFLED[5] = {9, 4, 13, 0, 18};
    static const size_t SERPENT1[27] = {0, 1, 2, 2, 1, 0, 0, 1, 2, 2, 1, 0, 0, 1, 2, 2, 1, 0, 0, 1, 2, 2, 1, 0, 0, 1, 2};
    static const size_t SERPENT2[30] = {0, 1, 2, 3, 4, 5, 5, 4, 3, 2, 1, 0, 0, 1, 2,
                                        3, 4, 5, 5, 4, 3, 2, 1, 0, 0, 1, 2, 3, 4, 5};
    for (size_t m = 0; m < 5; m++) {
        if (p->pal) {
            size_t x = SHUF3[m] + slot / 3;
            size_t y = SERPENT1[slot] + ((sequence + OFF[m]) % p->dif_sequences) * 3;
            xy[m][0] = x * 2;
            xy[m][1] = y * 2;
        } else {
            size_t row = (sequence + OFF[m]) % p->dif_sequences;
            size_t k = slot + (size_t)(m == 1 || m == 2) * 3;
            size_t x = L_START_SHUFFLED[m] + k / 6;
            size_t y = SERPENT2[k] + row * 6;
            if (x > 21) y = y * 2 - row * 6;
            xy[m][0] = x * 4;
            xy[m][1] = y;
        }
    }
}

/* ---- transforms (decoder.rs:507-602) ---- */

/*
 * cos(((2x+1) as f64 * u as f64 * PI) / 16.0): the argument is fl(k*PI)/16 with k=(2x+1)u.
 * The reference calls libm cos at run time; the oracle reads the same doubles from a table
 * (gen_cos_table.py checks that glibc cos returns exactly these values) so that it gives
 * identical results on every host libm.
 */
#include "cos_table.h"
static double dv_cos16(int k) { return ORC_COS16[k]; }
/* cos(((2y+1) as f64 * v as f64 * PI) / 8.0) == cos(fl(2k*PI)/16): doubling is exact */
static double dv_cos8(int k) { return ORC_COS16[2 * k]; }

double orc_dv_cos(int k) { return dv_cos16(k); }

static const double FRAC_1_SQRT_2 = 0.7071067811865476;

static uint8_t round_clamp_u8(double v) {
    double r = round(v);
    if (r < 0.0) r = 0.0;
    if (r > 255.0) r = 255.0;
    return (uint8_t)r;
}

/* decoder.rs:520-548 inverse_88 */
void orc_dv_idct88(const int32_t c[64], uint8_t out[64]) {
    for (int y = 0; y < 8; y++)
        for (int x = 0; x < 8; x++) {
            double sum = 0.0;
            for (int v = 0; v < 8; v++)
                for (int u = 0; u < 8; u++) {
                    double cu = u == 0 ? FRAC_1_SQRT_2 : 1.0;
                    double cv = v == 0 ? FRAC_1_SQRT_2 : 1.0;
                    sum += cu * cv * (double)c[v * 8 + u] * dv_cos16((2 * x + 1) * u) * dv_cos16((2 * y + 1) * v);
                }
            out[y * 8 + x] = round_clamp_u8(sum / 4.0);
        }
}

/* decoder.rs:555-602 inverse_248 */
void orc_dv_idct248(const int32_t c[64], uint8_t out[64]) {
    double butterfly[64];
    for (int pair = 0; pair < 4; pair++)
        for (int u = 0; u < 8; u++) {
            double first = (double)c[pair * 16 + u];
            double second = (double)c[pair * 16 + 8 + u];
            butterfly[pair * 16 + u] = first + second;
            butterfly[pair * 16 + 8 + u] = first - second;
        }
    double horizontal[64];
    for (int row = 0; row < 8; row++)
        for (int x = 0; x < 8; x++) {
            double sum = 0.0;
            for (int u = 0; u < 8; u++) {
                double cu = u == 0 ? FRAC_1_SQRT_2 : 1.0;
                sum += cu * butterfly[row * 8 + u] * dv_cos16((2 * x + 1) * u);
            }
            horizontal[row * 8 + x] = sum / 2.0;
        }
    for (int field = 0; field < 2; field++)
        for (int y = 0; y < 4; y++)
            for (int x = 0; x < 8; x++) {
                double sum = 0.0;
                for (int v = 0; v < 4; v++) {
                    double cv = v == 0 ? FRAC_1_SQRT_2 : 1.0;
                    sum += cv * horizontal[(v * 2 + field) * 8 + x] * dv_cos8((2 * y + 1) * v);
                }
                out[(y * 2 + field) * 8 + x] = round_clamp_u8(sum / 2.0);
            }
}

void orc_dv_idct88_many(const int32_t *coefficients, size_t n, uint8_t *out) {
    for (size_t b = 0; b < n; b++) orc_dv_idct88(coefficients + 64 * b, out + 64 * b);
}

void orc_dv_idct248_many(const int32_t *coefficients, size_t n, uint8_t *out) {
    for (size_t b = 0; b < n; b++) orc_dv_idct248(coefficients + 64 * b, out + 64 * b);
}

/* decoder.rs:470-505 put_block / put_split_chroma */
static int put_block(orc_plane *pl, size_t x, size_t y, const uint8_t px[64], orc_result *res) {
    if (x + 8 > pl->width || y + 8 > pl->height) {
        set_err(res, ORC_INVALID_DATA, "DV macroblock placement (%zu, %zu) exceeds %zux%zu plane", x, y, pl->width,
                pl->height);
        return ORC_INVALID_DATA;
    }
    for (size_t row = 0; row < 8; row++) memcpy(pl->data + (y + row) * pl->width + x, px + row * 8, 8);
    return ORC_OK;
}

static int put_split_chroma(orc_plane *pl, size_t x, size_t y, const uint8_t px[64], orc_result *res) {
    for (size_t row = 0; row < 8; row++) {
        size_t top = (y + row) * pl->width + x;
        size_t bottom = (y + 8 + row) * pl->width + x;
        if (bottom + 4 > pl->width * pl->height) {
            set_err(res, ORC_INVALID_DATA, "split DV chroma placement exceeds plane");
            return ORC_INVALID_DATA;
        }
        memcpy(pl->data + top, px + row * 8, 4);
        memcpy(pl->data + bottom, px + row * 8 + 4, 4);
    }
    return ORC_OK;
}

/* decoder.rs:432-468 place_macroblock */
static int place_macroblock(const profile_t *p, orc_plane planes[3], dctblock_t blocks[6], size_t mb_x, size_t mb_y,
                            orc_result *res) {
    uint8_t px[6][64];
    for (int i = 0; i < 6; i++) {
        if (blocks[i].dct_mode) orc_dv_idct248(blocks[i].coefficients, px[i]);
        else orc_dv_idct88(blocks[i].coefficients, px[i]);
    }
    size_t x = mb_x * 8, y = mb_y * 8;
    int st;
    if (p->pal) {
        if ((st = put_block(&planes[0], x, y, px[0], res))) return st;
        if ((st = put_block(&planes[0], x + 8, y, px[1], res))) return st;
        if ((st = put_block(&planes[0], x, y + 8, px[2], res))) return st;
        if ((st = put_block(&planes[0], x + 8, y + 8, px[3], res))) return st;
        if ((st = put_block(&planes[2], x / 2, y / 2, px[4], res))) return st;
        if ((st = put_block(&planes[1], x / 2, y / 2, px[5], res))) return st;
    } else if (mb_x < 88) {
        for (size_t i = 0; i < 4; i++)
            if ((st = put_block(&planes[0], x + i * 8, y, px[i], res))) return st;
        if ((st = put_block(&planes[2], x / 4, y, px[4], res))) return st;
        if ((st = put_block(&planes[1], x / 4, y, px[5], res))) return st;
    } else {
        if ((st = put_block(&planes[0], x, y, px[0], res))) return st;
        if ((st = put_block(&planes[0], x + 8, y, px[1], res))) return st;
        if ((st = put_block(&planes[0], x, y + 8, px[2], res))) return st;
        if ((st = put_block(&planes[0], x + 8, y + 8, px[3], res))) return st;
        if ((st = put_split_chroma(&planes[2], x / 4, y, px[4], res))) return st;
        if ((st = put_split_chroma(&planes[1], x / 4, y, px[5], res))) return st;
    }
    return ORC_OK;
}

static void free_blocks(dctblock_t *b, size_t n) {
    for (size_t i = 0; i < n; i++) bits_free(&b[i].partial);
}

size_t orc_dv_vlc_entries(uint16_t *code, uint8_t *len, uint8_t *run, int16_t *level, size_t cap) {
    build_vlc();
    size_t n = 0;
    for (int i = 0; i < VLC_COUNT && n < cap; i++, n++) {
        code[n] = VLC[i].code;
        len[n] = VLC[i].len;
        run[n] = VLC[i].run;
        level[n] = VLC[i].level;
    }
    return n;
}

/* Coefficient capture for the transform tests (orc_dv_coefficients): every
 * decoded block's coefficients and DCT mode, in segment order. */
static int32_t *g_cap_coef;
static uint8_t *g_cap_mode;
static size_t g_cap_n, g_cap_cap;

/* decoder.rs:152-191 decode_segment */
static int decode_segment(const uint8_t *data, const profile_t *p, const uint8_t *issue_flags, orc_plane planes[3],
                          size_t sequence, size_t slot, orc_result *res) {
    dctblock_t blocks[30];
    memset(blocks, 0, sizeof blocks);
    bits_t segment_pool;
    memset(&segment_pool, 0, sizeof segment_pool);
    int st = ORC_OK;
    for (size_t m = 0; m < 5; m++) {
        size_t vn = slot * 5 + m;
        size_t block_index = sequence * 150 + 7 + (vn / 15) * 16 + vn % 15;
        if (issue_flags[block_index]) {
            set_err(res, ORC_INVALID_DATA, "DV video segment %zu in sequence %zu has a damaged DIF identifier", slot,
                    sequence);
            st = ORC_INVALID_DATA;
            goto done;
        }
        bits_t overflow;
        st = decode_macroblock(data + block_index * 80, blocks + m * 6, &overflow, res);
        if (st) goto done;
        bits_extend(&segment_pool, overflow.b, overflow.n);
        bits_free(&overflow);
    }
    {
        bits_t rest;
        st = consume_pool(blocks, 30, segment_pool.b, segment_pool.n, &rest, res);
        bits_free(&rest);
        if (st) goto done;
    }
    for (int i = 0; i < 30; i++)
        if (!blocks[i].complete) {
            set_err(res, ORC_INVALID_DATA, "DV video segment %zu in sequence %zu has incomplete coefficients", slot,
                    sequence);
            st = ORC_INVALID_DATA;
            goto done;
        }
    if (g_cap_coef)
        for (int i = 0; i < 30 && g_cap_n < g_cap_cap; i++, g_cap_n++) {
            memcpy(g_cap_coef + 64 * g_cap_n, blocks[i].coefficients, 64 * sizeof(int32_t));
            g_cap_mode[g_cap_n] = (uint8_t)(blocks[i].dct_mode != 0);
        }
    {
        size_t xy[5][2];
        macroblock_coordinates(p, sequence, slot, xy);
        for (int m = 0; m < 5; m++) {
            st = place_macroblock(p, planes, blocks + m * 6, xy[m][0], xy[m][1], res);
            if (st) goto done;
        }
    }
done:
    free_blocks(blocks, 30);
    bits_free(&segment_pool);
    return st;
}

/* decoder.rs:87-150 decode_video_with_options (after dif.rs parse_frame) */
int orc_dv_decode(const uint8_t *data, size_t len, int conceal, orc_frame *out, orc_dv_concealed *concealed,
                  size_t concealed_cap, size_t *concealed_count, orc_result *res) {
    build_vlc();
    res->status = ORC_OK;
    res->message[0] = 0;
    memset(out, 0, sizeof(*out));
    if (concealed_count) *concealed_count = 0;
    profile_t p;
    uint8_t *flags = NULL;
    size_t issues, first_issue;
    int st = parse_frame(data, len, &p, &flags, &issues, &first_issue, res);
    if (st) return st;
    size_t cw = p.pal ? p.width / 2 : p.width / 4;
    size_t ch = p.pal ? p.height / 2 : p.height;
    orc_plane planes[3];
    planes[0] = (orc_plane){malloc(p.width * p.height), p.width, p.height};
    planes[1] = (orc_plane){malloc(cw * ch), cw, ch};
    planes[2] = (orc_plane){malloc(cw * ch), cw, ch};
    memset(planes[0].data, 16, p.width * p.height);
    memset(planes[1].data, 128, cw * ch);
    memset(planes[2].data, 128, cw * ch);
    for (size_t sequence = 0; sequence < p.dif_sequences; sequence++)
        for (size_t slot = 0; slot < 27; slot++) {
            orc_result seg_res;
            int e = decode_segment(data, &p, flags, planes, sequence, slot, &seg_res);
            if (e) {
                if (!conceal) {
                    *res = seg_res;
                    free(flags);
                    for (int i = 0; i < 3; i++) free(planes[i].data);
                    return e;
                }
                if (concealed_count) {
                    if (concealed && *concealed_count < concealed_cap)
                        concealed[*concealed_count] = (orc_dv_concealed){sequence, slot};
                    (*concealed_count)++;
                }
            }
        }
    free(flags);
    out->format = p.format;
    out->range = ORC_RANGE_LIMITED;
    out->width = p.width;
    out->height = p.height;
    out->plane_count = 3;
    for (int i = 0; i < 3; i++) out->planes[i] = planes[i];
    return ORC_OK;
}

/* The dequantised coefficients (natural order) and DCT modes of every block of a
 * frame, as decode_segment hands them to the transforms, in segment order (30
 * blocks per segment). Returns the number of blocks written (at most cap), or 0
 * when the frame fails. Not thread-safe (test infrastructure). */
size_t orc_dv_coefficients(const uint8_t *data, size_t len, int32_t *coef, uint8_t *modes, size_t cap) {
    orc_frame fr;
    orc_result res;
    g_cap_coef = coef;
    g_cap_mode = modes;
    g_cap_n = 0;
    g_cap_cap = cap;
    int st = orc_dv_decode(data, len, 0, &fr, NULL, 0, NULL, &res);
    size_t n = g_cap_n;
    g_cap_coef = NULL;
    g_cap_mode = NULL;
    if (st) return 0;
    orc_frame_free(&fr);
    return n;
}
