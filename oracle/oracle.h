/*
 * CPU oracle for the MMRecode MJPEG / DV25 intra-decode path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a statement-for-statement C restatement of
 * the reference decoder (markusmoenig/MMRecode, Rust) used as the checker for
 * the CUDA implementation. Nothing in the product library links, includes or
 * calls this code; only tests/, the smoke check and the CPU-baseline leg of
 * bench.py load it.
 *
 * It must be compiled with -ffp-contract=off: the reference IDCTs are IEEE-754
 * binary64 multiply/add sequences in a fixed order, and Rust never contracts
 * a*b+c into an FMA.
 *
 * Parity pins: the reference's own known-answer tests and fixtures (see
 * tests/test_oracle.py) -- IDCT DC cases, entropy known answers, the grey
 * restart vector, fixture dimensions/formats, error vectors and the DV
 * constant-96 round trip.
 */
#ifndef MMR_ORACLE_H
#define MMR_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes: crates/capi/src/lib.rs:26-32 */
#define ORC_OK 0
#define ORC_INVALID_ARGUMENT 1
#define ORC_INVALID_DATA 2
#define ORC_UNSUPPORTED 3
#define ORC_INVALID_STATE 4
#define ORC_INTERNAL 100

/* Pixel formats: crates/capi/src/lib.rs:34-38 */
#define ORC_FMT_GRAY8 1
#define ORC_FMT_YUV420P8 2
#define ORC_FMT_YUV422P8 3
#define ORC_FMT_YUV444P8 4
#define ORC_FMT_YUV411P8 5

#define ORC_RANGE_FULL 1
#define ORC_RANGE_LIMITED 2

typedef struct orc_plane {
    uint8_t *data; /* malloc'd, stride == width */
    size_t width;
    size_t height;
} orc_plane;

typedef struct orc_frame {
    uint32_t format;
    uint32_t range;
    size_t width;
    size_t height;
    size_t plane_count;
    orc_plane planes[3];
} orc_frame;

/* Result of one oracle call: status + reference-style diagnostic. */
typedef struct orc_result {
    int status;
    char message[512];
} orc_result;

/* ---- MJPEG (crates/codecs/mjpeg) ---- */

/* Parse-only view used by the parser tests (parser.rs:18-81, 373-414). */
typedef struct orc_jpeg_info {
    size_t width, height;       /* first SOF0 */
    size_t component_count;
    size_t scan_count;
    size_t data_offset;         /* first entropy scan */
    size_t data_length;
    size_t restart_count;       /* RST markers recorded in the first scan */
    size_t restart_offsets[64]; /* first 64 of them */
    uint8_t restart_numbers[64];
    size_t segment_count;
    uint8_t last_marker;        /* code of the last segment */
    size_t trailing_length;
} orc_jpeg_info;

int orc_jpeg_parse(const uint8_t *data, size_t len, orc_jpeg_info *info, orc_result *res);

/*
 * decode_jpeg + into_video_frame (decoder.rs:140-167, 69-126). On success the
 * frame owns malloc'd planes (free with orc_frame_free). *color_model receives
 * the JpegColorModel ordinal (0 Grayscale, 1 YCbCr, 2 Rgb, 3 Cmyk, 4 Ycck,
 * 5 Unknown) when decoding got that far, else -1.
 */
int orc_jpeg_decode(const uint8_t *data, size_t len, orc_frame *out, int *color_model,
                    orc_result *res);

/* transform.rs:86-109 on one block (natural order, dequantised). */
void orc_jpeg_idct(const int32_t coefficients[64], uint8_t out[64]);

/* ---- DV25 (crates/codecs/dv) ---- */

typedef struct orc_dv_concealed {
    size_t sequence;
    size_t slot;
} orc_dv_concealed;

/*
 * parse_frame + decode_video_with_options (dif.rs:181-232, decoder.rs:87-150).
 * With conceal != 0 failed segments are left at limited-range black and listed
 * in concealed[0..*concealed_count) (capacity given by concealed_cap).
 */
int orc_dv_decode(const uint8_t *data, size_t len, int conceal, orc_frame *out,
                  orc_dv_concealed *concealed, size_t concealed_cap, size_t *concealed_count,
                  orc_result *res);

/* Number of structural DIF issues found by parse_frame (dif.rs:181-232). */
int orc_dv_issue_count(const uint8_t *data, size_t len, size_t *count, size_t *first_offset,
                       orc_result *res);

/* The DV VLC codes (decoder.rs:319-354 vlc_entries, sign bits appended, sorted by
 * length): up to cap (code, length, run, level) entries; returns the number. */
size_t orc_dv_vlc_entries(uint16_t *code, uint8_t *len, uint8_t *run, int16_t *level, size_t cap);

/* Dequantised coefficients and DCT modes of every block of a frame (segment order). */
size_t orc_dv_coefficients(const uint8_t *data, size_t len, int32_t *coef, uint8_t *modes, size_t cap);

/* decoder.rs:520-548 and 555-602 on one block. */
void orc_dv_idct88(const int32_t coefficients[64], uint8_t out[64]);
void orc_dv_idct248(const int32_t coefficients[64], uint8_t out[64]);

/* The libm cos values the DV transforms use: cos(fl(k*PI)/16), k = 0..127. */
double orc_dv_cos(int k);

/* ---- MJPEG encoder side (crates/codecs/mjpeg/src/encoder.rs; encode.c) ---- */

/* Layout and tables of a baseline JPEG written from chosen quantised levels. */
typedef struct orc_jpeg_layout {
    uint32_t width, height;
    uint32_t ncomp;            /* 1..3; component ids 1..ncomp */
    uint8_t h[3], v[3];        /* sampling factors */
    uint8_t tq[3];             /* quantisation table of each component (0 or 1) */
    uint8_t annex_k;           /* 0: the reference encoder's simple Huffman tables; 1: Annex K */
    uint16_t restart_interval; /* MCUs per interval, 0 = no DRI */
    uint8_t qt[2][64];         /* natural order */
} orc_jpeg_layout;

/* transform.rs:111-134 forward_dct_quantize on one block. */
void orc_jpeg_fdct_quantize(const uint8_t samples[64], const uint8_t quantization[64], int32_t out[64]);
void orc_jpeg_fdct_quantize_many(const uint8_t *samples, const uint8_t *quantization, size_t n, int32_t *out);

int orc_jpeg_write_levels(const orc_jpeg_layout *layout, const int32_t *levels, size_t nblocks, uint8_t *out,
                          size_t cap, size_t *len, orc_result *res);

/* encode_jpeg (encoder.rs:44-87) plus the Annex K / restart options. */
int orc_jpeg_encode(const orc_frame *frame, int quality, int annex_k, int restart_interval, uint8_t *out,
                    size_t cap, size_t *len, orc_result *res);

/* Many blocks at once (test volume): n blocks of 64, consecutive. */
void orc_jpeg_idct_many(const int32_t *coefficients, size_t n, uint8_t *out);
void orc_dv_idct88_many(const int32_t *coefficients, size_t n, uint8_t *out);
void orc_dv_idct248_many(const int32_t *coefficients, size_t n, uint8_t *out);

/* transform.rs:2-84, shared by jpeg.c and encode.c */
extern const double ORC_IDCT_MATRIX[8][8];

/* ---- Colour (crates/cli/src/terminal_preview.rs:7159-7236, 7308-7330) ---- */

/* Interleaved RGB24 at 1:1 scale; out holds width*height*3 bytes. */
int orc_rgb24(const orc_frame *frame, uint8_t *out, orc_result *res);

void orc_frame_free(orc_frame *frame);

#ifdef __cplusplus
}
#endif

#endif
