/*
 * MMRecode C ABI, version 1 -- GB300 implementation.
 *
 * This header is ABI-identical to the reference library's public header
 * (crates/capi/include/mmrecode.h): same type layouts, constants and function
 * signatures, so an existing C caller (for example crates/capi/tests/smoke.c)
 * compiles and links against libmmrecode_gpu.so unchanged. The MJPEG and DV
 * decode entry points run on the GPU (sm_103a CUDA kernels); there is no CPU
 * decode path behind them, and they fail with MMR_STATUS_INTERNAL_ERROR when no
 * CUDA device is usable.
 *
 * Conventions (crates/capi/src/lib.rs):
 *  - out_frame / out_buffer must be zero-initialised with struct_size set to
 *    sizeof(*out); a mismatch returns MMR_STATUS_INVALID_ARGUMENT and leaves
 *    the structure untouched (lib.rs:604-610).
 *  - data == NULL with len > 0 returns MMR_STATUS_INVALID_ARGUMENT; len == 0
 *    is an empty input (lib.rs:1129-1150).
 *  - The last diagnostic is thread-local and cleared on success (lib.rs:46-48).
 *  - Planes are library-owned malloc allocations with stride == width; free
 *    them with mmr_video_frame_free, which is NULL-safe and idempotent.
 *  - Calls are reentrant: concurrent callers each use their own GPU decode
 *    engine (a small pool inside the library).
 */
#ifndef MMRECODE_H
#define MMRECODE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32) && defined(MMR_BUILD_SHARED)
#define MMR_API __declspec(dllexport)
#elif defined(_WIN32) && defined(MMR_USE_SHARED)
#define MMR_API __declspec(dllimport)
#elif defined(__GNUC__) && __GNUC__ >= 4
#define MMR_API __attribute__((visibility("default")))
#else
#define MMR_API
#endif

/* mmrecode.h:21-22 */
#define MMR_ABI_VERSION 1u
#define MMR_MAX_PLANES 3u

/* mmrecode.h:24-32 */
typedef int32_t mmr_status;

#define MMR_STATUS_OK ((mmr_status)0)
#define MMR_STATUS_INVALID_ARGUMENT ((mmr_status)1)
#define MMR_STATUS_INVALID_DATA ((mmr_status)2)
#define MMR_STATUS_UNSUPPORTED ((mmr_status)3)
#define MMR_STATUS_INVALID_STATE ((mmr_status)4)
#define MMR_STATUS_IO_ERROR ((mmr_status)5)
#define MMR_STATUS_INTERNAL_ERROR ((mmr_status)100)

/* mmrecode.h:34-40 */
typedef uint32_t mmr_pixel_format;

#define MMR_PIXEL_FORMAT_GRAY8 ((mmr_pixel_format)1u)
#define MMR_PIXEL_FORMAT_YUV420P8 ((mmr_pixel_format)2u)
#define MMR_PIXEL_FORMAT_YUV422P8 ((mmr_pixel_format)3u)
#define MMR_PIXEL_FORMAT_YUV444P8 ((mmr_pixel_format)4u)
#define MMR_PIXEL_FORMAT_YUV411P8 ((mmr_pixel_format)5u)

/* mmrecode.h:42-46 */
typedef uint32_t mmr_color_range;

#define MMR_COLOR_RANGE_UNSPECIFIED ((mmr_color_range)0u)
#define MMR_COLOR_RANGE_FULL ((mmr_color_range)1u)
#define MMR_COLOR_RANGE_LIMITED ((mmr_color_range)2u)

/* mmrecode.h:48-55: a borrowed plane. */
typedef struct mmr_plane_view {
    const uint8_t *data;
    size_t data_len;
    size_t stride;
    size_t width;
    size_t height;
} mmr_plane_view;

/* mmrecode.h:57-66: a borrowed progressive frame (encoder input). */
typedef struct mmr_video_frame_view {
    size_t struct_size;
    mmr_pixel_format format;
    mmr_color_range range;
    size_t width;
    size_t height;
    size_t plane_count;
    mmr_plane_view planes[MMR_MAX_PLANES];
} mmr_video_frame_view;

/* mmrecode.h:68-75: one library-owned plane. */
typedef struct mmr_owned_plane {
    uint8_t *data;
    size_t data_len;
    size_t stride;
    size_t width;
    size_t height;
} mmr_owned_plane;

/* mmrecode.h:77-86: a decoded frame owned by the library. */
typedef struct mmr_video_frame {
    size_t struct_size;
    mmr_pixel_format format;
    mmr_color_range range;
    size_t width;
    size_t height;
    size_t plane_count;
    mmr_owned_plane planes[MMR_MAX_PLANES];
} mmr_video_frame;

/* mmrecode.h:88-93: an encoded byte buffer owned by the library. */
typedef struct mmr_buffer {
    size_t struct_size;
    uint8_t *data;
    size_t len;
} mmr_buffer;

/* mmrecode.h:95-106 (MPEG-2 is outside this library; kept for ABI identity). */
typedef struct mmr_mpeg2_encode_options {
    size_t struct_size;
    uint32_t frame_rate_numerator;
    uint32_t frame_rate_denominator;
    uint32_t gop_size;
    uint32_t b_frames;
    uint32_t quantiser_scale_code;
    uint32_t motion_search_range;
    uint32_t progressive;
    uint32_t top_field_first;
} mmr_mpeg2_encode_options;

/* Replaces mmrecode.h:109 / lib.rs:285: returns MMR_ABI_VERSION. */
MMR_API uint32_t mmr_abi_version(void);

/* Replaces mmrecode.h:112 / lib.rs:291: process-lifetime version string. */
MMR_API const char *mmr_version(void);

/*
 * Replaces mmrecode.h:118 / lib.rs:305: copies the calling thread's last
 * diagnostic (NUL-terminated, truncated to capacity); returns the capacity
 * needed including the NUL. buffer may be NULL for a size query.
 */
MMR_API size_t mmr_last_error_message(char *buffer, size_t capacity);

/*
 * Replaces mmrecode.h:124 / lib.rs:331 (decode_jpeg + into_video_frame).
 * Decodes one complete baseline JPEG on the GPU: marker scan, Huffman decode,
 * dequantisation and the reference's binary64 IDCT reproduced bit for bit.
 * Output is planar YCbCr or Gray8 at native sampling, full range.
 */
MMR_API mmr_status mmr_mjpeg_decode(const uint8_t *data, size_t len, mmr_video_frame *out_frame);

/*
 * Replaces mmrecode.h:130 / lib.rs:350 (parse_frame + decode_video).
 * Decodes one 120000-byte (525/60) or 144000-byte (625/50) DV25 frame on the
 * GPU. Output is planar 4:1:1 or 4:2:0, limited range.
 */
MMR_API mmr_status mmr_dv_decode(const uint8_t *data, size_t len, mmr_video_frame *out_frame);

/* mmrecode.h:136 / lib.rs:367: outside this library; returns MMR_STATUS_UNSUPPORTED. */
MMR_API mmr_status mmr_mpeg2_picture_count(const uint8_t *data, size_t len, size_t *out_count);

/* mmrecode.h:145 / lib.rs:385: outside this library; returns MMR_STATUS_UNSUPPORTED. */
MMR_API mmr_status mmr_mpeg2_decode_picture(const uint8_t *data, size_t len, size_t presentation_index,
                                            mmr_video_frame *out_frame);

/* Replaces mmrecode.h:152 / lib.rs:406: NULL-safe, idempotent; resets the struct. */
MMR_API void mmr_video_frame_free(mmr_video_frame *frame);

/*
 * Replaces mmrecode.h:159 / lib.rs:427 (encode_jpeg, crates/codecs/mjpeg/src/encoder.rs:44-87).
 * CPU encoder, byte-identical to the reference: scaled Annex K quantisation,
 * the reference's fixed "simple" Huffman tables, no restart markers.
 */
MMR_API mmr_status mmr_mjpeg_encode(const mmr_video_frame_view *frame, uint8_t quality, mmr_buffer *out_buffer);

/*
 * Replaces mmrecode.h:165 / lib.rs:446 (encode_video, crates/codecs/dv/src/encoder.rs:67-103).
 * CPU encoder, byte-identical to the reference (8-8 DCT mode only).
 */
MMR_API mmr_status mmr_dv_encode(const mmr_video_frame_view *frame, mmr_buffer *out_buffer);

/* mmrecode.h:173 / lib.rs:465: outside this library; returns MMR_STATUS_UNSUPPORTED. */
MMR_API mmr_status mmr_mpeg2_encode(const mmr_video_frame_view *frames, size_t frame_count,
                                    const mmr_mpeg2_encode_options *options, mmr_buffer *out_buffer);

/* mmrecode.h:180 / lib.rs:484: outside this library; returns MMR_STATUS_UNSUPPORTED. */
MMR_API mmr_status mmr_mpegts_mux_mpeg2(const uint8_t *data, size_t len, mmr_buffer *out_buffer);

/* mmrecode.h:186 / lib.rs:502: outside this library; returns MMR_STATUS_UNSUPPORTED. */
MMR_API mmr_status mmr_mpegts_mux_mpeg2_mp2(const uint8_t *video_data, size_t video_len, const uint8_t *audio_data,
                                            size_t audio_len, mmr_buffer *out_buffer);

/* mmrecode.h:194 / lib.rs:522: outside this library; returns MMR_STATUS_UNSUPPORTED. */
MMR_API mmr_status mmr_mpegts_demux_mpeg2(const uint8_t *data, size_t len, mmr_buffer *out_buffer);

/* mmrecode.h:200 / lib.rs:540: outside this library; returns MMR_STATUS_UNSUPPORTED. */
MMR_API mmr_status mmr_mpegts_demux_mp2(const uint8_t *data, size_t len, mmr_buffer *out_buffer);

/* Replaces mmrecode.h:206 / lib.rs:559: NULL-safe, idempotent; resets the struct. */
MMR_API void mmr_buffer_free(mmr_buffer *buffer);

#ifdef __cplusplus
}
#endif

#endif
