/*
 * GB300 batch / context API for the MJPEG and DV25 decode path.
 *
 * Additive to the v1 ABI in mmrecode.h (which it includes); none of these
 * symbols exist in the reference library. The reference decodes one packet per
 * call on one CPU thread (crates/capi/src/lib.rs:331-359, decode_jpeg in
 * crates/codecs/mjpeg/src/decoder.rs:140 and decode_video in
 * crates/codecs/dv/src/decoder.rs:78); this API hands many packets to the GPU
 * at once. Every output sample equals what the reference decoder produces for
 * the same packet; every status equals the reference's status.
 */
#ifndef MMRECODE_GPU_H
#define MMRECODE_GPU_H

#include "mmrecode.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Codec of a packet. */
#define MMR_CODEC_MJPEG 1u
#define MMR_CODEC_DV 2u

/* Output layout of a decoded packet. */
#define MMR_OUTPUT_PLANAR 0u /* native planes, Y | Cb | Cr concatenated, stride == plane width */
#define MMR_OUTPUT_RGB24 1u  /* interleaved RGB at 1:1, integer BT.601 (crates/cli/src/terminal_preview.rs:7159-7330) */

/* Item flags. */
#define MMR_ITEM_CONCEAL 1u      /* DV: fill undecodable segments with black instead of failing
                                    (decode_video_with_options, crates/codecs/dv/src/decoder.rs:87-150) */
#define MMR_ITEM_OUT_DEVICE 2u   /* `out` is device memory */

typedef struct mmr_gpu_context mmr_gpu_context;

typedef struct mmr_gpu_config {
    size_t struct_size;
    int32_t device;   /* CUDA device ordinal */
    uint32_t flags;   /* reserved, 0 */
    uint32_t engines; /* batches decoded concurrently, each on its own CUDA stream with its own
                         device arenas; 0 = 4. A large batch is split over them so that planning,
                         uploads, kernels and read-backs of its parts overlap. */
} mmr_gpu_config;

/* Creates a decode context on a device. */
MMR_API mmr_status mmr_gpu_context_create(const mmr_gpu_config *config, mmr_gpu_context **out_context);

/* Destroys a context; NULL is ignored. */
MMR_API void mmr_gpu_context_destroy(mmr_gpu_context *context);

/* Output geometry of one packet, from its headers only. */
typedef struct mmr_gpu_frame_info {
    size_t struct_size;
    mmr_status status; /* header-level status; decoding can still fail later */
    mmr_pixel_format format;
    mmr_color_range range;
    size_t width, height;
    size_t plane_count;
    size_t plane_width[MMR_MAX_PLANES], plane_height[MMR_MAX_PLANES];
    size_t planar_bytes; /* output size with MMR_OUTPUT_PLANAR */
    size_t rgb_bytes;    /* output size with MMR_OUTPUT_RGB24 */
} mmr_gpu_frame_info;

/* Reads a packet's headers on the host and reports its output geometry. */
MMR_API mmr_status mmr_gpu_probe(uint32_t codec, const uint8_t *data, size_t len, mmr_gpu_frame_info *info);

/* One packet of a batch. */
typedef struct mmr_gpu_item {
    size_t struct_size;
    const uint8_t *data;        /* host copy of the packet (headers are read on the host) */
    const uint8_t *device_data; /* optional device copy of the same bytes; skips the upload */
    size_t len;
    uint32_t codec;
    uint32_t output;
    uint32_t flags;
    uint8_t *out;               /* output buffer (host, or device with MMR_ITEM_OUT_DEVICE) */
    size_t out_capacity;
    /* filled in by the call */
    mmr_status status;
    mmr_pixel_format format;
    mmr_color_range range;
    size_t width, height;
    size_t plane_count;
    size_t plane_offset[MMR_MAX_PLANES], plane_width[MMR_MAX_PLANES], plane_height[MMR_MAX_PLANES];
    size_t out_bytes;
    uint32_t concealed_segments; /* DV with MMR_ITEM_CONCEAL: segments filled with black */
    char message[200];           /* per-item diagnostic, "" on success */
} mmr_gpu_item;

/*
 * Decodes `count` packets in one pass on the context's stream and returns when
 * all are done. Per-item status is in items[i].status; the call itself returns
 * MMR_STATUS_OK unless its arguments are invalid or the device failed.
 */
MMR_API mmr_status mmr_gpu_decode_batch(mmr_gpu_context *context, mmr_gpu_item *items, size_t count);

/* Device time (CUDA events on the context stream) of the last batch, in ms. */
MMR_API double mmr_gpu_last_batch_ms(const mmr_gpu_context *context);

/* Kernel launches of the last batch. */
MMR_API uint32_t mmr_gpu_last_batch_launches(const mmr_gpu_context *context);

/*
 * Bits per slice of the chunked entropy decoder for the following batches: each
 * restart interval (the whole scan without DRI) is cut into slices of this many
 * bits that decode in parallel. Accepted: multiples of 32 in 128..1048576; 0
 * restores the context's automatic choice. Output never depends on it.
 */
MMR_API mmr_status mmr_gpu_set_slice_bits(mmr_gpu_context *context, uint32_t bits);

/* Stage times of the last batch (CUDA events on the context stream) and its sizes. */
typedef struct mmr_gpu_batch_stats {
    size_t struct_size;
    double total_ms, upload_ms, scan_ms, entropy_ms, idct_ms, dv_ms, rgb_ms, download_ms;
    uint64_t input_bytes, output_bytes, jpeg_blocks, dv_blocks, rgb_pixels;
    uint64_t idct_exact_samples; /* samples the fp32 IDCT left to the exact binary64 pass */
    uint32_t launches;
    /* inside entropy_ms: speculative slice decode, slice synchronisation + block prefix, final decode */
    double slice_spec_ms, slice_sync_ms, slice_decode_ms;
    uint32_t graph_replays; /* parts of the batch whose launches replayed a captured CUDA graph */
    /* slices of the chunked entropy decoder, and those whose levels the final decode
       pass redid instead of taking the speculative decode's */
    uint64_t slices, slices_redone;
    /* inside dv_ms: DIF identifier check + segment (VLC) decode, then transform + placement */
    double dv_segment_ms, dv_idct_ms;
    /* of slices_redone, those the final decode redid from their start */
    uint64_t slices_redone_whole;
} mmr_gpu_batch_stats;

/*
 * Autotuner, two tables per context:
 *  - kind 0, entropy classes (restart layout: none / intervals of <= 8 MCUs /
 *    longer; log2 of the compressed bits per interval): decodes up to 64 of the
 *    sample's MJPEG frames of the class at every candidate slice size (1024, 2048,
 *    4096, 8192 bits) and keeps the fastest entropy stage;
 *  - kind 1, tiling classes of the sample's RGB24 MJPEG frames the fused
 *    transform takes ((layout: 0 = 4:4:4, 1 = 4:2:2, 2 = 4:2:0) << 8 | bit length
 *    of the MCU columns): decodes up to 64 of them with the narrow and the wide
 *    strip of MCUs per CTA (8 or 16 at 4:4:4, 4 or 8 otherwise) and keeps the
 *    fastest transform stage.
 * Later batches of this context use the tables (other classes keep the default:
 * automatic slice size, wide strip). The items are decoded (outputs written)
 * several times. report (capacity entries, may be NULL) receives one entry per
 * class; *count the number of classes. mmr_gpu_set_tuning installs a table
 * saved from an earlier run (only frame_class, kind, slice_bits and strip_mcus
 * are read).
 */
typedef struct mmr_gpu_tune_entry {
    uint32_t frame_class; /* kind 0: (layout << 8) | log2(bits per interval); kind 1: tiling class */
    uint32_t slice_bits;  /* kind 0: chosen */
    uint32_t frames;      /* sample frames of the class */
    uint32_t kind;        /* 0: entropy slice size, 1: transform strip */
    double entropy_ms[4]; /* kind 0, per candidate: 1024, 2048, 4096, 8192 bits */
    uint32_t strip_mcus;  /* kind 1: chosen MCUs per transform CTA */
    uint32_t pad;
    double transform_ms[2]; /* kind 1: narrow strip, wide strip */
} mmr_gpu_tune_entry;

MMR_API mmr_status mmr_gpu_autotune(mmr_gpu_context *context, mmr_gpu_item *items, size_t count,
                                    mmr_gpu_tune_entry *report, size_t capacity, size_t *report_count);
MMR_API mmr_status mmr_gpu_set_tuning(mmr_gpu_context *context, const mmr_gpu_tune_entry *entries, size_t count);

/*
 * CUDA-graph replay (default on): a batch whose packets stay on the device and
 * whose plan, buffers and pointers equal one of an engine's recent batches is
 * captured on its second occurrence and replayed as one graph launch afterwards.
 */
MMR_API mmr_status mmr_gpu_set_graphs(mmr_gpu_context *context, int enable);

MMR_API mmr_status mmr_gpu_last_batch_stats(const mmr_gpu_context *context, mmr_gpu_batch_stats *stats);

/* Stream generation: the reference encoders plus the options the decode benchmarks need. */
typedef struct mmr_jpeg_encode_options {
    size_t struct_size;
    uint8_t quality;           /* 1..100 */
    uint8_t annex_k_huffman;   /* 1: ITU-T T.81 Annex K.3 tables (luma/chroma); 0: the reference's tables */
    uint16_t restart_interval; /* MCUs per restart interval, 0 = none */
} mmr_jpeg_encode_options;

/* mmr_mjpeg_encode (crates/codecs/mjpeg/src/encoder.rs:44-87) with Annex K Huffman and DRI options. */
MMR_API mmr_status mmr_mjpeg_encode_ex(const mmr_video_frame_view *frame, const mmr_jpeg_encode_options *options,
                                       mmr_buffer *out_buffer);

/*
 * Batch JPEG encode on the GPU: the forward DCT, quantisation and Huffman coding
 * of encode_jpeg (crates/codecs/mjpeg/src/encoder.rs:44-87, 341-545) for many
 * frames per pass, every output byte equal to mmr_mjpeg_encode_ex's with the same
 * options (mmr_mjpeg_encode's with quality only). No counterpart in the reference
 * library.
 */
#define MMR_ITEM_IN_DEVICE 4u /* encode: the frame's plane data is device memory */

typedef struct mmr_gpu_encode_item {
    size_t struct_size;
    mmr_video_frame_view frame; /* planar input (host memory, or device with MMR_ITEM_IN_DEVICE) */
    uint32_t flags;             /* MMR_ITEM_IN_DEVICE, MMR_ITEM_OUT_DEVICE */
    uint8_t *out;               /* the JPEG bytes (host, or device with MMR_ITEM_OUT_DEVICE) */
    size_t out_capacity;        /* mmr_gpu_jpeg_encode_bound() always suffices */
    /* filled in by the call */
    mmr_status status;
    size_t out_len;
    char message[200];          /* per-item diagnostic, "" on success */
} mmr_gpu_encode_item;

/* An output capacity that holds any encoded frame of this format and size. */
MMR_API size_t mmr_gpu_jpeg_encode_bound(mmr_pixel_format format, size_t width, size_t height,
                                         uint16_t restart_interval);

/*
 * Encodes `count` frames with one set of options in one pass on the context's
 * device. Per-item status in items[i].status; the call returns MMR_STATUS_OK
 * unless its arguments are invalid or the device failed.
 */
MMR_API mmr_status mmr_gpu_jpeg_encode_batch(mmr_gpu_context *context, const mmr_jpeg_encode_options *options,
                                             mmr_gpu_encode_item *items, size_t count);

typedef struct mmr_gpu_encode_stats {
    size_t struct_size;
    double device_ms;            /* uploads, kernels and downloads of the last encode batch */
    uint64_t blocks;             /* 8x8 blocks transformed */
    uint64_t exact_coefficients; /* quotients the fp32 transform left to the binary64 recomputation */
    uint64_t bytes_out;          /* JPEG bytes produced */
} mmr_gpu_encode_stats;

MMR_API mmr_status mmr_gpu_last_encode_stats(const mmr_gpu_context *context, mmr_gpu_encode_stats *stats);

#define MMR_DV_MODE_88 0u       /* every block 8-8 (the reference encoder) */
#define MMR_DV_MODE_ACTIVITY 1u /* 2-4-8 where inter-field activity exceeds intra-field activity */

/* mmr_dv_encode (crates/codecs/dv/src/encoder.rs:67-103) with a DCT-mode policy. */
MMR_API mmr_status mmr_dv_encode_ex(const mmr_video_frame_view *frame, uint32_t mode_policy, mmr_buffer *out_buffer);

/*
 * DV25 decode that allocates nothing. No counterpart in the reference library.
 *
 * For callers that must not allocate memory while decoding: a real-time capture
 * or playback thread that cannot take cudaMalloc's implicit device
 * synchronisation, an application whose GPU memory is budgeted up front, or a
 * host runtime that forbids allocations outside its own arena. The packet
 * (120000 or 144000 bytes) and the output buffer (planar Y | Cb | Cr, at least
 * info->planar_bytes after the call; 622080 bytes covers both systems) are the
 * caller's host memory; all device work uses one fixed 2.25 MiB array inside
 * the library, which every GPU that loads the library keeps until the process
 * exits. Packets longer than 144000 bytes are rejected with
 * MMR_STATUS_INVALID_ARGUMENT. Results equal mmr_dv_decode's for the same
 * packet. On success the call performs no allocation at all; a failing call
 * stores its diagnostic for mmr_last_error_message like every other entry point.
 *
 * The first call on a device sets that device up (it looks up the array's
 * device address and writes a lookup table into it), so make that first call
 * before any stream capture. All calls share the array: calls that overlap on
 * the GPU (several threads decoding on the same device) race, so serialise them.
 * The work runs on the calling thread's per-thread default stream
 * (cudaStreamPerThread), so it does not wait for, or hold back, the
 * application's other streams; the call returns when its output is in `out`.
 * After a device reset (cudaDeviceReset) the next call notices that the lookup
 * table is gone and sets the device up again.
 * info->struct_size must be sizeof(mmr_gpu_frame_info); the call fills *info.
 */
MMR_API mmr_status mmr_dv_decode_static(const uint8_t *data, size_t len, uint8_t *out, size_t out_capacity,
                                        mmr_gpu_frame_info *info);

/*
 * Serving: requests from many streams, admitted against a device-memory budget
 * and batched continuously. No counterpart in the reference library (whose
 * decoders run one packet per call on the calling thread).
 *
 * Each engine takes the oldest queued requests that fit its share of the
 * budget (memory_budget / engines, estimated from the packet headers) and at
 * most max_batch of them, decodes them as one batch and takes the next ones, so
 * requests arriving while others are on the GPU join the next free batch.
 * A request whose estimate alone exceeds an engine's share is refused with
 * MMR_STATUS_INVALID_ARGUMENT.
 */
typedef struct mmr_gpu_server mmr_gpu_server;

typedef struct mmr_gpu_server_config {
    size_t struct_size;
    int32_t device;
    uint32_t engines;       /* batches in flight; 0 = 3 */
    uint32_t max_batch;     /* packets per batch; 0 = 64 */
    uint32_t pad;
    uint64_t memory_budget; /* device bytes for all batches in flight; 0 = no cap */
} mmr_gpu_server_config;

typedef struct mmr_gpu_server_stats {
    size_t struct_size;
    uint64_t submitted, completed, failed, rejected, batches, in_flight, queued;
    double p50_ms, p99_ms, max_ms, mean_ms; /* submit -> completion, requests completed in the window */
    double frames_per_s, window_s;          /* completions over the window (since creation or reset) */
    uint64_t peak_budget_bytes;             /* largest estimated footprint of the batches in flight */
} mmr_gpu_server_stats;

MMR_API mmr_status mmr_gpu_server_create(const mmr_gpu_server_config *config, mmr_gpu_server **out_server);

/* Completes every submitted request, then destroys the server; NULL is ignored. */
MMR_API void mmr_gpu_server_destroy(mmr_gpu_server *server);

/*
 * Queues one packet and returns at once with a ticket. The item's fields are
 * read now (data, len, codec, output, flags, out, out_capacity, as for
 * mmr_gpu_decode_batch); the packet bytes and the output buffer must stay valid
 * until mmr_gpu_server_wait has returned the ticket.
 */
MMR_API mmr_status mmr_gpu_server_submit(mmr_gpu_server *server, const mmr_gpu_item *item, uint64_t *ticket);

/*
 * Waits for a ticket (timeout_ns < 0: without limit). On completion fills the
 * result fields of *result (status, format, ..., message; its struct_size must
 * be set) and *latency_ms (submit to completion), forgets the ticket and returns
 * MMR_STATUS_OK; on timeout returns MMR_STATUS_INVALID_STATE and the ticket stays
 * valid. Unknown tickets are MMR_STATUS_INVALID_ARGUMENT.
 */
MMR_API mmr_status mmr_gpu_server_wait(mmr_gpu_server *server, uint64_t ticket, int64_t timeout_ns,
                                       mmr_gpu_item *result, double *latency_ms);

/* Counters and latency percentiles of the window (since creation or the last reset);
   reset != 0 starts a new window after reading this one. */
MMR_API mmr_status mmr_gpu_server_stats_get(mmr_gpu_server *server, int reset, mmr_gpu_server_stats *stats);

/*
 * Open-loop load replay: submits items[i] arrival_ns[i] nanoseconds after the
 * call starts (offsets non-decreasing) from a native thread, and returns when
 * every item has completed, with its result in items[i], its submit-to-completion
 * latency in latency_ms[i] and the largest delay of a submission past its
 * arrival time in *max_lag_ns (NULL allowed).
 */
MMR_API mmr_status mmr_gpu_server_replay(mmr_gpu_server *server, mmr_gpu_item *items, size_t count,
                                         const int64_t *arrival_ns, double *latency_ms, int64_t *max_lag_ns);

/* mmr_gpu_set_slice_bits for a server's engines. */
MMR_API mmr_status mmr_gpu_server_set_slice_bits(mmr_gpu_server *server, uint32_t bits);
/* mmr_gpu_set_tuning for a server's engines (batches formed after the call use it). */
MMR_API mmr_status mmr_gpu_server_set_tuning(mmr_gpu_server *server, const mmr_gpu_tune_entry *entries,
                                             size_t count);

/*
 * Decoder sessions: the reference's Decoder trait (crates/core/src/codec.rs:102-130)
 * as MjpegDecoder (crates/codecs/mjpeg/src/codec.rs:16-71) and DvDecoder
 * (crates/codecs/dv/src/codec.rs:16-66) implement it, decoding on the GPU. A sent
 * packet is copied and queued at once on a continuous-batching server that all
 * sessions of the process share (created with the first packet, on device 0), so
 * packets of many sessions decode in the same batches; each session receives its
 * frames in the order it sent the packets.
 *
 * States and messages are the reference's: send_packet, receive_frame and flush
 * fail with MMR_STATUS_INVALID_STATE until configure has succeeded, and configure
 * checks the descriptor. One difference: the reference's send_packet decodes
 * before it returns, so a decode error comes back from send_packet; here it comes
 * back, with the same status and message, from the receive_frame call that reaches
 * that packet. Calls on one session must not overlap; different sessions may be
 * used from different threads.
 */
typedef struct mmr_gpu_decoder mmr_gpu_decoder;

/* A session for MMR_CODEC_MJPEG or MMR_CODEC_DV; it starts unconfigured. */
MMR_API mmr_status mmr_gpu_decoder_create(uint32_t codec, mmr_gpu_decoder **out_decoder);

/* Waits for the session's packets still being decoded, frees its queued frames and
   the session; NULL is ignored. */
MMR_API void mmr_gpu_decoder_destroy(mmr_gpu_decoder *decoder);

/* configure: codec_id must be the session's ("video/mjpeg" or "video/dv") and
   media_type "video", else MMR_STATUS_INVALID_DATA with the reference's message.
   Discards the queued frames. */
MMR_API mmr_status mmr_gpu_decoder_configure(mmr_gpu_decoder *decoder, const char *codec_id,
                                             const char *media_type);

/* send_packet: copies the packet, queues it for decode and returns. user_tag comes
   back with the packet's frame (the reference carries the packet's pts and duration
   into the frame's timing; a caller keeps them by tag). */
MMR_API mmr_status mmr_gpu_decoder_send_packet(mmr_gpu_decoder *decoder, const uint8_t *data, size_t len,
                                               uint64_t user_tag);

/*
 * receive_frame: the frame of the oldest queued packet, waiting up to wait_ns for it
 * (< 0: without limit; 0: only if it is done). *out_frame is initialised by the
 * caller as for mmr_mjpeg_decode and freed with mmr_video_frame_free.
 * *out_has_frame = 1: the frame is in *out_frame and the packet's tag in
 * *out_user_tag (NULL allowed). *out_has_frame = 0 with MMR_STATUS_OK: nothing is
 * queued, or the oldest packet is not done within wait_ns (the reference's Ok(None)).
 * A packet that failed to decode leaves the queue here: the call returns its status
 * and message, the frame stays empty and *out_user_tag is set.
 */
MMR_API mmr_status mmr_gpu_decoder_receive_frame(mmr_gpu_decoder *decoder, int64_t wait_ns,
                                                 mmr_video_frame *out_frame, uint64_t *out_user_tag,
                                                 int *out_has_frame);

/* flush: end of input. Returns when every queued packet is decoded, so that
   receive_frame with wait_ns 0 then drains the session. */
MMR_API mmr_status mmr_gpu_decoder_flush(mmr_gpu_decoder *decoder);

/*
 * Where a session delivers its frames: MMR_SESSION_HOST_FRAMES (the default;
 * receive_frame) or MMR_SESSION_DEVICE_FRAMES (receive_device_frame: the planes stay
 * in device memory of device 0, nothing is downloaded). Changes only while no packet
 * is queued (else MMR_STATUS_INVALID_STATE); receiving with the other call is
 * MMR_STATUS_INVALID_STATE.
 */
#define MMR_SESSION_HOST_FRAMES 0u
#define MMR_SESSION_DEVICE_FRAMES 1u
MMR_API mmr_status mmr_gpu_decoder_set_output(mmr_gpu_decoder *decoder, uint32_t where);

/* A decoded frame in device memory. The planes are one library-owned buffer,
   valid until mmr_gpu_device_frame_release; each plane's stride is its width. */
typedef struct mmr_gpu_device_frame {
    size_t struct_size;
    mmr_pixel_format format;
    mmr_color_range range;
    size_t width, height;
    size_t plane_count;
    const uint8_t *planes[MMR_MAX_PLANES]; /* device pointers */
    size_t plane_width[MMR_MAX_PLANES], plane_height[MMR_MAX_PLANES];
    void *buffer;        /* the library's: handed back by the release call */
    size_t buffer_bytes;
} mmr_gpu_device_frame;

/* receive_frame for a session set to MMR_SESSION_DEVICE_FRAMES; the same waiting,
   tag and error rules. *out_frame needs its struct_size set and is reset by the call. */
MMR_API mmr_status mmr_gpu_decoder_receive_device_frame(mmr_gpu_decoder *decoder, int64_t wait_ns,
                                                        mmr_gpu_device_frame *out_frame, uint64_t *out_user_tag,
                                                        int *out_has_frame);

/* Gives a device frame's buffer back to the library (reused by later frames) and
   resets the frame to empty; NULL, empty frames and frames of another struct_size are
   ignored. The work reading the frame on the device must be complete (synchronise the
   streams that read it first). */
MMR_API void mmr_gpu_device_frame_release(mmr_gpu_device_frame *frame);

/*
 * Whole-stream decode to Y4M: the reference CLI's `mmrecode decode <in> <out>`
 * for MJPEG and raw DV input (crates/cli/src/main.rs:1533-1580, 1605-1633), with
 * the stream uploaded once and framed on the GPU, every frame decoded in one
 * batch from device memory, and the Y4M bytes its Y4mWriter would write
 * (crates/containers/y4m/src/lib.rs:219-300) laid out in the caller's buffer.
 * The reference CLI reads the file itself; these calls take its bytes.
 */
#define MMR_STREAM_NONE 0u   /* empty input: "input contains no media frames" */
#define MMR_STREAM_MJPEG 1u  /* concatenated JFIF images, each ending after its EOI */
#define MMR_STREAM_DV 2u     /* raw DV frames, profile from the first DIF block */
#define MMR_STREAM_MPEGTS 3u /* MPEG transport stream: outside this library */
#define MMR_STREAM_MPEG2 4u  /* MPEG-2 video elementary stream: outside this library */

typedef struct mmr_gpu_stream mmr_gpu_stream;

typedef struct mmr_gpu_stream_info {
    size_t struct_size;
    uint32_t kind;           /* MMR_STREAM_*, detected in the CLI's order (main.rs:1536-1553, 1908-1921) */
    mmr_status frame_status; /* MMR_STATUS_OK, or the error that ends the framing after frame_count frames
                                (a parse_jpeg error of the next image, an incomplete raw DV frame, ...) */
    size_t frame_count;      /* frames framed before frame_status's error */
    size_t y4m_bytes;        /* capacity mmr_gpu_stream_decode_y4m needs */
    uint64_t candidates;     /* marker candidates the device scan found (MJPEG) */
    double upload_ms;        /* device time of the stream's upload */
    double scan_ms;          /* device time of the marker-candidate scan (MJPEG) */
    char message[512];       /* frame_status's message as the CLI prints it, "" when OK */
} mmr_gpu_stream_info;

/*
 * Uploads the stream and frames it. `data` must stay valid until the stream is
 * closed, and the context must outlive the stream. `input_name` is the name the
 * CLI would print in "'<input>' ends with an incomplete raw DV frame" (NULL:
 * "input"). Returns MMR_STATUS_OK with a stream also when framing stops at an
 * error (reported in *info); other statuses leave *out_stream NULL.
 */
MMR_API mmr_status mmr_gpu_stream_open(mmr_gpu_context *context, const uint8_t *data, size_t len,
                                       const char *input_name, mmr_gpu_stream **out_stream,
                                       mmr_gpu_stream_info *info);

/* Offset and length in the stream of framed frame `index`. */
MMR_API mmr_status mmr_gpu_stream_frame(const mmr_gpu_stream *stream, size_t index, uint64_t *offset,
                                        uint64_t *length);

typedef struct mmr_gpu_stream_result {
    size_t struct_size;
    mmr_status status;     /* the CLI's first error (a frame that fails to decode, one the Y4M writer
                              rejects, then the framing error), MMR_STATUS_OK if none */
    size_t frames_written; /* frames in the Y4M bytes */
    size_t bytes_written;  /* Y4M bytes at the start of `out`: what the CLI's output file holds */
    char message[512];     /* status's message as the CLI prints it, "" when OK */
} mmr_gpu_stream_result;

/*
 * Decodes every framed frame and writes the Y4M stream to out[0, capacity)
 * (capacity >= info.y4m_bytes; bytes past result->bytes_written are scratch).
 * Returns MMR_STATUS_OK unless an argument is invalid or the device failed;
 * the stream's own outcome is in *result.
 */
MMR_API mmr_status mmr_gpu_stream_decode_y4m(mmr_gpu_stream *stream, uint8_t *out, size_t capacity,
                                             mmr_gpu_stream_result *result);

/* Frees a stream and its device copy; NULL is ignored. */
MMR_API void mmr_gpu_stream_close(mmr_gpu_stream *stream);

#ifdef __cplusplus
}
#endif

#endif
