/*
 * C caller of the decoder session API (include/mmrecode_gpu.h, mmr_gpu_decoder_*),
 * the reference's Decoder trait over the GPU: configures one session, sends every
 * file as a packet tagged with its argument index, flushes, then receives until
 * nothing is queued, printing each frame's plane geometry and FNV-1a hashes (or
 * the packet's status and message) in the order the packets were sent.
 *
 * usage: session_decode mjpeg|dv <file>...
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mmrecode_gpu.h"

static uint8_t *read_file(const char *path, size_t *length) {
    FILE *f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    uint8_t *data = (uint8_t *)malloc(n > 0 ? (size_t)n : 1);
    if (!data || fread(data, 1, (size_t)n, f) != (size_t)n) {
        fclose(f);
        free(data);
        return NULL;
    }
    fclose(f);
    *length = (size_t)n;
    return data;
}

static uint64_t fnv1a(const uint8_t *p, size_t n) {
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < n; i++) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

static void print_error(const char *what, mmr_status st) {
    char msg[512];
    mmr_last_error_message(msg, sizeof(msg));
    printf("%s status %d %s\n", what, st, msg);
}

int main(int argc, char **argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s mjpeg|dv <file>...\n", argv[0]);
        return 2;
    }
    const int dv = strcmp(argv[1], "dv") == 0;
    mmr_gpu_decoder *decoder = NULL;
    mmr_status st = mmr_gpu_decoder_create(dv ? MMR_CODEC_DV : MMR_CODEC_MJPEG, &decoder);
    if (st != MMR_STATUS_OK) {
        print_error("create", st);
        return 3;
    }
    st = mmr_gpu_decoder_configure(decoder, dv ? "video/dv" : "video/mjpeg", "video");
    if (st != MMR_STATUS_OK) {
        print_error("configure", st);
        mmr_gpu_decoder_destroy(decoder);
        return 3;
    }
    for (int i = 2; i < argc; i++) {
        size_t len = 0;
        uint8_t *data = read_file(argv[i], &len);
        if (!data) {
            mmr_gpu_decoder_destroy(decoder);
            return 4;
        }
        st = mmr_gpu_decoder_send_packet(decoder, data, len, (uint64_t)i);
        free(data); /* the session copied the packet */
        if (st != MMR_STATUS_OK) {
            print_error("send", st);
            mmr_gpu_decoder_destroy(decoder);
            return 5;
        }
    }
    st = mmr_gpu_decoder_flush(decoder);
    if (st != MMR_STATUS_OK) {
        print_error("flush", st);
        mmr_gpu_decoder_destroy(decoder);
        return 5;
    }
    for (;;) {
        mmr_video_frame frame;
        memset(&frame, 0, sizeof(frame));
        frame.struct_size = sizeof(frame);
        uint64_t tag = 0;
        int has_frame = 0;
        st = mmr_gpu_decoder_receive_frame(decoder, 0, &frame, &tag, &has_frame);
        if (st != MMR_STATUS_OK) {
            char what[64];
            snprintf(what, sizeof(what), "frame %llu", (unsigned long long)tag);
            print_error(what, st);
            continue;
        }
        if (!has_frame) break;
        printf("frame %llu format %u %zux%zu planes %zu\n", (unsigned long long)tag, frame.format, frame.width,
               frame.height, frame.plane_count);
        for (size_t c = 0; c < frame.plane_count; c++)
            printf("frame %llu plane %zu %zux%zu %016llx\n", (unsigned long long)tag, c, frame.planes[c].width,
                   frame.planes[c].height, (unsigned long long)fnv1a(frame.planes[c].data, frame.planes[c].data_len));
        mmr_video_frame_free(&frame);
    }
    mmr_gpu_decoder_destroy(decoder);
    return 0;
}
