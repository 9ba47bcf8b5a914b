/*
 * C caller of the v1 ABI (include/mmrecode.h): decodes an MJPEG or DV file,
 * re-encodes MJPEG output, and prints the frame geometry plus an FNV-1a hash
 * of each plane so a test can compare it with the oracle's planes.
 *
 * usage: smoke_decode mjpeg|dv <file>
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mmrecode.h"

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

int main(int argc, char **argv) {
    if (argc != 3) {
        fprintf(stderr, "usage: %s mjpeg|dv <file>\n", argv[0]);
        return 2;
    }
    if (mmr_abi_version() != MMR_ABI_VERSION || strlen(mmr_version()) == 0) return 3;
    size_t len = 0;
    uint8_t *data = read_file(argv[2], &len);
    if (!data) return 4;
    mmr_video_frame frame;
    memset(&frame, 0, sizeof(frame));
    frame.struct_size = sizeof(frame);
    int dv = strcmp(argv[1], "dv") == 0;
    mmr_status st = dv ? mmr_dv_decode(data, len, &frame) : mmr_mjpeg_decode(data, len, &frame);
    free(data);
    if (st != MMR_STATUS_OK) {
        char msg[512];
        mmr_last_error_message(msg, sizeof(msg));
        printf("status %d %s\n", st, msg);
        return 0;
    }
    printf("format %u range %u %zux%zu planes %zu\n", frame.format, frame.range, frame.width, frame.height,
           frame.plane_count);
    for (size_t i = 0; i < frame.plane_count; i++)
        printf("plane %zu %zux%zu %016llx\n", i, frame.planes[i].width, frame.planes[i].height,
               (unsigned long long)fnv1a(frame.planes[i].data, frame.planes[i].data_len));
    if (!dv) {
        mmr_video_frame_view view;
        memset(&view, 0, sizeof(view));
        view.struct_size = sizeof(view);
        view.format = frame.format;
        view.range = frame.range;
        view.width = frame.width;
        view.height = frame.height;
        view.plane_count = frame.plane_count;
        for (size_t i = 0; i < frame.plane_count; i++) {
            view.planes[i].data = frame.planes[i].data;
            view.planes[i].data_len = frame.planes[i].data_len;
            view.planes[i].stride = frame.planes[i].stride;
            view.planes[i].width = frame.planes[i].width;
            view.planes[i].height = frame.planes[i].height;
        }
        mmr_buffer out;
        memset(&out, 0, sizeof(out));
        out.struct_size = sizeof(out);
        st = mmr_mjpeg_encode(&view, 75, &out);
        if (st != MMR_STATUS_OK || out.len < 4 || out.data[0] != 0xff || out.data[1] != 0xd8) return 6;
        printf("encoded %zu bytes\n", out.len);
        mmr_buffer_free(&out);
    }
    mmr_video_frame_free(&frame);
    mmr_video_frame_free(&frame);
    return 0;
}
