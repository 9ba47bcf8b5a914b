/*
 * Oracle restatement of the reference's integer YCbCr -> RGB24 conversion.
 * TEST INFRASTRUCTURE ONLY (see oracle.h).
 *
 * Follows crates/cli/src/terminal_preview.rs:7159-7236 (video_frame_image) at
 * 1:1 scale -- bounds equal to the frame, so fitted_dimensions (:7238-7256)
 * returns the frame size and source_x[x] = x, source_y[y] = y -- and
 * :7308-7330 (ycbcr_to_rgb) for both colour ranges.
 */
#include <string.h>

#include "oracle.h"

static uint8_t clamp_u8(int32_t v) { return (uint8_t)(v < 0 ? 0 : v > 255 ? 255 : v); }

/* terminal_preview.rs:7308-7330 */
static void ycbcr_to_rgb(uint8_t y8, uint8_t cb8, uint8_t cr8, uint32_t range, uint8_t out[3]) {
    int32_t cb = (int32_t)cb8 - 128;
    int32_t cr = (int32_t)cr8 - 128;
    int32_t r, g, b;
    if (range == ORC_RANGE_LIMITED) {
        int32_t y = (int32_t)y8 - 16;
        if (y < 0) y = 0;
        r = (298 * y + 409 * cr + 128) >> 8;
        g = (298 * y - 100 * cb - 208 * cr + 128) >> 8;
        b = (298 * y + 516 * cb + 128) >> 8;
    } else {
        int32_t y = y8;
        r = y + ((359 * cr + 128) >> 8);
        g = y - ((88 * cb + 183 * cr + 128) >> 8);
        b = y + ((454 * cb + 128) >> 8);
    }
    out[0] = clamp_u8(r);
    out[1] = clamp_u8(g);
    out[2] = clamp_u8(b);
}

/* terminal_preview.rs:7159-7236 with width = frame.width, height = frame.height */
int orc_rgb24(const orc_frame *f, uint8_t *out, orc_result *res) {
    res->status = ORC_OK;
    res->message[0] = 0;
    size_t W = f->width, H = f->height;
    if (f->format == ORC_FMT_GRAY8) {
        const orc_plane *p = &f->planes[0];
        for (size_t y = 0; y < H; y++)
            for (size_t x = 0; x < W; x++) memset(out + (y * W + x) * 3, p->data[y * p->width + x], 3);
        return ORC_OK;
    }
    const orc_plane *luma = &f->planes[0], *bc = &f->planes[1], *rc = &f->planes[2];
    for (size_t y = 0; y < H; y++) {
        size_t ly = y * luma->height / H;
        if (ly > luma->height - 1) ly = luma->height - 1;
        size_t by = y * bc->height / H;
        if (by > bc->height - 1) by = bc->height - 1;
        size_t ry = y * rc->height / H;
        if (ry > rc->height - 1) ry = rc->height - 1;
        for (size_t x = 0; x < W; x++) {
            size_t bx = x * bc->width / W;
            if (bx > bc->width - 1) bx = bc->width - 1;
            size_t rx = x * rc->width / W;
            if (rx > rc->width - 1) rx = rc->width - 1;
            ycbcr_to_rgb(luma->data[ly * luma->width + x], bc->data[by * bc->width + bx],
                         rc->data[ry * rc->width + rx], f->range, out + (y * W + x) * 3);
        }
    }
    return ORC_OK;
}
