"""Seeded synthetic streams of the benchmark shapes.

Content (per frame, seeded by (workload seed, frame index) through numpy's
PCG64): a smooth diagonal gradient per plane, axis-aligned rectangles of
uniform random colour (20 for MJPEG; one moving rectangle for DV), and
Gaussian noise (sigma 8 for MJPEG, 6 for DV) clamped to 0..255. Frames are
encoded with the library's CPU encoders (reference-identical MJPEG encoder with
Annex K Huffman tables and restart markers; DV encoder with per-block 8-8/2-4-8
choice). No public dataset is used.
"""

from __future__ import annotations

import concurrent.futures
import os
from dataclasses import dataclass

import numpy as np

from . import (DV_MODE_ACTIVITY, RANGE_FULL, RANGE_LIMITED, YUV411P8, YUV420P8, YUV422P8, YUV444P8, Plane,
               VideoFrame, encode_dv, encode_jpeg)

SUBSAMPLING = {"420": (YUV420P8, 2, 2), "422": (YUV422P8, 2, 1), "444": (YUV444P8, 1, 1)}


def _planes(rng, w, h, cw, ch, sigma, n_rect, moving=None):
    out = []
    for p, (pw, ph) in enumerate(((w, h), (cw, ch), (cw, ch))):
        yy, xx = np.mgrid[0:ph, 0:pw].astype(np.float64)
        a, b = rng.uniform(0.2, 1.0, 2)
        phase = rng.uniform(0, 255)
        base = (a * xx / max(pw, 1) + b * yy / max(ph, 1)) * 200.0 / (a + b) + phase * 0.2
        if p:
            base = 128.0 + (base - 100.0) * 0.5
        out.append(base)
    colours = rng.uniform(16, 240, (max(n_rect, 1), 3))
    rects = []
    for k in range(n_rect):
        x0, y0 = rng.uniform(0, 0.9, 2)
        rw, rh = rng.uniform(0.05, 0.4, 2)
        rects.append((x0, y0, rw, rh, colours[k]))
    if moving is not None:
        rects.append(moving)
    for x0, y0, rw, rh, col in rects:
        for p, (pw, ph) in enumerate(((w, h), (cw, ch), (cw, ch))):
            xa, xb = int(x0 * pw), int(min(1.0, x0 + rw) * pw)
            ya, yb = int(y0 * ph), int(min(1.0, y0 + rh) * ph)
            out[p][ya:yb, xa:xb] = col[p]
    planes = []
    for p, (pw, ph) in enumerate(((w, h), (cw, ch), (cw, ch))):
        noisy = out[p] + rng.normal(0.0, sigma, out[p].shape)
        planes.append(np.clip(np.rint(noisy), 0, 255).astype(np.uint8))
    return planes


def mjpeg_frame(seed: int, index: int, w: int, h: int, sub: str) -> VideoFrame:
    fmt, sx, sy = SUBSAMPLING[sub]
    cw, ch = (w + sx - 1) // sx, (h + sy - 1) // sy
    rng = np.random.Generator(np.random.PCG64([seed, index]))
    y, cb, cr = _planes(rng, w, h, cw, ch, 8.0, 20)
    return VideoFrame(fmt, w, h, [Plane(y.tobytes(), w, w, h), Plane(cb.tobytes(), cw, cw, ch),
                                  Plane(cr.tobytes(), cw, cw, ch)], RANGE_FULL)


def dv_frame(seed: int, index: int, pal: bool = False) -> VideoFrame:
    w, h = 720, (576 if pal else 480)
    cw, ch = (360, 288) if pal else (180, 480)
    rng = np.random.Generator(np.random.PCG64([seed, index]))
    mrng = np.random.Generator(np.random.PCG64([seed, 1 << 30]))
    x0, y0, vx, vy = mrng.uniform(0.1, 0.6), mrng.uniform(0.1, 0.6), mrng.uniform(-0.01, 0.01), mrng.uniform(-0.01, 0.01)
    col = mrng.uniform(16, 240, 3)
    moving = ((x0 + vx * index) % 0.7, (y0 + vy * index) % 0.7, 0.25, 0.25, col)
    y, cb, cr = _planes(rng, w, h, cw, ch, 6.0, 0, moving)
    return VideoFrame(YUV420P8 if pal else YUV411P8, w, h, [Plane(y.tobytes(), w, w, h), Plane(cb.tobytes(), cw, cw, ch),
                                                           Plane(cr.tobytes(), cw, cw, ch)], RANGE_LIMITED)


@dataclass
class Stream:
    codec: int          # CODEC_MJPEG / CODEC_DV
    packets: list       # encoded frames (bytes)
    describe: dict      # workload parameters


def _pool():
    return concurrent.futures.ThreadPoolExecutor(max_workers=min(32, os.cpu_count() or 4))


def mjpeg_stream(seed, count, w, h, sub, quality, restart_interval, annex_k=True) -> list:
    def one(i):
        return encode_jpeg(mjpeg_frame(seed, i, w, h, sub), quality, annex_k, restart_interval)
    with _pool() as ex:
        return list(ex.map(one, range(count)))


def dv_stream(seed, count, pal=False, mode=DV_MODE_ACTIVITY) -> list:
    def one(i):
        return encode_dv(dv_frame(seed, i, pal), mode)
    with _pool() as ex:
        return list(ex.map(one, range(count)))


def mixed_mjpeg_stream(seed, count) -> list:
    """Mixed-size batch: sizes in steps of 16 within 320x240..3840x2160, subsampling,
    quality 50..95 and restart interval in {none, one MCU row, 4 MCUs} drawn per frame."""
    rng = np.random.Generator(np.random.PCG64([seed, 7]))
    params = []
    for i in range(count):
        w = int(rng.integers(320 // 16, 3840 // 16 + 1)) * 16
        h = int(rng.integers(240 // 16, 2160 // 16 + 1)) * 16
        sub = ["420", "422", "444"][int(rng.integers(0, 3))]
        q = int(rng.integers(50, 96))
        _, sx, _ = SUBSAMPLING[sub]
        row = (w + 8 * sx - 1) // (8 * sx)
        ri = [0, row, 4][int(rng.integers(0, 3))]
        params.append((i, w, h, sub, q, ri))

    def one(p):
        i, w, h, sub, q, ri = p
        return encode_jpeg(mjpeg_frame(seed, i, w, h, sub), q, True, ri)
    with _pool() as ex:
        return list(ex.map(one, params)), params
