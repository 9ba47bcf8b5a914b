"""Seeded synthetic MJPEG input made without the product library.

TEST INFRASTRUCTURE ONLY: the benchmark's reference arm and the tests build
their input here, so that timing the reference's algorithm never loads the
product's shared library. The content is the workload's (per frame, seeded by
(workload seed, frame index) through numpy's PCG64: a diagonal gradient per
plane, 20 axis-aligned rectangles of uniform random colour, Gaussian noise
sigma 8, clamped to 0..255) and the encoder is the oracle's restatement of the
reference encoder (oracle/encode.c) with Annex K tables and restart markers.
A test checks that these packets equal the product generator's byte for byte.
"""

from __future__ import annotations

import numpy as np

from . import FMT_YUV420P8, FMT_YUV422P8, FMT_YUV444P8, jpeg_encode

SUBSAMPLING = {"420": (FMT_YUV420P8, 2, 2), "422": (FMT_YUV422P8, 2, 1), "444": (FMT_YUV444P8, 1, 1)}


def planes(rng, w, h, cw, ch, sigma, n_rect):
    """Gradient + rectangles + clamped Gaussian noise for the three planes."""
    dims = ((w, h), (cw, ch), (cw, ch))
    base_planes = []
    for p, (pw, ph) in enumerate(dims):
        yy, xx = np.mgrid[0:ph, 0:pw].astype(np.float64)
        a, b = rng.uniform(0.2, 1.0, 2)
        phase = rng.uniform(0, 255)
        base = (a * xx / max(pw, 1) + b * yy / max(ph, 1)) * 200.0 / (a + b) + phase * 0.2
        if p:
            base = 128.0 + (base - 100.0) * 0.5
        base_planes.append(base)
    colours = rng.uniform(16, 240, (max(n_rect, 1), 3))
    for k in range(n_rect):
        x0, y0 = rng.uniform(0, 0.9, 2)
        rw, rh = rng.uniform(0.05, 0.4, 2)
        for p, (pw, ph) in enumerate(dims):
            xa, xb = int(x0 * pw), int(min(1.0, x0 + rw) * pw)
            ya, yb = int(y0 * ph), int(min(1.0, y0 + rh) * ph)
            base_planes[p][ya:yb, xa:xb] = colours[k][p]
    out = []
    for p in range(3):
        noisy = base_planes[p] + rng.normal(0.0, sigma, base_planes[p].shape)
        out.append(np.clip(np.rint(noisy), 0, 255).astype(np.uint8))
    return out


def mjpeg_packet(seed: int, index: int, w: int, h: int, sub: str, quality: int, restart_interval: int,
                 annex_k: bool = True) -> bytes:
    fmt, sx, sy = SUBSAMPLING[sub]
    cw, ch = (w + sx - 1) // sx, (h + sy - 1) // sy
    rng = np.random.Generator(np.random.PCG64([seed, index]))
    y, cb, cr = planes(rng, w, h, cw, ch, 8.0, 20)
    return jpeg_encode(fmt, w, h, [(w, h, y.tobytes()), (cw, ch, cb.tobytes()), (cw, ch, cr.tobytes())], quality,
                       annex_k, restart_interval)


def _one(args):
    return mjpeg_packet(*args)


def mjpeg_stream(seed, count, w, h, sub, quality, restart_interval, annex_k=True, pool=None) -> list:
    jobs = [(seed, i, w, h, sub, quality, restart_interval, annex_k) for i in range(count)]
    if pool is None:
        return [_one(j) for j in jobs]
    return pool.map(_one, jobs, chunksize=max(1, count // 64))
