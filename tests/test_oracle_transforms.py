"""The oracle's binary64 transforms against a second restatement, written here in numpy
from the reference source with the same operations in the same order (binary64
products and sums, never fused; Rust's round half away from zero), on the adversarial
block sets: bit-exact. Covers the MJPEG inverse DCT (crates/codecs/mjpeg/src/transform.rs:86-109)
and forward DCT + quantisation (:111-134), and the DV 8-8 (crates/codecs/dv/src/decoder.rs:520-548)
and 2-4-8 (:555-602) inverse transforms; the reference's own tests pin none of the
last three beyond single known answers."""
import math

import numpy as np

import adversarial
import oracle

FRAC = 0.7071067811865476  # std::f64::consts::FRAC_1_SQRT_2


def rust_round(x):
    """f64::round: half away from zero (x - trunc(x) is exact in binary64)."""
    t = np.trunc(x)
    f = x - t
    return t + np.where(np.abs(f) >= 0.5, np.sign(x), 0.0)


def to_u8(x):
    return np.clip(rust_round(x), 0.0, 255.0).astype(np.uint8)


def jpeg_idct(c):
    M = adversarial.idct_matrix()
    c = np.asarray(c, np.float64)
    t = np.zeros((len(c), 64))
    for v in range(8):
        for x in range(8):
            for u in range(8):
                t[:, v * 8 + x] = t[:, v * 8 + x] + M[x, u] * c[:, v * 8 + u]
    out = np.zeros((len(c), 64), np.uint8)
    for y in range(8):
        for x in range(8):
            s = np.zeros(len(c))
            for v in range(8):
                s = s + M[y, v] * t[:, v * 8 + x]
            out[:, y * 8 + x] = to_u8(s + 128.0)
    return out


def fdct_quantize(samples, quant):
    M = adversarial.idct_matrix()
    s = np.asarray(samples, np.float64)
    q = np.asarray(quant, np.float64)
    t = np.zeros((len(s), 64))
    for y in range(8):
        for u in range(8):
            for x in range(8):
                t[:, y * 8 + u] = t[:, y * 8 + u] + M[x, u] * (s[:, y * 8 + x] - 128.0)
    out = np.zeros((len(s), 64), np.int32)
    for v in range(8):
        for u in range(8):
            value = np.zeros(len(s))
            for y in range(8):
                value = value + M[y, v] * t[:, y * 8 + u]
            out[:, v * 8 + u] = rust_round(value / q[:, v * 8 + u]).astype(np.int32)
    return out


def cos16(a, b):
    return math.cos(float(a) * float(b) * math.pi / 16.0)


def cos8(a, b):
    return math.cos(float(a) * float(b) * math.pi / 8.0)


def dv_idct88(c):
    c = np.asarray(c, np.float64)
    out = np.zeros((len(c), 64), np.uint8)
    for y in range(8):
        for x in range(8):
            s = np.zeros(len(c))
            for v in range(8):
                for u in range(8):
                    cu = FRAC if u == 0 else 1.0
                    cv = FRAC if v == 0 else 1.0
                    s = s + cu * cv * c[:, v * 8 + u] * cos16(2 * x + 1, u) * cos16(2 * y + 1, v)
            out[:, y * 8 + x] = to_u8(s / 4.0)
    return out


def dv_idct248(c):
    c = np.asarray(c, np.float64)
    b = np.zeros((len(c), 64))
    for pair in range(4):
        for u in range(8):
            first, second = c[:, pair * 16 + u], c[:, pair * 16 + 8 + u]
            b[:, pair * 16 + u] = first + second
            b[:, pair * 16 + 8 + u] = first - second
    h = np.zeros((len(c), 64))
    for row in range(8):
        for x in range(8):
            s = np.zeros(len(c))
            for u in range(8):
                cu = FRAC if u == 0 else 1.0
                s = s + cu * b[:, row * 8 + u] * cos16(2 * x + 1, u)
            h[:, row * 8 + x] = s / 2.0
    out = np.zeros((len(c), 64), np.uint8)
    for field in range(2):
        for y in range(4):
            for x in range(8):
                s = np.zeros(len(c))
                for v in range(4):
                    cv = FRAC if v == 0 else 1.0
                    s = s + cv * h[:, (v * 2 + field) * 8 + x] * cos8(2 * y + 1, v)
                out[:, (y * 2 + field) * 8 + x] = to_u8(s / 2.0)
    return out


def first_difference(a, b):
    bad = np.argwhere(a != b)
    return None if bad.size == 0 else (tuple(bad[0]), int(a[tuple(bad[0])]), int(b[tuple(bad[0])]))


def test_rust_round_half_away_from_zero():
    x = np.array([0.5, -0.5, 1.5, -1.5, 2.5, 0.49999999999999994, -0.49999999999999994, 254.5, -0.0])
    assert rust_round(x).tolist() == [1.0, -1.0, 2.0, -2.0, 3.0, 0.0, 0.0, 255.0, 0.0]


def test_jpeg_idct_two_restatements_agree():
    c, kinds, near = adversarial.jpeg_idct_blocks(31, dense=20_000)
    assert first_difference(jpeg_idct(c), oracle.jpeg_idct_many(c)) is None
    assert near > 10_000 and len(c) > 100_000


def test_fdct_quantize_two_restatements_agree():
    s, q, kinds, near = adversarial.fdct_blocks(37, n=20_000)
    assert first_difference(fdct_quantize(s, q), oracle.fdct_quantize_many(s, q)) is None
    assert near > 5_000


def test_dv_transforms_two_restatements_agree():
    c, modes, kinds, near = adversarial.dv_idct_blocks(41, n=20_000)
    for mode, ours, theirs in ((0, dv_idct88, oracle.dv_idct88_many), (1, dv_idct248, oracle.dv_idct248_many)):
        sel = c[modes == mode]
        assert first_difference(ours(sel), theirs(sel)) is None, mode
    assert near > 10_000
