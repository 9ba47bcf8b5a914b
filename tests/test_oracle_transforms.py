"""The oracle's binary64 transforms against a second restatement, written here in numpy
from the reference source with the same operations in the same order (binary64
products and sums, never fused; Rust's round half away from zero), on the adversarial
block sets: bit-exact (the restatements are in tests/restatements.py). Covers the MJPEG inverse DCT (crates/codecs/mjpeg/src/transform.rs:86-109)
and forward DCT + quantisation (:111-134), and the DV 8-8 (crates/codecs/dv/src/decoder.rs:520-548)
and 2-4-8 (:555-602) inverse transforms; the reference's own tests pin none of the
last three beyond single known answers."""
import numpy as np

import adversarial
import oracle
from restatements import dv_idct88, dv_idct248, fdct_quantize, jpeg_idct, rust_round


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
