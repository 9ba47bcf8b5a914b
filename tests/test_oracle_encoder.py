"""The oracle's encoder restatement (oracle/encode.c) and its input generator.

The benchmark's reference arm builds its workload with these so that it never
loads the product library; the adversarial transform tests write their crafted
streams with the coefficient-level writer. Pins: the reference's golden stream
(crates/codecs/mjpeg/src/encoder.rs:621-630), its forward-DCT known answers,
and byte equality with the product's own encoder on every benchmark shape."""

import numpy as np
import pytest

import mmrecode_gb300 as m
import oracle
import oracle.synth as osynth
from mmrecode_gb300 import synth
from helpers import fixture, read_y4m_420


def _frames():
    return read_y4m_420(fixture("y4m/valid/two-frame-420.y4m"))


# encoder.rs:621-630 encoded_output_is_deterministic: two-frame-420.y4m at q85
def test_oracle_encoder_reproduces_the_golden_stream():
    out = b""
    for w, h, y, cb, cr in _frames():
        cw, ch = (w + 1) // 2, (h + 1) // 2
        out += oracle.jpeg_encode(oracle.FMT_YUV420P8, w, h, [(w, h, y), (cw, ch, cb), (cw, ch, cr)], 85)
    assert out == fixture("jpeg/encoded/mmrecode-q85-420.mjpg")


# transform.rs:151-156 transforms_constant_blocks_to_dc_only: flat 138 with unit quantisers -> DC 80 only
def test_forward_dct_known_answers():
    q = np.ones((1, 64), np.uint8)
    c = oracle.fdct_quantize_many(np.full((1, 64), 138, np.uint8), q)[0]
    assert c[0] == 80 and not c[1:].any()
    assert not oracle.fdct_quantize_many(np.full((1, 64), 128, np.uint8), q).any()


@pytest.mark.parametrize("args", [
    (20261203, 0, 1920, 1080, "422", 90, 120),   # the 1080p 4:2:2 benchmark frame
    (20261201, 3, 640, 480, "420", 75, 0),       # the VGA 4:2:0 q75 plain configuration
    (7, 1, 333, 97, "444", 50, 4),
    (9, 2, 1000, 64, "422", 95, 63),
])
def test_generator_equals_the_product_generator(args):
    seed, index = args[0], args[1]
    a = osynth.mjpeg_packet(*args)
    b = synth.mjpeg_stream(seed, index + 1, *args[2:])[index]
    assert a == b


def test_level_writer_round_trips_through_the_oracle_decoder():
    rng = np.random.default_rng(3)
    n = 4 * 2  # 16x32 gray: 2 x 4 MCUs
    lv = np.zeros((n, 64), np.int32)
    lv[:, 0] = rng.integers(-300, 300, n)
    lv[:, 1:] = rng.integers(-1023, 1024, (n, 63)) * (rng.random((n, 63)) < 0.5)
    qt = [np.ones(64, np.uint8)]
    pkt = oracle.jpeg_write_levels(16, 32, [(1, 1)], [0], qt, lv, restart_interval=3)
    r = oracle.jpeg_decode(pkt)
    assert r.status == 0
    plane = np.frombuffer(r.frame.planes[0][2], np.uint8).reshape(32, 16)
    blocks = oracle.jpeg_idct_many(lv)
    for b in range(n):
        by, bx = divmod(b, 2)
        assert plane[by * 8:by * 8 + 8, bx * 8:bx * 8 + 8].tobytes() == blocks[b].tobytes()
    with pytest.raises(ValueError):
        bad = lv.copy()
        bad[1, 0] = bad[0, 0] + 2048
        oracle.jpeg_write_levels(16, 32, [(1, 1)], [0], qt, bad)


def test_product_encoder_equals_the_oracle_encoder_on_random_settings():
    """mmr_mjpeg_encode_ex (the CPU encoder the GPU encoder is checked against) and the
    oracle's encoder: byte-identical streams for 200 random frames (gray, 4:2:0, 4:2:2,
    4:4:4; 1x1 to 89x69, odd sizes), every quality 1..100 reachable, both table sets,
    restart intervals from 1 to 65535; the same message for rejected qualities."""
    rng = np.random.default_rng(77)
    for i in range(200):
        sub = ["420", "422", "444", "gray"][i % 4]
        w, h = int(rng.integers(1, 90)), int(rng.integers(1, 70))
        q, annex_k = int(rng.integers(1, 101)), bool(rng.integers(0, 2))
        ri = int(rng.choice([0, 1, 2, 3, 7, 64, 65535]))
        if sub == "gray":
            y = rng.integers(0, 256, (h, w), dtype=np.uint8).tobytes()
            frame = m.VideoFrame(m.GRAY8, w, h, [m.Plane(y, w, w, h)], m.RANGE_FULL)
        else:
            frame = synth.mjpeg_frame(900 + i, 0, w, h, sub)
        planes = [(p.width, p.height, bytes(p.data)) for p in frame.planes]
        got = m.encode_jpeg(frame, q, annex_k=annex_k, restart_interval=ri)
        want = oracle.jpeg_encode(frame.format, w, h, planes, q, annex_k=annex_k, restart_interval=ri)
        assert got == want, (i, sub, w, h, q, annex_k, ri)
    frame = synth.mjpeg_frame(1, 0, 16, 16, "420")
    planes = [(p.width, p.height, bytes(p.data)) for p in frame.planes]
    for q in (0, 101, 255):
        with pytest.raises(m.MmrError) as got:
            m.encode_jpeg(frame, q)
        with pytest.raises(ValueError) as want:
            oracle.jpeg_encode(frame.format, 16, 16, planes, q)
        assert got.value.status == m.INVALID_DATA and got.value.message == "invalid data: " + str(want.value)
