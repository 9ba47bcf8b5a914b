"""CPU encoders (stream generation and mmr_*_encode) against the reference's pins."""

import numpy as np
import pytest

import mmrecode_gb300 as m
import oracle
from helpers import fixture, read_y4m_420


def _y4m_frames():
    out = []
    for w, h, y, cb, cr in read_y4m_420(fixture("y4m/valid/two-frame-420.y4m")):
        cw, ch = (w + 1) // 2, (h + 1) // 2
        out.append(m.VideoFrame(m.YUV420P8, w, h, [m.Plane(y, w, w, h), m.Plane(cb, cw, cw, ch), m.Plane(cr, cw, cw, ch)],
                                m.RANGE_FULL))
    return out


# crates/codecs/mjpeg/src/encoder.rs:621-630 encoded_output_is_deterministic
def test_mjpeg_encoder_matches_golden_bytes():
    stream = b"".join(m.encode_jpeg(f, 85) for f in _y4m_frames())
    assert stream == fixture("jpeg/encoded/mmrecode-q85-420.mjpg")


def test_mjpeg_encoder_sampling_modes_and_errors():
    frames = _y4m_frames()
    assert m.encode_jpeg(frames[0], 90)[:2] == b"\xff\xd8"
    with pytest.raises(m.MmrError) as e:
        m.encode_jpeg(frames[0], 0)
    assert e.value.status == m.INVALID_DATA and "quality" in e.value.message
    bad = m.VideoFrame(m.YUV420P8, 16, 16, frames[0].planes, m.RANGE_LIMITED)
    with pytest.raises(m.MmrError) as e:
        m.encode_jpeg(bad, 75)
    assert e.value.status == m.UNSUPPORTED


def test_annex_k_tables_are_complete_baseline_tables():
    # Every (run, size) symbol plus EOB and ZRL appears once in each AC table, and the
    # encoded stream decodes (oracle) to the same samples as the reference tables' stream.
    f = _y4m_frames()[0]
    a = oracle.jpeg_decode(m.encode_jpeg(f, 85))
    b = oracle.jpeg_decode(m.encode_jpeg(f, 85, annex_k=True))
    c = oracle.jpeg_decode(m.encode_jpeg(f, 85, annex_k=True, restart_interval=1))
    assert a.status == b.status == c.status == 0
    assert a.frame.planes == b.frame.planes == c.frame.planes


# crates/codecs/dv/src/encoder.rs:648-657 constant_frames_encode_deterministically_and_reconstruct
@pytest.mark.parametrize("pal", [False, True])
def test_dv_constant_96_round_trip(pal):
    w, h = 720, (576 if pal else 480)
    cw, ch = (360, 288) if pal else (180, 480)
    f = m.VideoFrame(m.YUV420P8 if pal else m.YUV411P8, w, h,
                     [m.Plane(bytes([96]) * (w * h), w, w, h), m.Plane(bytes([128]) * (cw * ch), cw, cw, ch),
                      m.Plane(bytes([128]) * (cw * ch), cw, cw, ch)])
    a, b = m.encode_dv(f), m.encode_dv(f)
    assert a == b and len(a) == (144000 if pal else 120000)
    r = oracle.dv_decode(a)
    assert r.status == 0 and r.frame.planes[0][2] == f.planes[0].data


def test_dv_248_mode_round_trip():
    r = oracle.dv_decode(fixture("dv/valid/dv25-525-60-one-frame.dv"))
    f = m.VideoFrame(r.frame.format, 720, 480, [m.Plane(b, w, w, h) for w, h, b in r.frame.planes])
    enc = m.encode_dv(f, m.DV_MODE_ACTIVITY)
    # at least some blocks use 2-4-8 mode (bit 9 of a block header)
    modes = 0
    for blk in range(1500):
        if (enc[blk * 80] >> 5) != 4:
            continue
        bits = "".join(f"{x:08b}" for x in enc[blk * 80 + 4: blk * 80 + 80])
        for start in (0, 112, 224, 336, 448, 528):
            modes += bits[start + 9] == "1"
    assert modes > 100
    d = oracle.dv_decode(enc)
    assert d.status == 0
    y0 = np.frombuffer(r.frame.planes[0][2], np.uint8).astype(int)
    y1 = np.frombuffer(d.frame.planes[0][2], np.uint8).astype(int)
    assert ((y0 - y1) ** 2).mean() < 2.0


def test_gpu_encode_bound_covers_worst_case_outputs():
    # mmr_gpu_jpeg_encode_bound is host code: every frame the encoder can produce fits.
    lib = m._lib.load()
    rng = np.random.default_rng(3)
    cases = [(m.GRAY8, 1, 1, 1), (m.YUV420P8, 2, 2, 3), (m.YUV422P8, 2, 1, 3), (m.YUV444P8, 1, 1, 3)]
    for fmt, sx, sy, n in cases:
        for w, h in [(1, 1), (9, 7), (64, 48), (123, 77)]:
            cw, ch = (w + sx - 1) // sx, (h + sy - 1) // sy
            dims = [(w, h)] + [(cw, ch)] * (n - 1)
            planes = [m.Plane(rng.integers(0, 256, (ph, pw), dtype=np.uint8).tobytes(), pw, pw, ph) for pw, ph in dims]
            frame = m.VideoFrame(fmt, w, h, planes, m.RANGE_FULL)
            for annex, ri in [(False, 0), (True, 1), (True, 3)]:
                data = m.encode_jpeg(frame, 100, annex, ri)  # q100 noise: the largest coefficients
                assert len(data) <= lib.mmr_gpu_jpeg_encode_bound(fmt, w, h, ri)
