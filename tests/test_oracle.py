"""The CPU oracle against every known answer and fixture of the reference's own tests.

Each test names the reference test it restates."""

import hashlib
import json
import math
import os

import numpy as np
import pytest

import oracle
from helpers import GOLDEN, JPEG_FIXTURES, DV_FIXTURES, fixture, jpeg


# transform.rs:140-149 reconstructs_constant_dc_blocks
@pytest.mark.parametrize("c0,value", [(0, 128), (80, 138), (-1024, 0)])
def test_jpeg_idct_dc_known_answers(c0, value):
    assert oracle.jpeg_idct([c0] + [0] * 63) == bytes([value]) * 64


# dv/src/decoder.rs:639-645 inverse_dc_block_is_constant
def test_dv_idct_dc_known_answers():
    c = [1024] + [0] * 63
    assert oracle.dv_idct88(c) == bytes([128]) * 64
    assert oracle.dv_idct248(c) == bytes([128]) * 64


def test_round_half_away_from_zero_tie():
    # a DC-only block whose value lands exactly on x.5: C*(C*4) + 128 = 128.5 -> 129 (f64::round)
    assert oracle.jpeg_idct([4] + [0] * 63)[0] == 129


# decoder.rs:583-609 decodes_checked_in_baseline_vectors
def test_fixture_dimensions_and_formats():
    expect = {
        "jpeg/valid/baseline-420.jpg": (16, 16, 3, [(16, 16), (8, 8), (8, 8)]),
        "jpeg/valid/minimal-gray.jpg": (8, 8, 3, None),
        "jpeg/valid/unknown-app-marker.jpg": (16, 16, 3, None),
        "jpeg/valid/restart-interval.jpg": (16, 8, 1, None),
    }
    for rel, (w, h, n, dims) in expect.items():
        r = oracle.jpeg_decode(fixture(rel))
        assert r.status == 0, (rel, r.message)
        assert (r.frame.width, r.frame.height, len(r.frame.planes)) == (w, h, n)
        if dims:
            assert [(p[0], p[1]) for p in r.frame.planes] == dims
    r = oracle.jpeg_decode(fixture("jpeg/valid/baseline-420.jpg"))
    assert r.color_model == 1  # YCbCr
    r = oracle.jpeg_decode(fixture("jpeg/valid/restart-interval.jpg"))
    assert r.color_model == 0 and set(r.frame.planes[0][2]) == {128}


# parser.rs:447-502
def test_parser_known_answers():
    for rel, dims in [("jpeg/valid/baseline-420.jpg", (16, 16)), ("jpeg/valid/minimal-gray.jpg", (8, 8)),
                      ("jpeg/valid/unknown-app-marker.jpg", (16, 16)), ("jpeg/valid/restart-interval.jpg", (16, 8))]:
        st, _, info = oracle.jpeg_parse(fixture(rel))
        assert st == 0 and (info["width"], info["height"]) == dims and info["last_marker"] == 0xD9
    st, _, info = oracle.jpeg_parse(fixture("jpeg/parser/stuffed-restarts.jpg"))
    assert st == 0 and info["data_length"] == 9 and info["restart_numbers"] == [0, 7]
    st, msg, _ = oracle.jpeg_parse(fixture("jpeg/invalid/invalid-length.jpg"))
    assert st == oracle.INVALID_DATA and "0x00000004" in msg
    assert oracle.jpeg_parse(fixture("jpeg/invalid/missing-eoi.jpg"))[0] != 0
    assert oracle.jpeg_parse(fixture("jpeg/invalid/truncated-marker.jpg"))[0] != 0


# entropy.rs:190-213: canonical codes [1,2,...] read 0b0101_1000 as symbols of lengths 1,2,2;
# FF 00 is one 0xFF data byte; receive_extend(0b001, 3) = -6 and (0b100, 3) = 4.
def test_entropy_known_answers_through_a_crafted_stream():
    # DC table counts [1, 2]: code 0 -> cat 0, 10 -> cat 3, 11 -> cat 1 (the decoder's first
    # three canonical codes, as in the reference test); AC table: EOB only.
    dc = ([1, 2] + [0] * 14, [0, 3, 1])
    ac = ([1] + [0] * 15, [0])
    # block 1: DC cat 3 bits 001 -> diff -6; block 2: DC cat 3 bits 100 -> +4 (pred -2)
    # bits: 10 001 0 | 10 100 0 | padding 1111
    entropy = bytes([0b10001010, 0b10001111])
    data = jpeg(16, 8, [(1, 1, 1, 0)], dht=[(0, 0, *dc), (1, 0, *ac)], entropy=entropy)
    r = oracle.jpeg_decode(data)
    assert r.status == 0, r.message
    y = r.frame.planes[0][2]
    # DC-only blocks: sample = round(C00^2 * dc + 128) with C00^2 ~ 1/8
    assert y[0] == 127 and y[8] == 128
    # FF 00 is one 0xFF data byte: DC code 11 (cat 1), value bit 1 (+1), then the AC decoder
    # reads 1111... where only "0" (EOB) is a code -> no code matches within 16 bits.
    data = jpeg(8, 8, [(1, 1, 1, 0)], dht=[(0, 0, *dc), (1, 0, *ac)], entropy=bytes([0xFF, 0x00] * 4))
    r = oracle.jpeg_decode(data)
    assert r.status == oracle.INVALID_DATA and "no Huffman code matches" in r.message
    # 11 1 0 then padding: DC +1, EOB -> 1/8 + 128
    data = jpeg(8, 8, [(1, 1, 1, 0)], dht=[(0, 0, *dc), (1, 0, *ac)], entropy=bytes([0b11100111]))
    r = oracle.jpeg_decode(data)
    assert r.status == 0 and r.frame.planes[0][2][0] == 128


# decoder.rs:611-618 restart vector (all 128) and parser RST handling
def test_restart_vector_decodes_to_grey():
    r = oracle.jpeg_decode(fixture("jpeg/valid/restart-interval.jpg"))
    assert r.status == 0 and r.frame.planes[0][2] == bytes([128]) * 128


# dv/tests/reference_vectors.rs:11-33 and :48-64
def test_dv_fixtures_and_damage():
    for rel, fmt, w, h in [(DV_FIXTURES[0], oracle.FMT_YUV411P8, 720, 480), (DV_FIXTURES[1], oracle.FMT_YUV420P8, 720, 576)]:
        data = fixture(rel)
        assert oracle.dv_issue_count(data)[:2] == (0, 0)
        r = oracle.dv_decode(data)
        assert r.status == 0 and r.frame.format == fmt and (r.frame.width, r.frame.height) == (w, h)
        assert any(r.frame.planes[0][2])
    damaged = bytearray(fixture(DV_FIXTURES[0]))
    damaged[7 * 80] = 0x76
    assert oracle.dv_decode(bytes(damaged)).status == oracle.INVALID_DATA
    r = oracle.dv_decode(bytes(damaged), conceal=True)
    assert r.status == 0 and r.concealed == [(0, 0)]


# dif.rs:296-308 reports_localized_identifier_damage; profile.rs:129-146
def test_dv_profile_detection():
    ntsc = bytearray(b"\xff" * 120000)
    ntsc[:4] = b"\x1f\x07\x00\x3f"
    assert oracle.dv_issue_count(bytes(ntsc))[0] == 0
    pal_header_ntsc_size = bytearray(ntsc)
    pal_header_ntsc_size[3] = 0xBF
    assert oracle.dv_decode(bytes(pal_header_ntsc_size)).status == oracle.INVALID_DATA
    assert oracle.dv_decode(b"\x00\x00").status == oracle.INVALID_DATA


def test_oracle_outputs_match_pinned_checksums():
    pinned = json.load(open(os.path.join(GOLDEN, "oracle_outputs.json")))
    for rel in JPEG_FIXTURES + DV_FIXTURES:
        r = oracle.jpeg_decode(fixture(rel)) if rel.startswith("jpeg") else oracle.dv_decode(fixture(rel))
        p = pinned[rel]
        assert (r.status, r.message) == (p["status"], p["message"]), rel
        if r.frame:
            got = [[w, h, hashlib.sha256(b).hexdigest()] for w, h, b in r.frame.planes]
            assert got == p["planes"], rel
            assert hashlib.sha256(oracle.rgb24(r.frame)).hexdigest() == p["rgb24"], rel


def test_cos_table_is_libm_cos():
    # the reference calls libm cos(fl(k*PI)/16); the oracle's table must equal it here
    for k in range(128):
        assert oracle.dv_cos(k) == math.cos(float(k) * math.pi / 16.0)


# terminal_preview.rs:7576-7611 converts_limited_range_yuv_to_rgb_preview
def test_rgb_conversion_known_answer():
    f = oracle.Frame(oracle.FMT_YUV420P8, oracle.RANGE_LIMITED, 2, 2,
                     [(2, 2, bytes([16, 235, 81, 145])), (1, 1, bytes([128])), (1, 1, bytes([128]))])
    rgb = oracle.rgb24(f)
    assert rgb[0:3] == bytes([0, 0, 0]) and rgb[3:6] == bytes([255, 255, 255])


def _rgb_reference(fmt, rng_kind, w, h, planes):
    """video_frame_image at 1:1 (terminal_preview.rs:7159-7236) and ycbcr_to_rgb
    (:7308-7330), restated here in numpy from the reference source."""
    if fmt == oracle.FMT_GRAY8:
        y = np.frombuffer(planes[0][2], np.uint8).reshape(h, w)
        return np.repeat(y[:, :, None], 3, axis=2).tobytes()
    (yw, yh, yb), (bw, bh, bb), (rw, rh, rb) = planes
    xs, ys = np.arange(w), np.arange(h)

    def sample(pw, ph, data):
        a = np.frombuffer(data, np.uint8).reshape(ph, pw).astype(np.int64)
        cx = np.minimum(xs * pw // w, pw - 1)
        cy = np.minimum(ys * ph // h, ph - 1)
        return a[cy][:, cx]

    y, cb, cr = sample(yw, yh, yb), sample(bw, bh, bb) - 128, sample(rw, rh, rb) - 128
    if rng_kind == oracle.RANGE_LIMITED:
        y = np.maximum(y - 16, 0)
        r = (298 * y + 409 * cr + 128) >> 8
        g = (298 * y - 100 * cb - 208 * cr + 128) >> 8
        b = (298 * y + 516 * cb + 128) >> 8
    else:
        r = y + ((359 * cr + 128) >> 8)
        g = y - ((88 * cb + 183 * cr + 128) >> 8)
        b = y + ((454 * cb + 128) >> 8)
    return np.clip(np.stack([r, g, b], axis=2), 0, 255).astype(np.uint8).tobytes()


@pytest.mark.parametrize("rng_kind", [oracle.RANGE_FULL, oracle.RANGE_LIMITED], ids=["full", "limited"])
def test_rgb_conversion_every_triple(rng_kind):
    """All 2^24 (Y, Cb, Cr) triples through the oracle's conversion at 4:4:4 against the
    restatement: pins the full-range formula, which the reference's tests leave unpinned."""
    v = np.arange(1 << 24, dtype=np.uint32)
    planes = [(4096, 4096, (v >> 16).astype(np.uint8).tobytes()), (4096, 4096, ((v >> 8) & 255).astype(np.uint8).tobytes()),
              (4096, 4096, (v & 255).astype(np.uint8).tobytes())]
    f = oracle.Frame(oracle.FMT_YUV444P8, rng_kind, 4096, 4096, planes)
    assert oracle.rgb24(f) == _rgb_reference(oracle.FMT_YUV444P8, rng_kind, 4096, 4096, planes)


def test_rgb_conversion_subsampled_layouts():
    """Gray and every chroma layout, odd sizes, both ranges: the nearest-sample chroma
    index min(x * cw / W, cw - 1) and the row index alike."""
    rng = np.random.default_rng(12)
    layouts = {oracle.FMT_YUV420P8: (2, 2), oracle.FMT_YUV422P8: (2, 1), oracle.FMT_YUV444P8: (1, 1),
               oracle.FMT_YUV411P8: (4, 1), oracle.FMT_GRAY8: None}
    for i in range(60):
        fmt = list(layouts)[i % 5]
        w, h = int(rng.integers(1, 70)), int(rng.integers(1, 50))
        planes = [(w, h, rng.integers(0, 256, w * h, dtype=np.uint8).tobytes())]
        if layouts[fmt]:
            sx, sy = layouts[fmt]
            cw, ch = (w + sx - 1) // sx, (h + sy - 1) // sy
            planes += [(cw, ch, rng.integers(0, 256, cw * ch, dtype=np.uint8).tobytes()) for _ in range(2)]
        for rk in (oracle.RANGE_FULL, oracle.RANGE_LIMITED):
            f = oracle.Frame(fmt, rk, w, h, planes)
            assert oracle.rgb24(f) == _rgb_reference(fmt, rk, w, h, planes), (i, fmt, w, h, rk)
