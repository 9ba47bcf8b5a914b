"""GPU whole-stream decode (mmr_gpu_stream_*) vs the stream oracle: the same
framing, the same first error (status and message), the same Y4M bytes."""

import os

import numpy as np
import pytest

import mmrecode_gb300 as m
import oracle
from mmrecode_gb300 import synth
from oracle import stream as ost

from helpers import fixture

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = m.Context()
    yield c
    c.close()


def candidates_np(data: bytes) -> int:
    """Positions whose byte is 0xFF and whose next byte is not 0x00, 0xFF or RST0..7."""
    a = np.frombuffer(data, np.uint8)
    if len(a) < 2:
        return 0
    nx = a[1:]
    return int(((a[:-1] == 0xFF) & (nx != 0) & (nx != 0xFF) & ((nx & 0xF8) != 0xD0)).sum())


def check(ctx, data: bytes, name: str = "input"):
    ref = ost.decode_stream_y4m(data, name)
    with ctx.open_stream(data, name) as ms:
        assert ms.kind == ref["kind"]
        if ms.kind == ost.KIND_MJPEG:
            assert ms.candidates == candidates_np(data)
            ext, st, msg = ost.frame_extents(data)
            assert ms.frames() == ext
            assert (ms.frame_status, ms.frame_message) == (st, msg)
        out, y4m = ms.decode_y4m()
    assert out.status == ref["status"], (out.message, ref["message"])
    if ref["kind"] in (ost.KIND_MPEGTS, ost.KIND_MPEG2):
        return out
    assert out.message == ref["message"]
    assert out.frames_written == ref["frames"]
    assert y4m == (ref["y4m"] or b"")
    return out


def _ecs_end(jpg: bytes) -> int:
    """Offset of the EOI marker that ends a single-scan image."""
    assert jpg.endswith(b"\xff\xd9")
    return len(jpg) - 2


def _with_com(jpg: bytes, payload: bytes) -> bytes:
    """The image with a COM segment right after SOI."""
    seg = b"\xff\xfe" + (len(payload) + 2).to_bytes(2, "big") + payload
    return jpg[:2] + seg + jpg[2:]


@pytest.fixture(scope="module")
def small():
    return synth.mjpeg_stream(11, 6, 320, 240, "420", 75, 0)


def test_reference_fixtures(ctx):
    enc = fixture("jpeg/encoded/mmrecode-q85-420.mjpg")
    out = check(ctx, enc)
    assert (out.status, out.frames_written) == (0, 2)
    for name in ("baseline-420.jpg", "minimal-gray.jpg", "restart-interval.jpg", "unknown-app-marker.jpg"):
        one = fixture(f"jpeg/valid/{name}")
        check(ctx, one)
        check(ctx, one * 3)
    check(ctx, fixture("jpeg/parser/stuffed-restarts.jpg") * 2)
    for name in ("invalid-length.jpg", "missing-eoi.jpg", "truncated-marker.jpg"):
        bad = fixture(f"jpeg/invalid/{name}")
        check(ctx, bad)
        check(ctx, enc + bad)


def test_errors_between_and_after_frames(ctx):
    enc = fixture("jpeg/encoded/mmrecode-q85-420.mjpg")
    assert check(ctx, enc + b"junk").frames_written == 2
    assert check(ctx, enc + fixture("jpeg/valid/minimal-gray.jpg")).frames_written == 2  # format change
    for tiny in (b"", b"\xff", b"\xff\xd8\xff", b"\x00\x01\x02"):
        check(ctx, tiny)
    ts = bytearray(3 * 188)
    for k in range(3):
        ts[k * 188] = 0x47
    assert check(ctx, bytes(ts)).status == oracle.UNSUPPORTED
    es = bytearray(enc)
    es[40:44] = b"\x00\x00\x01\xb3"
    assert check(ctx, bytes(es)).status == oracle.UNSUPPORTED


def test_synthetic_streams(ctx, small):
    check(ctx, b"".join(small))
    check(ctx, b"".join(synth.mjpeg_stream(12, 5, 256, 128, "422", 90, 16)))  # restart interval of one MCU row
    check(ctx, b"".join(synth.mjpeg_stream(13, 4, 200, 136, "444", 60, 4)))
    # 0xFF fill before each SOI and inside the marker that ends each scan
    filled = [b"\xff\xff" + p[:_ecs_end(p)] + b"\xff\xff\xff\xd9" for p in small]
    check(ctx, b"".join(filled))


def test_markers_inside_header_segments(ctx, small):
    # FF D9 / FF DA / FF D8 bytes in a COM payload are candidates that the framing must skip
    doctored = [_with_com(p, b"x\xff\xd9\xff\xda\xff\xd8\xffy") for p in small]
    check(ctx, b"".join(doctored))


def test_more_candidates_than_the_first_pass_holds(ctx, small):
    payload = b"\xff\x01" * 30000  # 30000 candidates per COM segment
    big = _with_com(_with_com(_with_com(small[0], payload), payload), payload)
    with ctx.open_stream(big + small[1]) as ms:
        assert ms.candidates == candidates_np(big + small[1]) > 65536
    check(ctx, big + small[1])


def test_truncated_streams(ctx, small):
    whole = b"".join(small[:3])
    last = small[3]
    check(ctx, whole + last[: len(last) - 10])  # no terminating marker
    ecs0 = last.index(b"\xff\xda") + 2
    ecs0 += int.from_bytes(last[ecs0:ecs0 + 2], "big")
    stuffed = last.index(b"\xff\x00", ecs0)
    out = check(ctx, whole + last[: stuffed + 1])  # ends in the middle of a stuffed 0xFF
    assert "truncated marker in entropy-coded data" in out.message


def test_corrupted_middle_frame(ctx, small):
    frames = list(small[:4])
    p = bytearray(frames[2])
    mid = len(p) // 2
    p[mid:mid + 8] = b"\xff\x00" * 4  # 32 one bits: no Huffman code matches
    frames[2] = bytes(p)
    out = check(ctx, b"".join(frames))
    assert (out.frames_written, out.status) == (2, oracle.INVALID_DATA)


def test_dv_streams(ctx):
    ntsc = fixture("dv/valid/dv25-525-60-one-frame.dv")
    pal = fixture("dv/valid/dv25-625-50-one-frame.dv")
    assert check(ctx, ntsc * 3).frames_written == 3
    assert check(ctx, pal * 2).frames_written == 2
    check(ctx, ntsc * 2 + b"\0", "clip.dv")  # incomplete raw DV frame
    gen = b"".join(synth.dv_stream(21, 3))
    assert check(ctx, gen).frames_written == 3
    bad = bytearray(ntsc * 3)
    bad[120000] = 0xFF  # the second frame's first DIF block is not a header
    check(ctx, bytes(bad))


def test_vga_stream_matches_oracle(ctx):
    check(ctx, b"".join(synth.mjpeg_stream(31, 40, 640, 480, "420", 75, 0, annex_k=True)))


def test_1080p_stream_properties(ctx):
    # 120 frames of the benchmark's kind: 135 MB of stream, more than the 129 MB L2
    packets = synth.mjpeg_stream(41, 120, 1920, 1080, "422", 90, 120, annex_k=True)
    data = b"".join(packets)
    with ctx.open_stream(data) as ms:
        assert ms.frame_count == 120 and ms.frame_status == 0
        assert ms.candidates == candidates_np(data)
        offs = np.cumsum([0] + [len(p) for p in packets[:-1]]).tolist()
        assert ms.frames() == list(zip(offs, [len(p) for p in packets]))
        out, y4m = ms.decode_y4m()
    assert (out.status, out.frames_written) == (0, 120)
    head = b"YUV4MPEG2 W1920 H1080 Ip C422 XCOLORRANGE=FULL\n"
    plane = 1920 * 1080 * 2
    assert len(y4m) == len(head) + 120 * (6 + plane) and y4m.startswith(head)
    for k in (0, 77, 119):
        ref = oracle.jpeg_decode(packets[k])
        at = len(head) + k * (6 + plane)
        assert y4m[at:at + 6] == b"FRAME\n"
        assert y4m[at + 6:at + 6 + plane] == b"".join(ref.frame.plane_bytes())


def test_decode_file(ctx, tmp_path, small):
    src = tmp_path / "in.mjpg"
    src.write_bytes(b"".join(small))
    dst = tmp_path / "out.y4m"
    line = m.decode_file(str(src), str(dst), ctx)
    assert line == f"Decoded 6 JPEG frame(s) to {dst}"
    assert dst.read_bytes() == ost.decode_stream_y4m(src.read_bytes())["y4m"]
    dv = tmp_path / "in.dv"
    dv.write_bytes(fixture("dv/valid/dv25-525-60-one-frame.dv") * 2)
    assert m.decode_file(str(dv), str(tmp_path / "dv.y4m"), ctx) == f"Decoded 2 raw DV frame(s) to {tmp_path / 'dv.y4m'}"
    # rejected before the output exists
    dv.write_bytes(fixture("dv/valid/dv25-525-60-one-frame.dv") + b"\0")
    gone = tmp_path / "none.y4m"
    with pytest.raises(m.MmrError) as e:
        m.decode_file(str(dv), str(gone), ctx)
    assert e.value.message == f"'{dv}' ends with an incomplete raw DV frame" and not os.path.exists(gone)
    # an error after two frames: the two frames are written
    src.write_bytes(fixture("jpeg/encoded/mmrecode-q85-420.mjpg") + b"junk")
    with pytest.raises(m.MmrError):
        m.decode_file(str(src), str(dst), ctx)
    assert dst.read_bytes() == ost.decode_stream_y4m(src.read_bytes())["y4m"]
