"""The stream oracle (CLI ``decode`` + Y4M writer) pinned against the reference's
own known answers and fixtures; CPU only."""

import pytest

import oracle
from oracle import stream as ost

from helpers import fixture


def _gray_2x2():
    return oracle.Frame(oracle.FMT_GRAY8, oracle.RANGE_FULL, 2, 2, [(2, 2, b"\x01\x02\x03\x04")])


def test_y4m_writer_grayscale_known_answer():
    # crates/containers/y4m/src/lib.rs, writes_a_grayscale_frame
    w = ost.Y4mWriter()
    w.write_frame(_gray_2x2(), "p")
    assert bytes(w.out) == b"YUV4MPEG2 W2 H2 Ip Cmono XCOLORRANGE=FULL\nFRAME\n\x01\x02\x03\x04"


def test_y4m_writer_rejects_format_change_and_bad_planes():
    w = ost.Y4mWriter()
    w.write_frame(_gray_2x2(), "p")
    other = oracle.Frame(oracle.FMT_GRAY8, oracle.RANGE_FULL, 4, 2, [(4, 2, bytes(8))])
    with pytest.raises(ost.Y4mError) as e:
        w.write_frame(other, "p")
    assert e.value.message == "invalid data: Y4M stream dimensions or pixel format changed between frames"
    bad = oracle.Frame(oracle.FMT_YUV420P8, oracle.RANGE_FULL, 3, 3, [(3, 3, bytes(9)), (1, 2, bytes(2)), (2, 2, bytes(4))])
    with pytest.raises(ost.Y4mError) as e:
        ost.Y4mWriter().write_frame(bad, "p")
    assert e.value.message == "invalid data: Y4M plane 1 has inconsistent dimensions, stride, or storage"


def test_detection_order():
    assert ost.detect(b"") == ost.KIND_NONE
    ts = bytearray(3 * 188)
    for k in range(3):
        ts[k * 188] = 0x47
    assert ost.detect(bytes(ts)) == ost.KIND_MPEGTS
    es = bytearray(b"\xff" * 300)
    es[100:104] = b"\x00\x00\x01\xb3"
    assert ost.detect(bytes(es)) == ost.KIND_MPEG2
    es2 = bytearray(b"\xff" * 300)
    es2[256:260] = b"\x00\x00\x01\xb3"  # past the 256 windows the CLI looks at
    assert ost.detect(bytes(es2)) == ost.KIND_MJPEG
    assert ost.detect(b"\x1f\x07\x00\x3f") == ost.KIND_DV
    assert ost.detect(b"\x1f\x07\x00") == ost.KIND_MJPEG  # fewer than 4 bytes: not DV
    assert ost.detect(fixture("jpeg/valid/baseline-420.jpg")) == ost.KIND_MJPEG


def test_reference_encoded_stream_frames_at_each_eoi():
    # the reference encoder's two-image stream (mmrecode encode of two-frame-420.y4m at q85):
    # SOI at 0 and 727, EOI at 725 and 1477
    data = fixture("jpeg/encoded/mmrecode-q85-420.mjpg")
    ext, st, msg = ost.frame_extents(data)
    assert (ext, st, msg) == ([(0, 727), (727, 752)], oracle.OK, "")
    r = ost.decode_stream_y4m(data)
    assert (r["status"], r["message"], r["kind"], r["frames"]) == (oracle.OK, "", ost.KIND_MJPEG, 2)
    f0 = oracle.jpeg_decode(data[:727]).frame
    head = f"YUV4MPEG2 W{f0.width} H{f0.height} Ip C420jpeg XCOLORRANGE=FULL\n".encode()
    body = b"".join(b"FRAME\n" + b"".join(oracle.jpeg_decode(data[o:o + n]).frame.plane_bytes()) for o, n in ext)
    assert r["y4m"] == head + body


@pytest.mark.parametrize("name,height,chroma,plane", [("dv25-525-60-one-frame.dv", 480, "C411", 720 * 480 * 3 // 2),
                                                      ("dv25-625-50-one-frame.dv", 576, "C420jpeg", 720 * 576 * 3 // 2)])
def test_dv_fixture_streams(name, height, chroma, plane):
    one = fixture(f"dv/valid/{name}")
    r = ost.decode_stream_y4m(one + one)
    head = f"YUV4MPEG2 W720 H{height} Ib {chroma} XCOLORRANGE=LIMITED\n".encode()
    assert (r["status"], r["frames"]) == (oracle.OK, 2)
    assert len(r["y4m"]) == len(head) + 2 * (6 + plane) and r["y4m"].startswith(head)
    frame = b"".join(oracle.dv_decode(one).frame.plane_bytes())
    assert r["y4m"][len(head):] == (b"FRAME\n" + frame) * 2


def test_stream_errors():
    r = ost.decode_stream_y4m(b"")
    assert (r["status"], r["message"], r["y4m"]) == (oracle.INVALID_DATA, "input contains no media frames", None)
    one = fixture("dv/valid/dv25-525-60-one-frame.dv")
    r = ost.decode_stream_y4m(one + b"\0", "clip.dv")
    assert (r["status"], r["message"], r["y4m"]) == (oracle.INVALID_DATA,
                                                     "'clip.dv' ends with an incomplete raw DV frame", None)
    data = fixture("jpeg/encoded/mmrecode-q85-420.mjpg")
    r = ost.decode_stream_y4m(data + b"junk")
    assert (r["status"], r["frames"]) == (oracle.INVALID_DATA, 2)
    assert r["message"] == "invalid data: JPEG at byte 0x00000000: expected JPEG marker prefix 0xff"
    r = ost.decode_stream_y4m(data + fixture("jpeg/valid/minimal-gray.jpg"))
    assert (r["status"], r["frames"]) == (oracle.INVALID_DATA, 2)
    assert r["message"] == "invalid data: Y4M stream dimensions or pixel format changed between frames"
