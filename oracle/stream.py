"""CPU restatement of the reference CLI's ``decode`` command for MJPEG and raw DV input.

TEST INFRASTRUCTURE ONLY: only tests/ may use it, as the checker of the GPU
stream path (``mmr_gpu_stream_*``).

Restates, over the C oracle's parse_jpeg / decode_jpeg / parse_frame +
decode_video:
  crates/cli/src/main.rs:1533-1580   decode: detection, then parse_jpeg on what
                                     remains, one image at a time, each decoded
                                     and written before the next is parsed
  crates/cli/src/main.rs:1605-1633   decode_dv: exact frame-size chunks
  crates/cli/src/main.rs:1908-1921   is_mpeg2_video, is_mpegts
  crates/codecs/dv/src/profile.rs:107-123   detect_profile_prefix
  crates/containers/y4m/src/lib.rs:219-373  Y4mWriter::write_frame and its checks
Messages are what the CLI prints: the reference Error's Display (with its
"invalid data: " style prefix) or the CLI's own plain strings.
"""

from __future__ import annotations

from . import (FMT_GRAY8, FMT_YUV411P8, FMT_YUV420P8, FMT_YUV422P8, FMT_YUV444P8, INVALID_DATA, OK, RANGE_FULL,
               RANGE_LIMITED, UNSUPPORTED, dv_decode, jpeg_decode, jpeg_parse)

KIND_NONE, KIND_MJPEG, KIND_DV, KIND_MPEGTS, KIND_MPEG2 = 0, 1, 2, 3, 4
TS_PACKET_SIZE = 188

_PREFIX = {1: "invalid argument: ", 2: "invalid data: ", 3: "unsupported: ", 4: "invalid state: "}


def _display(status: int, message: str) -> str:
    """crates/core/src/error.rs:18-27."""
    return _PREFIX.get(status, "") + message


def detect(data: bytes) -> int:
    """The CLI's order of tests (main.rs:1536-1553)."""
    if not data:
        return KIND_NONE
    chunks = [data[i:i + TS_PACKET_SIZE] for i in range(0, min(len(data), 3 * TS_PACKET_SIZE), TS_PACKET_SIZE)]
    if len(data) >= TS_PACKET_SIZE and all(c[:1] == b"\x47" for c in chunks):
        return KIND_MPEGTS
    if any(data[i:i + 4] == b"\x00\x00\x01\xb3" for i in range(0, min(256, max(len(data) - 3, 0)))):
        return KIND_MPEG2
    if len(data) >= 4 and data[0] >> 5 == 0:
        return KIND_DV
    return KIND_MJPEG


class Y4mError(Exception):
    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status
        self.message = message


_CHROMA = {FMT_GRAY8: "Cmono", FMT_YUV420P8: "C420jpeg", FMT_YUV411P8: "C411", FMT_YUV422P8: "C422",
           FMT_YUV444P8: "C444"}
_NAMES = {FMT_GRAY8: "Gray8", FMT_YUV420P8: "Yuv420p8", FMT_YUV422P8: "Yuv422p8", FMT_YUV444P8: "Yuv444p8",
          FMT_YUV411P8: "Yuv411p8"}


def plane_dimensions(fmt: int, w: int, h: int) -> list:
    """lib.rs:340-373."""
    hw, qw, hh = (w + 1) // 2, (w + 3) // 4, (h + 1) // 2
    if fmt == FMT_GRAY8:
        return [(w, h)]
    if fmt == FMT_YUV420P8:
        return [(w, h), (hw, hh), (hw, hh)]
    if fmt == FMT_YUV411P8:
        return [(w, h), (qw, h), (qw, h)]
    if fmt == FMT_YUV422P8:
        return [(w, h), (hw, h), (hw, h)]
    if fmt == FMT_YUV444P8:
        return [(w, h)] * 3
    raise Y4mError(UNSUPPORTED, _display(UNSUPPORTED, "pixel format has no Y4M representation"))


class Y4mWriter:
    """Y4mWriter (lib.rs:219-300) over an in-memory output. ``field_order`` is the
    frame's: "p" progressive, "t"/"b" top/bottom field first."""

    def __init__(self):
        self.out = bytearray()
        self.stream_format = None

    def write_frame(self, frame, field_order: str) -> None:
        if frame.format not in _CHROMA:
            raise Y4mError(UNSUPPORTED, _display(UNSUPPORTED, "pixel format has no Y4M representation"))
        chroma = _CHROMA[frame.format]
        expected = plane_dimensions(frame.format, frame.width, frame.height)
        if len(frame.planes) != len(expected):
            raise Y4mError(INVALID_DATA, _display(
                INVALID_DATA, f"Y4M {_NAMES[frame.format]} frame requires {len(expected)} plane(s), "
                              f"found {len(frame.planes)}"))
        for i, ((pw, ph, data), (ew, eh)) in enumerate(zip(frame.planes, expected)):
            if (pw, ph) != (ew, eh) or len(data) < pw * ph:
                raise Y4mError(INVALID_DATA, _display(
                    INVALID_DATA, f"Y4M plane {i} has inconsistent dimensions, stride, or storage"))
        fmt = (frame.width, frame.height, frame.format)
        if self.stream_format is not None:
            if self.stream_format != fmt:
                raise Y4mError(INVALID_DATA, _display(
                    INVALID_DATA, "Y4M stream dimensions or pixel format changed between frames"))
        else:
            rng = {RANGE_FULL: " XCOLORRANGE=FULL", RANGE_LIMITED: " XCOLORRANGE=LIMITED"}.get(frame.range, "")
            self.out += f"YUV4MPEG2 W{frame.width} H{frame.height} I{field_order} {chroma}{rng}\n".encode()
            self.stream_format = fmt
        self.out += b"FRAME\n"
        for pw, ph, data in frame.planes:  # stride == width
            self.out += data[:pw * ph]


def frame_extents(data: bytes) -> tuple:
    """(extents, status, message): (offset, length) of each image parse_jpeg peels off
    a concatenated JFIF stream, and the parse error that stops it (OK, "" if none)."""
    out, pos = [], 0
    while pos < len(data):
        st, msg, info = jpeg_parse(data[pos:])
        if st != OK:
            return out, st, _display(st, msg)
        consumed = len(data) - pos - info["trailing_length"]
        out.append((pos, consumed))
        pos += consumed
    return out, OK, ""


def decode_stream_y4m(data: bytes, input_name: str = "input") -> dict:
    """status, message, kind, frames (written), y4m (the output file's bytes; None when
    the CLI fails before creating it)."""
    kind = detect(data)
    res = {"status": OK, "message": "", "kind": kind, "frames": 0, "y4m": None}
    if kind == KIND_NONE:
        res.update(status=INVALID_DATA, message="input contains no media frames")
        return res
    if kind in (KIND_MPEGTS, KIND_MPEG2):
        res.update(status=UNSUPPORTED, message="outside this library")
        return res
    w = Y4mWriter()
    if kind == KIND_DV:
        fs = 144000 if data[3] & 0x80 else 120000
        if len(data) % fs:
            res.update(status=INVALID_DATA, message=f"'{input_name}' ends with an incomplete raw DV frame")
            return res
        try:
            for off in range(0, len(data), fs):
                r = dv_decode(data[off:off + fs])
                if r.status != OK:
                    res.update(status=r.status, message=_display(r.status, r.message))
                    return res
                w.write_frame(r.frame, "b")  # dv decoder.rs:146
                res["frames"] += 1
        except Y4mError as e:
            res.update(status=e.status, message=e.message)
        finally:
            res["y4m"] = bytes(w.out)
        return res
    pos = 0
    try:
        while pos < len(data):
            st, msg, info = jpeg_parse(data[pos:])
            if st != OK:
                res.update(status=st, message=_display(st, msg))
                return res
            consumed = len(data) - pos - info["trailing_length"]
            r = jpeg_decode(data[pos:pos + consumed])
            if r.status != OK:
                res.update(status=r.status, message=_display(r.status, r.message))
                return res
            w.write_frame(r.frame, "p")  # mjpeg decoder.rs:93
            res["frames"] += 1
            pos += consumed
    except Y4mError as e:
        res.update(status=e.status, message=e.message)
    finally:
        res["y4m"] = bytes(w.out)
    return res
