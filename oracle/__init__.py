"""ctypes wrapper of the CPU oracle (oracle/*.c).

TEST INFRASTRUCTURE ONLY. The oracle restates the reference decoder
(markusmoenig/MMRecode, crates/codecs/{mjpeg,dv} and the terminal-preview RGB
conversion) in C. Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` may use it; the product library never does.
"""

from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass, field

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

OK, INVALID_ARGUMENT, INVALID_DATA, UNSUPPORTED, INVALID_STATE, INTERNAL = 0, 1, 2, 3, 4, 100
FMT_GRAY8, FMT_YUV420P8, FMT_YUV422P8, FMT_YUV444P8, FMT_YUV411P8 = 1, 2, 3, 4, 5
RANGE_FULL, RANGE_LIMITED = 1, 2


class _Plane(ctypes.Structure):
    _fields_ = [("data", ctypes.POINTER(ctypes.c_uint8)), ("width", ctypes.c_size_t), ("height", ctypes.c_size_t)]


class _Frame(ctypes.Structure):
    _fields_ = [
        ("format", ctypes.c_uint32),
        ("range", ctypes.c_uint32),
        ("width", ctypes.c_size_t),
        ("height", ctypes.c_size_t),
        ("plane_count", ctypes.c_size_t),
        ("planes", _Plane * 3),
    ]


class _Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("message", ctypes.c_char * 512)]


class _JpegInfo(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_size_t),
        ("height", ctypes.c_size_t),
        ("component_count", ctypes.c_size_t),
        ("scan_count", ctypes.c_size_t),
        ("data_offset", ctypes.c_size_t),
        ("data_length", ctypes.c_size_t),
        ("restart_count", ctypes.c_size_t),
        ("restart_offsets", ctypes.c_size_t * 64),
        ("restart_numbers", ctypes.c_uint8 * 64),
        ("segment_count", ctypes.c_size_t),
        ("last_marker", ctypes.c_uint8),
        ("trailing_length", ctypes.c_size_t),
    ]


class _JpegLayout(ctypes.Structure):
    _fields_ = [
        ("width", ctypes.c_uint32),
        ("height", ctypes.c_uint32),
        ("ncomp", ctypes.c_uint32),
        ("h", ctypes.c_uint8 * 3),
        ("v", ctypes.c_uint8 * 3),
        ("tq", ctypes.c_uint8 * 3),
        ("annex_k", ctypes.c_uint8),
        ("restart_interval", ctypes.c_uint16),
        ("qt", (ctypes.c_uint8 * 64) * 2),
    ]


class _Concealed(ctypes.Structure):
    _fields_ = [("sequence", ctypes.c_size_t), ("slot", ctypes.c_size_t)]


@dataclass
class Frame:
    """A decoded frame: planes are (width, height, bytes) with stride == width."""

    format: int
    range: int
    width: int
    height: int
    planes: list = field(default_factory=list)

    def plane_bytes(self) -> list[bytes]:
        return [p[2] for p in self.planes]


@dataclass
class Result:
    status: int
    message: str
    frame: Frame | None = None
    color_model: int = -1
    concealed: list = field(default_factory=list)


def build() -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        u8p = ctypes.POINTER(ctypes.c_uint8)
        L.orc_jpeg_decode.argtypes = [u8p, ctypes.c_size_t, ctypes.POINTER(_Frame), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(_Result)]
        L.orc_jpeg_parse.argtypes = [u8p, ctypes.c_size_t, ctypes.POINTER(_JpegInfo), ctypes.POINTER(_Result)]
        L.orc_dv_decode.argtypes = [u8p, ctypes.c_size_t, ctypes.c_int, ctypes.POINTER(_Frame), ctypes.POINTER(_Concealed),
                                    ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(_Result)]
        L.orc_dv_issue_count.argtypes = [u8p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t),
                                         ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(_Result)]
        L.orc_rgb24.argtypes = [ctypes.POINTER(_Frame), u8p, ctypes.POINTER(_Result)]
        L.orc_frame_free.argtypes = [ctypes.POINTER(_Frame)]
        L.orc_jpeg_idct.argtypes = [ctypes.POINTER(ctypes.c_int32), u8p]
        L.orc_dv_idct88.argtypes = [ctypes.POINTER(ctypes.c_int32), u8p]
        L.orc_dv_idct248.argtypes = [ctypes.POINTER(ctypes.c_int32), u8p]
        L.orc_dv_cos.argtypes = [ctypes.c_int]
        L.orc_dv_cos.restype = ctypes.c_double
        vp = ctypes.c_void_p
        for name in ("orc_jpeg_idct_many", "orc_dv_idct88_many", "orc_dv_idct248_many"):
            getattr(L, name).argtypes = [vp, ctypes.c_size_t, vp]
        L.orc_dv_coefficients.argtypes = [u8p, ctypes.c_size_t, vp, vp, ctypes.c_size_t]
        L.orc_dv_coefficients.restype = ctypes.c_size_t
        L.orc_dv_vlc_entries.argtypes = [vp, vp, vp, vp, ctypes.c_size_t]
        L.orc_dv_vlc_entries.restype = ctypes.c_size_t
        L.orc_jpeg_fdct_quantize_many.argtypes = [vp, vp, ctypes.c_size_t, vp]
        L.orc_jpeg_write_levels.argtypes = [ctypes.POINTER(_JpegLayout), vp, ctypes.c_size_t, vp, ctypes.c_size_t,
                                            ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(_Result)]
        L.orc_jpeg_encode.argtypes = [ctypes.POINTER(_Frame), ctypes.c_int, ctypes.c_int, ctypes.c_int, vp,
                                      ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(_Result)]
        _lib = L
    return _lib


def _buf(data: bytes):
    n = len(data)
    arr = (ctypes.c_uint8 * max(n, 1)).from_buffer_copy(data if n else b"\0")
    return arr, n


def _take_frame(f: _Frame) -> Frame:
    planes = []
    for i in range(f.plane_count):
        p = f.planes[i]
        planes.append((p.width, p.height, ctypes.string_at(p.data, p.width * p.height)))
    return Frame(f.format, f.range, f.width, f.height, planes)


def jpeg_decode(data: bytes) -> Result:
    """decode_jpeg(...).into_video_frame() (crates/codecs/mjpeg/src/decoder.rs:140-167, 69-126)."""
    L = lib()
    arr, n = _buf(data)
    fr, res, cm = _Frame(), _Result(), ctypes.c_int(-1)
    st = L.orc_jpeg_decode(arr, n, ctypes.byref(fr), ctypes.byref(cm), ctypes.byref(res))
    out = Result(st, res.message.decode(), None, cm.value)
    if st == OK:
        out.frame = _take_frame(fr)
        L.orc_frame_free(ctypes.byref(fr))
    return out


def jpeg_parse(data: bytes):
    """parse_jpeg (crates/codecs/mjpeg/src/parser.rs:18-81): (status, message, info dict)."""
    L = lib()
    arr, n = _buf(data)
    info, res = _JpegInfo(), _Result()
    st = L.orc_jpeg_parse(arr, n, ctypes.byref(info), ctypes.byref(res))
    d = {
        "width": info.width,
        "height": info.height,
        "component_count": info.component_count,
        "scan_count": info.scan_count,
        "data_offset": info.data_offset,
        "data_length": info.data_length,
        "restart_count": info.restart_count,
        "restart_offsets": list(info.restart_offsets[: min(64, info.restart_count)]),
        "restart_numbers": list(info.restart_numbers[: min(64, info.restart_count)]),
        "segment_count": info.segment_count,
        "last_marker": info.last_marker,
        "trailing_length": info.trailing_length,
    }
    return st, res.message.decode(), d


def dv_decode(data: bytes, conceal: bool = False) -> Result:
    """parse_frame + decode_video_with_options (crates/codecs/dv/src/{dif,decoder}.rs)."""
    L = lib()
    arr, n = _buf(data)
    fr, res = _Frame(), _Result()
    cap = 512
    conc = (_Concealed * cap)()
    cnt = ctypes.c_size_t(0)
    st = L.orc_dv_decode(arr, n, 1 if conceal else 0, ctypes.byref(fr), conc, cap, ctypes.byref(cnt), ctypes.byref(res))
    out = Result(st, res.message.decode())
    if st == OK:
        out.frame = _take_frame(fr)
        L.orc_frame_free(ctypes.byref(fr))
        out.concealed = [(conc[i].sequence, conc[i].slot) for i in range(min(cnt.value, cap))]
    return out


def dv_issue_count(data: bytes):
    L = lib()
    arr, n = _buf(data)
    cnt, first, res = ctypes.c_size_t(0), ctypes.c_size_t(0), _Result()
    st = L.orc_dv_issue_count(arr, n, ctypes.byref(cnt), ctypes.byref(first), ctypes.byref(res))
    return st, cnt.value, first.value


def rgb24(frame: Frame) -> bytes:
    """terminal_preview.rs video_frame_image at 1:1 scale (interleaved RGB24)."""
    L = lib()
    fr = _Frame()
    fr.format, fr.range, fr.width, fr.height, fr.plane_count = frame.format, frame.range, frame.width, frame.height, len(frame.planes)
    keep = []
    for i, (w, h, data) in enumerate(frame.planes):
        arr = (ctypes.c_uint8 * max(len(data), 1)).from_buffer_copy(data if data else b"\0")
        keep.append(arr)
        fr.planes[i].data = ctypes.cast(arr, ctypes.POINTER(ctypes.c_uint8))
        fr.planes[i].width, fr.planes[i].height = w, h
    out = (ctypes.c_uint8 * (frame.width * frame.height * 3))()
    res = _Result()
    st = L.orc_rgb24(ctypes.byref(fr), out, ctypes.byref(res))
    if st != OK:
        raise RuntimeError(res.message.decode())
    return bytes(out)


def _idct(fn, coefficients) -> bytes:
    c = (ctypes.c_int32 * 64)(*[int(v) for v in coefficients])
    out = (ctypes.c_uint8 * 64)()
    fn(c, out)
    return bytes(out)


def jpeg_idct(coefficients) -> bytes:
    return _idct(lib().orc_jpeg_idct, coefficients)


def dv_idct88(coefficients) -> bytes:
    return _idct(lib().orc_dv_idct88, coefficients)


def dv_idct248(coefficients) -> bytes:
    return _idct(lib().orc_dv_idct248, coefficients)


def dv_cos(k: int) -> float:
    return lib().orc_dv_cos(k)


# ------------------------------------------------------------ many blocks ---

def _blocks(fn, coefficients):
    """coefficients: int32 array (n, 64) -> uint8 array (n, 64)."""
    import numpy as np

    c = np.ascontiguousarray(coefficients, dtype=np.int32).reshape(-1, 64)
    out = np.empty(c.shape, dtype=np.uint8)
    fn(c.ctypes.data, c.shape[0], out.ctypes.data)
    return out


def jpeg_idct_many(coefficients):
    """transform.rs:86-109 on each row of an (n, 64) int32 array."""
    return _blocks(lib().orc_jpeg_idct_many, coefficients)


def dv_idct88_many(coefficients):
    """dv decoder.rs:520-548 on each row."""
    return _blocks(lib().orc_dv_idct88_many, coefficients)


def dv_idct248_many(coefficients):
    """dv decoder.rs:555-602 on each row."""
    return _blocks(lib().orc_dv_idct248_many, coefficients)


def fdct_quantize_many(samples, quant):
    """transform.rs:111-134: samples uint8 (n, 64), quantisers uint8 (n, 64) -> int32 (n, 64)."""
    import numpy as np

    s = np.ascontiguousarray(samples, dtype=np.uint8).reshape(-1, 64)
    q = np.ascontiguousarray(quant, dtype=np.uint8).reshape(-1, 64)
    out = np.empty(s.shape, dtype=np.int32)
    lib().orc_jpeg_fdct_quantize_many(s.ctypes.data, q.ctypes.data, s.shape[0], out.ctypes.data)
    return out


# ------------------------------------------------------------ encoder ---

def jpeg_write_levels(width, height, sampling, tq, qt, levels, annex_k=False, restart_interval=0) -> bytes:
    """A baseline JPEG whose quantised coefficients are `levels` (int32 (nblocks, 64),
    natural order, DC absolute, blocks in scan order); sampling = [(h, v)] per
    component, tq = quantisation table per component, qt = 1 or 2 tables of 64
    (natural order). Header and scan layout as the reference encoder writes them."""
    import numpy as np

    L = _JpegLayout()
    L.width, L.height, L.ncomp = width, height, len(sampling)
    for c, (h, v) in enumerate(sampling):
        L.h[c], L.v[c], L.tq[c] = h, v, tq[c]
    for t, table in enumerate(qt):
        for k in range(64):
            L.qt[t][k] = int(table[k])
    L.annex_k = 1 if annex_k else 0
    L.restart_interval = restart_interval
    lv = np.ascontiguousarray(levels, dtype=np.int32).reshape(-1, 64)
    cap = 256 + lv.shape[0] * 512
    out = (ctypes.c_uint8 * cap)()
    n, res = ctypes.c_size_t(0), _Result()
    st = lib().orc_jpeg_write_levels(ctypes.byref(L), lv.ctypes.data, lv.shape[0], out, cap, ctypes.byref(n),
                                     ctypes.byref(res))
    if st != OK:
        raise ValueError(res.message.decode())
    return bytes(out[:n.value])


def jpeg_encode(fmt, width, height, planes, quality, annex_k=False, restart_interval=0) -> bytes:
    """encode_jpeg (crates/codecs/mjpeg/src/encoder.rs:44-87) of planar 8-bit input:
    planes = [(width, height, bytes)] with stride == width."""
    fr = _Frame()
    fr.format, fr.range, fr.width, fr.height, fr.plane_count = fmt, RANGE_FULL, width, height, len(planes)
    keep = []
    for i, (w, h, data) in enumerate(planes):
        arr = (ctypes.c_uint8 * max(len(data), 1)).from_buffer_copy(data if data else b"\0")
        keep.append(arr)
        fr.planes[i].data = ctypes.cast(arr, ctypes.POINTER(ctypes.c_uint8))
        fr.planes[i].width, fr.planes[i].height = w, h
    cap = 4096 + 4 * sum(len(p[2]) for p in planes)
    out = (ctypes.c_uint8 * cap)()
    n, res = ctypes.c_size_t(0), _Result()
    st = lib().orc_jpeg_encode(ctypes.byref(fr), quality, 1 if annex_k else 0, restart_interval, out, cap,
                               ctypes.byref(n), ctypes.byref(res))
    if st != OK:
        raise ValueError(res.message.decode())
    return bytes(out[:n.value])


def dv_coefficients(data: bytes):
    """(coefficients int32 (n, 64), modes uint8 (n,)) of every block of a DV frame,
    as decode_segment hands them to the transforms (segment order)."""
    import numpy as np

    cap = 12 * 27 * 30
    coef = np.zeros((cap, 64), np.int32)
    modes = np.zeros(cap, np.uint8)
    arr, n = _buf(data)
    got = lib().orc_dv_coefficients(arr, n, coef.ctypes.data, modes.ctypes.data, cap)
    return coef[:got], modes[:got]


def dv_vlc_entries():
    """[(code, length, run, level)] of the DV VLC (decoder.rs:319-354), sorted by length."""
    import numpy as np

    cap = 1024
    code = np.zeros(cap, np.uint16)
    ln = np.zeros(cap, np.uint8)
    run = np.zeros(cap, np.uint8)
    level = np.zeros(cap, np.int16)
    n = lib().orc_dv_vlc_entries(code.ctypes.data, ln.ctypes.data, run.ctypes.data, level.ctypes.data, cap)
    return [(int(code[i]), int(ln[i]), int(run[i]), int(level[i])) for i in range(n)]
