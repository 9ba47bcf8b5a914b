"""GB300 MJPEG / DV25 intra-frame decoder: Python host API.

Mirrors the reference's decode interface for this path:

* ``decode_jpeg`` / ``decode_dv``: one packet -> ``VideoFrame`` through the C ABI
  (``mmr_mjpeg_decode`` / ``mmr_dv_decode``; crates/capi/src/lib.rs:331-359).
* ``MjpegDecoder`` / ``DvDecoder``: the ``Decoder`` trait
  (crates/core/src/codec.rs:102-130) -- configure / send_packet /
  receive_frame / flush, with the reference wrappers' state errors
  (crates/codecs/mjpeg/src/codec.rs:16-71, crates/codecs/dv/src/codec.rs:16-66).
  With ``batch > 1`` packets queue until a batch is full (or ``flush``) and
  decode together on the GPU.
* ``Context``: many packets per GPU pass (``mmr_gpu_decode_batch``).
* ``Server``: requests from many streams, admitted against a device-memory budget
  and batched continuously (``mmr_gpu_server_*``), with p50/p99 latency.

All decoding runs in CUDA kernels inside libmmrecode_gpu.so; there is no CPU
decode path.
"""

from __future__ import annotations

import collections
import ctypes
from dataclasses import dataclass, field

from . import _lib

STATUS_OK, INVALID_ARGUMENT, INVALID_DATA, UNSUPPORTED, INVALID_STATE, IO_ERROR, INTERNAL = 0, 1, 2, 3, 4, 5, 100
GRAY8, YUV420P8, YUV422P8, YUV444P8, YUV411P8 = 1, 2, 3, 4, 5
RANGE_UNSPECIFIED, RANGE_FULL, RANGE_LIMITED = 0, 1, 2
CODEC_MJPEG, CODEC_DV = 1, 2
SESSION_HOST_FRAMES, SESSION_DEVICE_FRAMES = 0, 1  # mmr_gpu_decoder_set_output
OUTPUT_PLANAR, OUTPUT_RGB24 = 0, 1
ITEM_CONCEAL, ITEM_OUT_DEVICE, ITEM_IN_DEVICE = 1, 2, 4
DV_MODE_88, DV_MODE_ACTIVITY = 0, 1
STREAM_NONE, STREAM_MJPEG, STREAM_DV, STREAM_MPEGTS, STREAM_MPEG2 = 0, 1, 2, 3, 4

MJPEG_CODEC_NAME = "video/mjpeg"  # crates/codecs/mjpeg/src/codec.rs:12
DV_CODEC_NAME = "video/dv"        # crates/codecs/dv/src/codec.rs:12


class MmrError(Exception):
    """A failed call: ``status`` is the C ABI status, ``message`` its diagnostic."""

    def __init__(self, status: int, message: str):
        super().__init__(message)
        self.status = status
        self.message = message


@dataclass
class Plane:
    data: bytes
    stride: int
    width: int
    height: int


@dataclass
class VideoFrame:
    format: int
    width: int
    height: int
    planes: list
    range: int = RANGE_UNSPECIFIED
    pts: object = None
    duration: object = None


@dataclass
class CodecDescriptor:
    codec_id: str
    media_type: str = "video"


@dataclass
class Packet:
    data: bytes
    pts: object = None
    duration: object = None


def version() -> str:
    return _lib.load().mmr_version().decode()


def abi_version() -> int:
    return _lib.load().mmr_abi_version()


def _frame_from_c(fr: _lib.VideoFrameC) -> VideoFrame:
    planes = []
    for i in range(fr.plane_count):
        p = fr.planes[i]
        planes.append(Plane(ctypes.string_at(p.data, p.data_len), p.stride, p.width, p.height))
    return VideoFrame(fr.format, fr.width, fr.height, planes, fr.range)


def _decode_one(fn, data: bytes) -> VideoFrame:
    lib = _lib.load()
    fr = _lib.VideoFrameC()
    fr.struct_size = ctypes.sizeof(_lib.VideoFrameC)
    buf = bytes(data)
    st = fn(buf, len(buf), ctypes.byref(fr))
    if st != STATUS_OK:
        raise MmrError(st, _lib.last_error())
    try:
        return _frame_from_c(fr)
    finally:
        lib.mmr_video_frame_free(ctypes.byref(fr))


def decode_jpeg(data: bytes) -> VideoFrame:
    """decode_jpeg(...).into_video_frame() on the GPU (crates/codecs/mjpeg/src/decoder.rs:140-167)."""
    return _decode_one(_lib.load().mmr_mjpeg_decode, data)


def decode_dv(data: bytes) -> VideoFrame:
    """parse_frame + decode_video on the GPU (crates/codecs/dv/src/{dif,decoder}.rs)."""
    return _decode_one(_lib.load().mmr_dv_decode, data)


def _view(frame: VideoFrame, keep: list) -> _lib.VideoFrameView:
    v = _lib.VideoFrameView()
    v.struct_size = ctypes.sizeof(_lib.VideoFrameView)
    v.format, v.range, v.width, v.height = frame.format, frame.range, frame.width, frame.height
    v.plane_count = len(frame.planes)
    for i, p in enumerate(frame.planes):
        data = bytes(p.data)
        arr = (ctypes.c_uint8 * max(len(data), 1)).from_buffer_copy(data or b"\0")
        keep.append(arr)
        v.planes[i].data = ctypes.cast(arr, _lib.u8p)
        v.planes[i].data_len = len(data)
        v.planes[i].stride, v.planes[i].width, v.planes[i].height = p.stride, p.width, p.height
    return v


def _take_buffer(st: int, b: _lib.Buffer) -> bytes:
    lib = _lib.load()
    if st != STATUS_OK:
        raise MmrError(st, _lib.last_error())
    try:
        return ctypes.string_at(b.data, b.len)
    finally:
        lib.mmr_buffer_free(ctypes.byref(b))


def encode_jpeg(frame: VideoFrame, quality: int = 75, annex_k: bool = False, restart_interval: int = 0) -> bytes:
    """Baseline JPEG encoder (crates/codecs/mjpeg/src/encoder.rs:44-87); the defaults reproduce it byte for byte."""
    lib = _lib.load()
    keep: list = []
    v = _view(frame, keep)
    b = _lib.Buffer()
    b.struct_size = ctypes.sizeof(_lib.Buffer)
    if not annex_k and not restart_interval:
        st = lib.mmr_mjpeg_encode(ctypes.byref(v), quality, ctypes.byref(b))
    else:
        o = _lib.JpegEncodeOptions(ctypes.sizeof(_lib.JpegEncodeOptions), quality, 1 if annex_k else 0, restart_interval)
        st = lib.mmr_mjpeg_encode_ex(ctypes.byref(v), ctypes.byref(o), ctypes.byref(b))
    return _take_buffer(st, b)


def encode_dv(frame: VideoFrame, mode_policy: int = DV_MODE_88) -> bytes:
    """DV25 encoder (crates/codecs/dv/src/encoder.rs:67-103); DV_MODE_88 reproduces it byte for byte."""
    lib = _lib.load()
    keep: list = []
    v = _view(frame, keep)
    b = _lib.Buffer()
    b.struct_size = ctypes.sizeof(_lib.Buffer)
    if mode_policy == DV_MODE_88:
        st = lib.mmr_dv_encode(ctypes.byref(v), ctypes.byref(b))
    else:
        st = lib.mmr_dv_encode_ex(ctypes.byref(v), mode_policy, ctypes.byref(b))
    return _take_buffer(st, b)


@dataclass
class FrameInfo:
    status: int
    format: int
    range: int
    width: int
    height: int
    plane_count: int
    plane_width: tuple
    plane_height: tuple
    planar_bytes: int
    rgb_bytes: int


def probe(codec: int, data: bytes) -> FrameInfo:
    """Output geometry of one packet from its headers (mmr_gpu_probe)."""
    lib = _lib.load()
    info = _lib.FrameInfo()
    info.struct_size = ctypes.sizeof(_lib.FrameInfo)
    buf = bytes(data)
    st = lib.mmr_gpu_probe(codec, buf, len(buf), ctypes.byref(info))
    if st != STATUS_OK:
        raise MmrError(st, _lib.last_error())
    return FrameInfo(info.status, info.format, info.range, info.width, info.height, info.plane_count,
                     tuple(info.plane_width), tuple(info.plane_height), info.planar_bytes, info.rgb_bytes)


@dataclass
class BatchResult:
    status: int
    message: str
    format: int = 0
    range: int = 0
    width: int = 0
    height: int = 0
    plane_count: int = 0
    plane_offset: tuple = ()
    plane_width: tuple = ()
    plane_height: tuple = ()
    out_bytes: int = 0
    concealed_segments: int = 0


def save_tuning(path: str, table: list) -> None:
    """Writes an autotuner table (``Context.autotune``'s list) as JSON."""
    import json
    with open(path, "w") as f:
        json.dump({"mmrecode_gpu_tuning": 1, "classes": table}, f, indent=1, sort_keys=True)


def load_tuning(path: str) -> list:
    """Reads a table written by ``save_tuning`` (for ``Context.set_tuning``)."""
    import json
    with open(path) as f:
        doc = json.load(f)
    if doc.get("mmrecode_gpu_tuning") != 1:
        raise ValueError(f"{path}: not an MMRecode GPU tuning table")
    return doc["classes"]


def _tune_entries(table) -> "ctypes.Array":
    arr = (_lib.TuneEntry * max(len(table), 1))()
    for k, t in enumerate(table):
        e = arr[k]
        e.frame_class = int(t["frame_class"])
        e.kind = 0 if t["kind"] == "slice" else 1
        e.slice_bits = int(t.get("slice_bits", 0))
        e.strip_mcus = int(t.get("strip_mcus", 0))
    return arr


class Context:
    """A GPU decode context: engines (CUDA stream + device arenas each) that decode batches."""

    def __init__(self, device: int = 0, engines: int = 0):
        """``engines``: batches decoded concurrently (own CUDA streams and arenas each); 0 = 4."""
        lib = _lib.load()
        cfg = _lib.GpuConfig(ctypes.sizeof(_lib.GpuConfig), device, 0, engines)
        h = ctypes.c_void_p()
        st = lib.mmr_gpu_context_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().mmr_gpu_context_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def last_batch_ms(self) -> float:
        return _lib.load().mmr_gpu_last_batch_ms(self._h)

    @property
    def last_batch_launches(self) -> int:
        return _lib.load().mmr_gpu_last_batch_launches(self._h)

    def autotune(self, items) -> list:
        """Tunes the slice size per entropy class and the transform strip per tiling class on
        a ``(_lib.GpuItem * n)`` sample (decoded several times); returns one dict per class:
        ``kind`` "slice" (``slice_bits``, ``entropy_ms`` per candidate) or "strip"
        (``strip_mcus``, ``transform_ms`` for the narrow and the wide strip)."""
        cap = 256
        rep = (_lib.TuneEntry * cap)()
        cnt = ctypes.c_size_t()
        st = _lib.load().mmr_gpu_autotune(self._h, items, len(items), rep, cap, ctypes.byref(cnt))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())
        out = []
        for k in range(min(cnt.value, cap)):
            e = rep[k]
            if e.kind == 0:
                out.append({"kind": "slice", "frame_class": e.frame_class, "slice_bits": e.slice_bits,
                            "frames": e.frames, "entropy_ms": dict(zip((1024, 2048, 4096, 8192), list(e.entropy_ms)))})
            else:
                out.append({"kind": "strip", "frame_class": e.frame_class, "strip_mcus": e.strip_mcus,
                            "frames": e.frames, "transform_ms": {"narrow": e.transform_ms[0], "wide": e.transform_ms[1]}})
        return out

    def set_tuning(self, table) -> None:
        """Installs an autotuner table (the list ``autotune`` returned, e.g. reloaded with
        ``load_tuning``) for later batches."""
        arr = _tune_entries(table)
        st = _lib.load().mmr_gpu_set_tuning(self._h, arr, len(table))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())

    def set_graphs(self, enable: bool) -> None:
        """CUDA-graph replay of repeated device-resident batches (default on)."""
        st = _lib.load().mmr_gpu_set_graphs(self._h, 1 if enable else 0)
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())

    def set_slice_bits(self, bits: int) -> None:
        """Bits per entropy-decoder slice for later batches (0: automatic). Output never depends on it."""
        st = _lib.load().mmr_gpu_set_slice_bits(self._h, bits)
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())

    def stats(self) -> dict:
        """Stage times (ms, CUDA events on the context stream) and sizes of the last batch."""
        s = _lib.BatchStats()
        s.struct_size = ctypes.sizeof(_lib.BatchStats)
        st = _lib.load().mmr_gpu_last_batch_stats(self._h, ctypes.byref(s))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())
        return {name: getattr(s, name) for name, _ in _lib.BatchStats._fields_ if name != "struct_size"}

    def decode_raw(self, items: "ctypes.Array") -> None:
        """Runs an already filled ``(_lib.GpuItem * n)`` array (pointers owned by the caller)."""
        st = _lib.load().mmr_gpu_decode_batch(self._h, items, len(items))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())

    def decode_batch(self, packets, codec=CODEC_MJPEG, output=OUTPUT_PLANAR, conceal=False):
        """Decodes a list of packets (bytes). ``codec`` / ``output`` may be per-packet lists.
        Returns ``[(BatchResult, bytes or None)]`` in packet order."""
        n = len(packets)
        codecs = codec if isinstance(codec, (list, tuple)) else [codec] * n
        outputs = output if isinstance(output, (list, tuple)) else [output] * n
        items = (_lib.GpuItem * max(n, 1))()
        keep = []
        outs = []
        for i, pkt in enumerate(packets):
            data = bytes(pkt)
            src = (ctypes.c_uint8 * max(len(data), 1)).from_buffer_copy(data or b"\0")
            keep.append(src)
            try:
                info = probe(codecs[i], data)
                need = info.rgb_bytes if outputs[i] == OUTPUT_RGB24 else info.planar_bytes
            except MmrError:
                need = 0
            dst = (ctypes.c_uint8 * max(need, 1))()
            outs.append(dst)
            it = items[i]
            it.struct_size = ctypes.sizeof(_lib.GpuItem)
            it.data = ctypes.addressof(src)
            it.len = len(data)
            it.codec = codecs[i]
            it.output = outputs[i]
            it.flags = ITEM_CONCEAL if conceal else 0
            it.out = ctypes.addressof(dst)
            it.out_capacity = need
        st = _lib.load().mmr_gpu_decode_batch(self._h, items, n)
        if st != STATUS_OK and st != INTERNAL:
            raise MmrError(st, _lib.last_error())
        res = []
        for i in range(n):
            it = items[i]
            r = BatchResult(it.status, it.message.decode("utf-8", "replace"), it.format, it.range, it.width, it.height,
                            it.plane_count, tuple(it.plane_offset), tuple(it.plane_width), tuple(it.plane_height),
                            it.out_bytes, it.concealed_segments)
            payload = ctypes.string_at(outs[i], it.out_bytes) if it.status == STATUS_OK else None
            res.append((r, payload))
        return res


    def encode_raw(self, items, quality: int = 75, annex_k: bool = False, restart_interval: int = 0) -> None:
        """``mmr_gpu_jpeg_encode_batch`` on a prepared ``(_lib.EncodeItem * n)`` array."""
        o = _lib.JpegEncodeOptions(ctypes.sizeof(_lib.JpegEncodeOptions), quality, 1 if annex_k else 0,
                                   restart_interval)
        st = _lib.load().mmr_gpu_jpeg_encode_batch(self._h, ctypes.byref(o), items, len(items))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())

    def encode_jpeg_batch(self, frames, quality: int = 75, annex_k: bool = False,
                          restart_interval: int = 0) -> list:
        """Encodes host frames in one GPU pass; (status, message, JPEG bytes or None) per frame,
        the bytes equal to :func:`encode_jpeg`'s with the same options."""
        lib = _lib.load()
        n = len(frames)
        items = (_lib.EncodeItem * n)()
        keep, outs = [], []
        for i, fr in enumerate(frames):
            it = items[i]
            it.struct_size = ctypes.sizeof(_lib.EncodeItem)
            it.frame = _view(fr, keep)
            cap = lib.mmr_gpu_jpeg_encode_bound(fr.format, fr.width, fr.height, restart_interval)
            buf = ctypes.create_string_buffer(cap)
            outs.append(buf)
            it.out = ctypes.cast(buf, ctypes.c_void_p)
            it.out_capacity = cap
        self.encode_raw(items, quality, annex_k, restart_interval)
        return [(items[i].status, items[i].message.decode("utf-8", "replace"),
                 outs[i].raw[: items[i].out_len] if items[i].status == STATUS_OK else None) for i in range(n)]

    def encode_stats(self) -> dict:
        """Device time, blocks, binary64 recomputations and bytes of the last encode batch."""
        st_ = _lib.EncodeStats()
        st_.struct_size = ctypes.sizeof(_lib.EncodeStats)
        st = _lib.load().mmr_gpu_last_encode_stats(self._h, ctypes.byref(st_))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())
        return {"device_ms": st_.device_ms, "blocks": st_.blocks, "exact_coefficients": st_.exact_coefficients,
                "bytes_out": st_.bytes_out}

    def open_stream(self, data, input_name: str = "input") -> "MediaStream":
        """Uploads a whole stream (concatenated JFIF images or raw DV frames) and frames it
        on the GPU; see :class:`MediaStream`."""
        return MediaStream(self, data, input_name)


@dataclass
class StreamOutcome:
    """What the reference CLI's ``decode`` loop ends with: ``status`` and ``message`` of its
    first error (0 and "" if none), and the frames and Y4M bytes written before it."""

    status: int
    message: str
    frames_written: int
    bytes_written: int


class MediaStream:
    """A whole MJPEG or raw DV stream framed on the GPU (``mmr_gpu_stream_*``), as the
    reference CLI's ``decode`` command frames it (crates/cli/src/main.rs:1533-1580,
    1605-1633). ``data`` is ``bytes`` or ``(address, length)`` of host memory that stays
    valid while the stream is open (pinned memory uploads fastest)."""

    def __init__(self, ctx: Context, data, input_name: str = "input"):
        lib = _lib.load()
        if isinstance(data, tuple):
            addr, n = data
        else:
            self._keep = bytes(data)
            addr, n = ctypes.cast(ctypes.c_char_p(self._keep), ctypes.c_void_p).value, len(self._keep)
        self._ctx = ctx  # the stream uses the context's engines
        info = _lib.StreamInfo()
        info.struct_size = ctypes.sizeof(_lib.StreamInfo)
        h = ctypes.c_void_p()
        st = lib.mmr_gpu_stream_open(ctx._h, addr, n, input_name.encode(), ctypes.byref(h), ctypes.byref(info))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())
        self._h = h
        self.kind = info.kind
        self.frame_status = info.frame_status
        self.frame_message = info.message.decode("utf-8", "replace")
        self.frame_count = info.frame_count
        self.y4m_bytes = info.y4m_bytes
        self.candidates = info.candidates
        self.upload_ms = info.upload_ms
        self.scan_ms = info.scan_ms

    def frames(self) -> list:
        """(offset, length) of every framed frame."""
        lib = _lib.load()
        out = []
        off, ln = ctypes.c_uint64(), ctypes.c_uint64()
        for i in range(self.frame_count):
            st = lib.mmr_gpu_stream_frame(self._h, i, ctypes.byref(off), ctypes.byref(ln))
            if st != STATUS_OK:
                raise MmrError(st, _lib.last_error())
            out.append((off.value, ln.value))
        return out

    def decode_into(self, address: int, capacity: int) -> StreamOutcome:
        """Decodes every frame and writes the Y4M stream at ``address`` (host memory of at
        least ``y4m_bytes``)."""
        r = _lib.StreamResult()
        r.struct_size = ctypes.sizeof(_lib.StreamResult)
        st = _lib.load().mmr_gpu_stream_decode_y4m(self._h, address, capacity, ctypes.byref(r))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())
        return StreamOutcome(r.status, r.message.decode("utf-8", "replace"), r.frames_written, r.bytes_written)

    def decode_y4m(self) -> tuple:
        """(:class:`StreamOutcome`, the Y4M bytes the CLI's output file holds)."""
        if not self.frame_count:
            return StreamOutcome(self.frame_status, self.frame_message, 0, 0), b""
        buf = bytearray(self.y4m_bytes)
        addr = ctypes.addressof((ctypes.c_char * len(buf)).from_buffer(buf))
        res = self.decode_into(addr, len(buf))
        return res, bytes(memoryview(buf)[: res.bytes_written])

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().mmr_gpu_stream_close(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def decode_stream_y4m(data, input_name: str = "input", ctx: Context | None = None) -> tuple:
    """The reference CLI's ``decode`` on a stream's bytes: (:class:`StreamOutcome`, Y4M bytes)."""
    own = ctx is None
    ctx = ctx or Context()
    try:
        with ctx.open_stream(data, input_name) as ms:
            return ms.decode_y4m()
    finally:
        if own:
            ctx.close()


def decode_file(input_path: str, output_path: str, ctx: Context | None = None) -> str:
    """``mmrecode decode <input> <output>`` for MJPEG and raw DV input (crates/cli/src/
    main.rs:1533-1580, 1605-1633): writes the Y4M file and returns the line the CLI prints,
    or raises :class:`MmrError` with the CLI's error after writing what it would have
    written (no file when the input is rejected before the output is created)."""
    with open(input_path, "rb") as f:
        data = f.read()
    own = ctx is None
    ctx = ctx or Context()
    try:
        with ctx.open_stream(data, str(input_path)) as ms:
            if not ms.frame_count and (ms.kind != STREAM_MJPEG or not data):
                # empty input, MPEG streams, an incomplete raw DV file: no output file
                raise MmrError(ms.frame_status, ms.frame_message)
            res, y4m = ms.decode_y4m()
            kind = ms.kind
    finally:
        if own:
            ctx.close()
    with open(output_path, "wb") as f:
        f.write(y4m)
    if res.status != STATUS_OK:
        raise MmrError(res.status, res.message)
    what = "JPEG frame(s)" if kind == STREAM_MJPEG else "raw DV frame(s)"
    return f"Decoded {res.frames_written} {what} to {output_path}"


def _result(it) -> BatchResult:
    return BatchResult(it.status, it.message.decode("utf-8", "replace"), it.format, it.range, it.width, it.height,
                       it.plane_count, tuple(it.plane_offset), tuple(it.plane_width), tuple(it.plane_height),
                       it.out_bytes, it.concealed_segments)


class Server:
    """Continuous-batching decode server (``mmr_gpu_server_*``).

    ``submit`` queues one packet and returns a ticket at once; the packet bytes and
    the output buffer are kept alive here until ``wait`` returns that ticket."""

    def __init__(self, device: int = 0, engines: int = 0, max_batch: int = 0, memory_budget: int = 0):
        lib = _lib.load()
        cfg = _lib.ServerConfig(ctypes.sizeof(_lib.ServerConfig), device, engines, max_batch, 0, memory_budget)
        h = ctypes.c_void_p()
        st = lib.mmr_gpu_server_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())
        self._h = h
        self._keep = {}

    def close(self):
        if getattr(self, "_h", None):
            _lib.load().mmr_gpu_server_destroy(self._h)
            self._h = None
            self._keep.clear()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, packet: bytes, codec: int = CODEC_MJPEG, output: int = OUTPUT_PLANAR, conceal: bool = False,
               out_device_ptr: int = 0, out_capacity: int = 0) -> int:
        """Queues a packet; output goes to a host buffer sized from the headers, or to
        ``out_device_ptr`` (device memory of ``out_capacity`` bytes) when given."""
        data = bytes(packet)
        src = (ctypes.c_uint8 * max(len(data), 1)).from_buffer_copy(data or b"\0")
        it = _lib.GpuItem()
        it.struct_size = ctypes.sizeof(_lib.GpuItem)
        it.data = ctypes.addressof(src)
        it.len = len(data)
        it.codec = codec
        it.output = output
        it.flags = (ITEM_CONCEAL if conceal else 0) | (ITEM_OUT_DEVICE if out_device_ptr else 0)
        dst = None
        if out_device_ptr:
            it.out = out_device_ptr
            it.out_capacity = out_capacity
        else:
            try:
                info = probe(codec, data)
                need = info.rgb_bytes if output == OUTPUT_RGB24 else info.planar_bytes
            except MmrError:
                need = 0
            dst = (ctypes.c_uint8 * max(need, 1))()
            it.out = ctypes.addressof(dst)
            it.out_capacity = need
        t = ctypes.c_uint64()
        st = _lib.load().mmr_gpu_server_submit(self._h, ctypes.byref(it), ctypes.byref(t))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())
        self._keep[t.value] = (src, dst)
        return t.value

    def submit_item(self, item) -> int:
        """Queues a prebuilt ``_lib.GpuItem`` (its buffers are the caller's to keep alive)."""
        t = ctypes.c_uint64()
        st = _lib.load().mmr_gpu_server_submit(self._h, ctypes.byref(item), ctypes.byref(t))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())
        return t.value

    def wait_item(self, ticket: int, result, timeout_s: float | None = None) -> float:
        """Waits for a ticket from ``submit_item``; fills ``result`` (a ``_lib.GpuItem``); returns the latency in ms."""
        lat = ctypes.c_double()
        ns = -1 if timeout_s is None else int(timeout_s * 1e9)
        st = _lib.load().mmr_gpu_server_wait(self._h, ticket, ns, ctypes.byref(result), ctypes.byref(lat))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())
        return lat.value

    def wait(self, ticket: int, timeout_s: float | None = None):
        """(BatchResult, payload bytes or None, latency ms); raises MmrError(INVALID_STATE) on timeout."""
        it = _lib.GpuItem()
        it.struct_size = ctypes.sizeof(_lib.GpuItem)
        lat = ctypes.c_double()
        ns = -1 if timeout_s is None else int(timeout_s * 1e9)
        st = _lib.load().mmr_gpu_server_wait(self._h, ticket, ns, ctypes.byref(it), ctypes.byref(lat))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())
        src, dst = self._keep.pop(ticket)
        r = _result(it)
        payload = ctypes.string_at(dst, it.out_bytes) if (dst is not None and it.status == STATUS_OK) else None
        return r, payload, lat.value

    def replay(self, items, arrival_s) -> tuple:
        """Open-loop replay of a ``(_lib.GpuItem * n)`` array at the given arrival
        offsets (seconds, non-decreasing), natively; returns (latencies ms, max
        submission lag ms). Results land in ``items``."""
        n = len(items)
        arr = (ctypes.c_int64 * n)(*[int(t * 1e9) for t in arrival_s])
        lat = (ctypes.c_double * n)()
        lag = ctypes.c_int64()
        st = _lib.load().mmr_gpu_server_replay(self._h, items, n, arr, lat, ctypes.byref(lag))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())
        return list(lat), lag.value / 1e6

    def stats(self, reset: bool = False) -> dict:
        s = _lib.ServerStats()
        s.struct_size = ctypes.sizeof(_lib.ServerStats)
        st = _lib.load().mmr_gpu_server_stats_get(self._h, 1 if reset else 0, ctypes.byref(s))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())
        return {name: getattr(s, name) for name, _ in _lib.ServerStats._fields_ if name != "struct_size"}

    def set_tuning(self, table) -> None:
        """Installs an autotuner table (``Context.autotune``'s list or ``load_tuning``'s) on
        the server's engines."""
        arr = _tune_entries(table)
        st = _lib.load().mmr_gpu_server_set_tuning(self._h, arr, len(table))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())

    def set_slice_bits(self, bits: int) -> None:
        st = _lib.load().mmr_gpu_server_set_slice_bits(self._h, bits)
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())


def frame_from_batch(r: BatchResult, payload: bytes) -> VideoFrame:
    planes = []
    for c in range(r.plane_count):
        off, w, h = r.plane_offset[c], r.plane_width[c], r.plane_height[c]
        planes.append(Plane(payload[off:off + w * h], w, w, h))
    return VideoFrame(r.format, r.width, r.height, planes, r.range)


class _GpuDecoder:
    """Decoder trait (crates/core/src/codec.rs:102-130) over the GPU library."""

    codec_name = ""
    codec = 0
    kind = ""

    def __init__(self, batch: int = 1, context: Context | None = None):
        if batch < 1:
            raise ValueError("batch must be at least 1")
        self._configured = False
        self._frames = collections.deque()
        self._pending: list[Packet] = []
        self._batch = batch
        self._ctx = context

    def configure(self, descriptor: CodecDescriptor) -> None:
        self._check_descriptor(descriptor)
        self._frames.clear()
        self._pending.clear()
        self._configured = True

    def _require(self, what: str) -> None:
        if not self._configured:
            raise MmrError(INVALID_STATE, f"invalid state: {self.kind} decoder must be configured before {what}")

    def send_packet(self, packet: Packet) -> None:
        self._require("receiving packets")
        if self._batch == 1:
            frame = self._decode_single(packet.data)
            frame.pts, frame.duration = packet.pts, packet.duration
            self._frames.append(frame)
            return
        self._pending.append(packet)
        if len(self._pending) >= self._batch:
            self._run_pending()

    def receive_frame(self):
        self._require("receiving frames")
        if not self._frames:
            return None
        item = self._frames.popleft()
        if isinstance(item, MmrError):
            raise item
        return item

    def flush(self) -> None:
        self._require("flushing")
        if self._pending:
            self._run_pending()

    def _run_pending(self) -> None:
        if self._ctx is None:
            self._ctx = Context()
        packets, self._pending = self._pending, []
        for pkt, (r, payload) in zip(packets, self._ctx.decode_batch([p.data for p in packets], self.codec)):
            if r.status != STATUS_OK:
                self._frames.append(MmrError(r.status, r.message))
                continue
            frame = frame_from_batch(r, payload)
            frame.pts, frame.duration = pkt.pts, pkt.duration
            self._frames.append(frame)


class MjpegDecoder(_GpuDecoder):
    """MjpegDecoder (crates/codecs/mjpeg/src/codec.rs:16-71) decoding on the GPU."""

    codec_name = MJPEG_CODEC_NAME
    codec = CODEC_MJPEG
    kind = "Motion JPEG"

    def _check_descriptor(self, d: CodecDescriptor) -> None:
        if d.codec_id != MJPEG_CODEC_NAME:
            raise MmrError(INVALID_DATA, f"invalid data: expected {MJPEG_CODEC_NAME}, received {d.codec_id}")
        if d.media_type != "video":
            raise MmrError(INVALID_DATA, "invalid data: Motion JPEG decoder requires a video stream descriptor")

    def _decode_single(self, data: bytes) -> VideoFrame:
        return decode_jpeg(data)


class DvDecoder(_GpuDecoder):
    """DvDecoder (crates/codecs/dv/src/codec.rs:16-66) decoding on the GPU."""

    codec_name = DV_CODEC_NAME
    codec = CODEC_DV
    kind = "DV"

    def _check_descriptor(self, d: CodecDescriptor) -> None:
        if d.codec_id != DV_CODEC_NAME or d.media_type != "video":
            raise MmrError(INVALID_DATA, "invalid data: DV decoder requires a video/dv video descriptor")

    def _decode_single(self, data: bytes) -> VideoFrame:
        return decode_dv(data)


class DecoderSession:
    """The C session API (``mmr_gpu_decoder_*``): the Decoder trait
    (crates/core/src/codec.rs:102-130) with packets queued on a server that every
    session of the process shares. ``send_packet`` returns at once; a packet's decode
    error is raised by the ``receive_frame`` that reaches it (``MmrError.tag`` is the
    packet's tag)."""

    def __init__(self, codec: int, device_frames: bool = False):
        lib = _lib.load()
        h = ctypes.c_void_p()
        st = lib.mmr_gpu_decoder_create(codec, ctypes.byref(h))
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())
        self._h = h  # send_packet copies each packet: the caller's bytes need not stay alive
        if device_frames:
            self._check(lib.mmr_gpu_decoder_set_output(h, SESSION_DEVICE_FRAMES))

    def close(self) -> None:
        """Waits for the packets still being decoded and frees the session."""
        h = getattr(self, "_h", None)
        if h:
            self._h = None
            _lib.load().mmr_gpu_decoder_destroy(h)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()

    def _check(self, st: int) -> None:
        if st != STATUS_OK:
            raise MmrError(st, _lib.last_error())

    def configure(self, descriptor: CodecDescriptor) -> None:
        self._check(_lib.load().mmr_gpu_decoder_configure(self._h, descriptor.codec_id.encode(),
                                                           descriptor.media_type.encode()))

    def send_packet(self, data: bytes, tag: int = 0) -> None:
        buf = bytes(data)
        self._check(_lib.load().mmr_gpu_decoder_send_packet(self._h, buf, len(buf), tag))

    def receive_frame(self, wait_ns: int = -1):
        """(frame, tag), or None when nothing is queued or the oldest packet is not
        decoded within wait_ns (< 0: wait without limit)."""
        lib = _lib.load()
        fr = _lib.VideoFrameC()
        fr.struct_size = ctypes.sizeof(_lib.VideoFrameC)
        tag, has = ctypes.c_uint64(0), ctypes.c_int(0)
        st = lib.mmr_gpu_decoder_receive_frame(self._h, wait_ns, ctypes.byref(fr), ctypes.byref(tag), ctypes.byref(has))
        if st != STATUS_OK:
            e = MmrError(st, _lib.last_error())
            e.tag = tag.value
            raise e
        if not has.value:
            return None
        try:
            return _frame_from_c(fr), tag.value
        finally:
            lib.mmr_video_frame_free(ctypes.byref(fr))

    def flush(self) -> None:
        self._check(_lib.load().mmr_gpu_decoder_flush(self._h))

    def receive_device_frame(self, wait_ns: int = -1):
        """For a session made with ``device_frames=True``: (DeviceFrame, tag), or None
        as for ``receive_frame``. Release the frame when done with its planes."""
        fr = _lib.DeviceFrame()
        fr.struct_size = ctypes.sizeof(_lib.DeviceFrame)
        tag, has = ctypes.c_uint64(0), ctypes.c_int(0)
        st = _lib.load().mmr_gpu_decoder_receive_device_frame(self._h, wait_ns, ctypes.byref(fr), ctypes.byref(tag),
                                                              ctypes.byref(has))
        if st != STATUS_OK:
            e = MmrError(st, _lib.last_error())
            e.tag = tag.value
            raise e
        if not has.value:
            return None
        return DeviceFrame(fr), tag.value


class DeviceFrame:
    """A session's frame in device memory (device 0): ``planes`` lists (device address,
    width, height) per plane, stride = width. ``release()`` hands the buffer back."""

    def __init__(self, raw: "_lib.DeviceFrame"):
        self._raw = raw
        self.format, self.range, self.width, self.height = raw.format, raw.range, raw.width, raw.height
        self.planes = [(raw.planes[c], raw.plane_width[c], raw.plane_height[c]) for c in range(raw.plane_count)]

    def release(self) -> None:
        if self._raw is not None:
            _lib.load().mmr_gpu_device_frame_release(ctypes.byref(self._raw))
            self._raw = None
            self.planes = []

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.release()
