"""The decoder session API (include/mmrecode_gpu.h, mmr_gpu_decoder_*) on CPU: the
Decoder trait's states and messages as MjpegDecoder (crates/codecs/mjpeg/src/codec.rs:16-71)
and DvDecoder (crates/codecs/dv/src/codec.rs:16-66) give them, and the C ABI's argument
checks. None of these calls reaches the GPU: the shared server is created by the first
packet a configured session accepts."""
import ctypes

import pytest

import mmrecode_gb300 as m
from mmrecode_gb300 import _lib

KINDS = [(m.CODEC_MJPEG, "Motion JPEG", "video/mjpeg"), (m.CODEC_DV, "DV", "video/dv")]


def create(codec):
    h = ctypes.c_void_p()
    assert _lib.load().mmr_gpu_decoder_create(codec, ctypes.byref(h)) == m.STATUS_OK
    assert h.value
    return h


def frame():
    fr = _lib.VideoFrameC()
    fr.struct_size = ctypes.sizeof(_lib.VideoFrameC)
    return fr


def receive(h, fr=None, wait_ns=0):
    fr = fr if fr is not None else frame()
    tag, has = ctypes.c_uint64(7), ctypes.c_int(9)
    st = _lib.load().mmr_gpu_decoder_receive_frame(h, wait_ns, ctypes.byref(fr), ctypes.byref(tag), ctypes.byref(has))
    return st, has.value, tag.value


def test_create_checks_its_arguments():
    lib = _lib.load()
    h = ctypes.c_void_p(1)
    assert lib.mmr_gpu_decoder_create(99, ctypes.byref(h)) == m.INVALID_ARGUMENT
    assert h.value is None  # the handle is cleared on failure
    assert lib.mmr_gpu_decoder_create(m.CODEC_MJPEG, None) == m.INVALID_ARGUMENT
    lib.mmr_gpu_decoder_destroy(None)  # NULL is ignored


@pytest.mark.parametrize("codec,kind,name", KINDS)
def test_every_call_needs_configure(codec, kind, name):
    lib = _lib.load()
    h = create(codec)
    try:
        assert lib.mmr_gpu_decoder_send_packet(h, b"\xff\xd8", 2, 1) == m.INVALID_STATE
        assert _lib.last_error() == f"invalid state: {kind} decoder must be configured before receiving packets"
        st, has, _ = receive(h)
        assert (st, has) == (m.INVALID_STATE, 0)
        assert _lib.last_error() == f"invalid state: {kind} decoder must be configured before receiving frames"
        assert lib.mmr_gpu_decoder_flush(h) == m.INVALID_STATE
        assert _lib.last_error() == f"invalid state: {kind} decoder must be configured before flushing"
    finally:
        lib.mmr_gpu_decoder_destroy(h)


def test_configure_checks_the_descriptor():
    lib = _lib.load()
    h = create(m.CODEC_MJPEG)
    try:
        assert lib.mmr_gpu_decoder_configure(h, b"video/dv", b"video") == m.INVALID_DATA
        assert _lib.last_error() == "invalid data: expected video/mjpeg, received video/dv"
        assert lib.mmr_gpu_decoder_configure(h, b"video/mjpeg", b"audio") == m.INVALID_DATA
        assert _lib.last_error() == "invalid data: Motion JPEG decoder requires a video stream descriptor"
        assert lib.mmr_gpu_decoder_configure(h, None, b"video") == m.INVALID_ARGUMENT
        # a failed configure leaves the session unconfigured
        assert lib.mmr_gpu_decoder_flush(h) == m.INVALID_STATE
        assert lib.mmr_gpu_decoder_configure(h, b"video/mjpeg", b"video") == m.STATUS_OK
        assert _lib.last_error() == ""
    finally:
        lib.mmr_gpu_decoder_destroy(h)
    h = create(m.CODEC_DV)
    try:
        for cid, mt in ((b"video/mjpeg", b"video"), (b"video/dv", b"audio")):
            assert lib.mmr_gpu_decoder_configure(h, cid, mt) == m.INVALID_DATA
            assert _lib.last_error() == "invalid data: DV decoder requires a video/dv video descriptor"
        assert lib.mmr_gpu_decoder_configure(h, b"video/dv", b"video") == m.STATUS_OK
    finally:
        lib.mmr_gpu_decoder_destroy(h)


@pytest.mark.parametrize("codec,kind,name", KINDS)
def test_configured_session_with_nothing_queued(codec, kind, name):
    lib = _lib.load()
    h = create(codec)
    try:
        assert lib.mmr_gpu_decoder_configure(h, name.encode(), b"video") == m.STATUS_OK
        fr = frame()
        fr.width = 5  # reset to empty by the call
        st, has, tag = receive(h, fr)
        assert (st, has, tag) == (m.STATUS_OK, 0, 7)  # the reference's Ok(None); the tag is left alone
        assert fr.width == 0 and fr.plane_count == 0 and fr.struct_size == ctypes.sizeof(_lib.VideoFrameC)
        assert lib.mmr_gpu_decoder_flush(h) == m.STATUS_OK
        # a null packet with a length, and a frame of another struct size, are refused
        assert lib.mmr_gpu_decoder_send_packet(h, None, 10, 1) == m.INVALID_ARGUMENT
        assert _lib.last_error() == "invalid argument: data is null while length is nonzero"
        bad = frame()
        bad.struct_size = 8
        bad.width = 5
        st, has, _ = receive(h, bad)
        assert (st, has) == (m.INVALID_ARGUMENT, 0)
        assert bad.width == 5 and bad.struct_size == 8  # left untouched (lib.rs:604-610)
        tag, has_c = ctypes.c_uint64(), ctypes.c_int()
        assert lib.mmr_gpu_decoder_receive_frame(h, 0, None, ctypes.byref(tag), ctypes.byref(has_c)) == \
            m.INVALID_ARGUMENT
        assert lib.mmr_gpu_decoder_receive_frame(h, 0, ctypes.byref(frame()), None, None) == m.INVALID_ARGUMENT
    finally:
        lib.mmr_gpu_decoder_destroy(h)


def test_python_session_mirror_states():
    with m.DecoderSession(m.CODEC_DV) as s:
        with pytest.raises(m.MmrError) as e:
            s.send_packet(b"\x00" * 16)
        assert e.value.status == m.INVALID_STATE
        with pytest.raises(m.MmrError) as e:
            s.configure(m.CodecDescriptor("video/mjpeg"))
        assert e.value.message == "invalid data: DV decoder requires a video/dv video descriptor"
        s.configure(m.CodecDescriptor(m.DV_CODEC_NAME))
        assert s.receive_frame(0) is None
        s.flush()
    with pytest.raises(m.MmrError) as e:
        m.DecoderSession(0)
    assert e.value.status == m.INVALID_ARGUMENT


def device_frame():
    fr = _lib.DeviceFrame()
    fr.struct_size = ctypes.sizeof(_lib.DeviceFrame)
    return fr


def test_device_frame_output_states():
    lib = _lib.load()
    h = create(m.CODEC_MJPEG)
    try:
        assert lib.mmr_gpu_decoder_set_output(h, 2) == m.INVALID_ARGUMENT
        assert lib.mmr_gpu_decoder_set_output(None, 1) == m.INVALID_ARGUMENT
        assert lib.mmr_gpu_decoder_configure(h, b"video/mjpeg", b"video") == m.STATUS_OK
        tag, has = ctypes.c_uint64(3), ctypes.c_int(9)
        # host frames by default: the device call is the wrong one
        fr = device_frame()
        fr.width = 5
        assert lib.mmr_gpu_decoder_receive_device_frame(h, 0, ctypes.byref(fr), ctypes.byref(tag),
                                                        ctypes.byref(has)) == m.INVALID_STATE
        assert _lib.last_error() == "invalid state: the session delivers host frames (mmr_gpu_decoder_receive_frame)"
        assert has.value == 0 and fr.width == 0  # reset
        assert lib.mmr_gpu_decoder_set_output(h, m.SESSION_DEVICE_FRAMES) == m.STATUS_OK
        st, has_frame, _ = receive(h)
        assert (st, has_frame) == (m.INVALID_STATE, 0)
        assert _lib.last_error() == \
            "invalid state: the session delivers device frames (mmr_gpu_decoder_receive_device_frame)"
        fr = device_frame()
        assert lib.mmr_gpu_decoder_receive_device_frame(h, 0, ctypes.byref(fr), ctypes.byref(tag),
                                                        ctypes.byref(has)) == m.STATUS_OK
        assert has.value == 0 and tag.value == 3 and not fr.buffer  # nothing queued: Ok(None)
        bad = device_frame()
        bad.struct_size = 16
        bad.width = 5
        assert lib.mmr_gpu_decoder_receive_device_frame(h, 0, ctypes.byref(bad), ctypes.byref(tag),
                                                        ctypes.byref(has)) == m.INVALID_ARGUMENT
        assert bad.width == 5  # untouched
        assert lib.mmr_gpu_decoder_receive_device_frame(h, 0, None, ctypes.byref(tag),
                                                        ctypes.byref(has)) == m.INVALID_ARGUMENT
        # release: NULL, an empty frame and a frame of another size are ignored
        lib.mmr_gpu_device_frame_release(None)
        lib.mmr_gpu_device_frame_release(ctypes.byref(fr))
        lib.mmr_gpu_device_frame_release(ctypes.byref(bad))
        assert bad.width == 5 and fr.struct_size == ctypes.sizeof(_lib.DeviceFrame)
    finally:
        lib.mmr_gpu_decoder_destroy(h)
    with m.DecoderSession(m.CODEC_DV, device_frames=True) as s:
        s.configure(m.CodecDescriptor(m.DV_CODEC_NAME))
        assert s.receive_device_frame(0) is None
        with pytest.raises(m.MmrError) as e:
            s.receive_frame(0)
        assert e.value.status == m.INVALID_STATE
