"""Decoder sessions (mmr_gpu_decoder_*, the Decoder trait of crates/core/src/codec.rs:102-130
over a server shared by the process) on the GPU against the oracle: every frame's samples,
every failed packet's status and message, tags and send order; packets received one by one
and drained after a flush; two sessions of both codecs interleaved on the shared server;
configure discarding queued packets; destroy with packets still queued; frames left in
device memory (read back through torch), released one by one and held together."""
import pytest

import mmrecode_gb300 as m
import oracle
from helpers import DV_FIXTURES, assert_same_decode, fixture, frame_planes_gpu, prefixed
from mmrecode_gb300 import _lib, synth

pytestmark = pytest.mark.gpu


def oracle_of(codec, packet):
    return oracle.jpeg_decode(packet) if codec == m.CODEC_MJPEG else oracle.dv_decode(packet)


def mjpeg_packets():
    pk = synth.mjpeg_stream(611, 5, 96, 64, "422", 85, 4, annex_k=True)
    bad = bytearray(pk[3])
    bad[len(bad) // 2:len(bad) // 2 + 8] = b"\xff\xd0" * 4  # restart markers out of order
    return pk[:2] + [b"", pk[2][:len(pk[2]) // 2], bytes(bad)] + pk[2:]


def dv_packets():
    pk = synth.dv_stream(612, 3) + [fixture(rel) for rel in DV_FIXTURES]
    return pk[:2] + [pk[0][:1000], b"\x00" * 120000] + pk[2:]


def check(codec, packet, got, label):
    ref = oracle_of(codec, packet)
    if isinstance(got, m.MmrError):
        assert_same_decode(got.status, got.message, [], ref, label)
        assert got.message == prefixed(ref.status, ref.message), label
    else:
        assert_same_decode(0, "", frame_planes_gpu(got), ref, label)
    return ref.status


def receive(session, wait_ns):
    try:
        r = session.receive_frame(wait_ns)
    except m.MmrError as e:
        return e, e.tag
    return (None, None) if r is None else r


def session(codec):
    s = m.DecoderSession(codec)
    s.configure(m.CodecDescriptor(m.MJPEG_CODEC_NAME if codec == m.CODEC_MJPEG else m.DV_CODEC_NAME))
    return s


@pytest.mark.parametrize("codec", [m.CODEC_MJPEG, m.CODEC_DV], ids=["mjpeg", "dv"])
def test_send_then_receive_each(codec):
    packets = mjpeg_packets() if codec == m.CODEC_MJPEG else dv_packets()
    statuses = []
    with session(codec) as s:
        for i, p in enumerate(packets):
            s.send_packet(p, 100 + i)
            got, tag = receive(s, -1)
            assert tag == 100 + i
            statuses.append(check(codec, p, got, f"packet {i}"))
            assert receive(s, 0) == (None, None)
    assert 0 in statuses and any(statuses)  # frames and failures both


@pytest.mark.parametrize("codec", [m.CODEC_MJPEG, m.CODEC_DV], ids=["mjpeg", "dv"])
def test_queue_flush_drain(codec):
    packets = (mjpeg_packets() if codec == m.CODEC_MJPEG else dv_packets()) * 3
    with session(codec) as s:
        for i, p in enumerate(packets):
            s.send_packet(p, i)
        s.flush()
        for i, p in enumerate(packets):
            got, tag = receive(s, 0)  # every packet is decoded after the flush
            assert tag == i
            check(codec, p, got, f"packet {i}")
        assert receive(s, 0) == (None, None)


def test_sessions_share_the_server():
    jp, dv = mjpeg_packets(), dv_packets()
    a, b = session(m.CODEC_MJPEG), session(m.CODEC_DV)
    try:
        for i in range(max(len(jp), len(dv))):
            if i < len(jp):
                a.send_packet(jp[i], i)
            if i < len(dv):
                b.send_packet(dv[i], 1000 + i)
        for i, p in enumerate(dv):  # the second session first
            got, tag = receive(b, -1)
            assert tag == 1000 + i
            check(m.CODEC_DV, p, got, f"dv {i}")
        for i, p in enumerate(jp):
            got, tag = receive(a, -1)
            assert tag == i
            check(m.CODEC_MJPEG, p, got, f"mjpeg {i}")
    finally:
        a.close()
        b.close()


def test_configure_discards_and_destroy_waits():
    jp = mjpeg_packets()
    s = session(m.CODEC_MJPEG)
    for i, p in enumerate(jp):
        s.send_packet(p, i)
    s.configure(m.CodecDescriptor(m.MJPEG_CODEC_NAME))  # reference: frames.clear()
    assert receive(s, -1) == (None, None)
    s.send_packet(jp[0], 5)
    got, tag = receive(s, -1)
    assert tag == 5
    check(m.CODEC_MJPEG, jp[0], got, "after configure")
    for i, p in enumerate(jp):
        s.send_packet(p, i)
    s.close()  # packets still on the GPU: destroy waits for them


class _DevicePlane:
    """A device plane as a CUDA array (read through torch)."""

    def __init__(self, ptr, n):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "|u1", "data": (ptr, False), "version": 2}


def device_planes(torch, frame):
    return [(w, h, torch.as_tensor(_DevicePlane(ptr, w * h), device="cuda").cpu().numpy().tobytes())
            for ptr, w, h in frame.planes]


@pytest.mark.parametrize("codec", [m.CODEC_MJPEG, m.CODEC_DV], ids=["mjpeg", "dv"])
def test_device_frames(codec):
    torch = pytest.importorskip("torch")
    packets = (mjpeg_packets() if codec == m.CODEC_MJPEG else dv_packets()) * 2
    s = m.DecoderSession(codec, device_frames=True)
    s.configure(m.CodecDescriptor(m.MJPEG_CODEC_NAME if codec == m.CODEC_MJPEG else m.DV_CODEC_NAME))
    try:
        half = len(packets) // 2
        for i, p in enumerate(packets[:half]):  # one by one: buffers are reused after release
            s.send_packet(p, i)
            try:
                got = s.receive_device_frame(-1)
            except m.MmrError as e:
                assert e.tag == i
                check(codec, p, e, f"packet {i}")
                continue
            frame, tag = got
            assert tag == i
            with frame:
                ref = oracle_of(codec, p)
                assert_same_decode(0, "", device_planes(torch, frame), ref, f"packet {i}")
                assert (frame.format, frame.width, frame.height) == (ref.frame.format, ref.frame.width,
                                                                     ref.frame.height)
        for i, p in enumerate(packets[half:], half):
            s.send_packet(p, i)
        # the output changes only with nothing queued
        assert _lib.load().mmr_gpu_decoder_set_output(s._h, m.SESSION_HOST_FRAMES) == m.INVALID_STATE
        s.flush()
        held = []
        for i, p in enumerate(packets[half:], half):  # held frames keep distinct buffers
            try:
                frame, tag = s.receive_device_frame(0)
            except m.MmrError as e:
                check(codec, p, e, f"packet {i}")
                continue
            assert tag == i
            held.append((p, frame))
        for i, (p, frame) in enumerate(held):
            assert_same_decode(0, "", device_planes(torch, frame), oracle_of(codec, p), f"held {i}")
            frame.release()
        assert s.receive_device_frame(0) is None
        for i, p in enumerate(packets[:3]):
            s.send_packet(p, i)
    finally:
        s.close()  # with packets queued: their buffers go back to the pool
