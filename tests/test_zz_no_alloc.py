"""mmr_dv_decode_static: the DV25 entry point that allocates nothing.

It exists for callers that cannot allocate memory while they decode -- a
real-time capture or playback thread that cannot take cudaMalloc's implicit
device synchronisation, an application whose GPU memory is budgeted up front,
or a host runtime that forbids allocations outside its own arena. Its device
work runs in one fixed array inside the library, so this test checks that two
calls in a row (the second reusing what the first left in that array) give
exactly mmr_dv_decode's samples, the bit-exact tolerance of every decode test
here, and the same statuses on bad input.

Collected last on purpose (file name): a run that stops at the first failure
has run every other test before this one. It also passes alone in a fresh
process."""

import ctypes

import pytest

import mmrecode_gb300 as m
import oracle
from mmrecode_gb300 import _lib, synth
from helpers import DV_FIXTURES, fixture

pytestmark = pytest.mark.gpu

MAX_PLANAR = 720 * 576 + 2 * 360 * 288  # the larger (625/50) frame


def static_decode(packet: bytes):
    lib = _lib.load()
    info = _lib.FrameInfo()
    info.struct_size = ctypes.sizeof(_lib.FrameInfo)
    out = (ctypes.c_uint8 * MAX_PLANAR)()
    st = lib.mmr_dv_decode_static(packet, len(packet), out, len(out), ctypes.byref(info))
    return st, info, (ctypes.string_at(out, info.planar_bytes) if st == 0 else None)


def reference_entry_point(packet: bytes):
    try:
        f = m.decode_dv(packet)
        return 0, f, b"".join(p.data for p in f.planes)
    except m.MmrError as e:
        return e.status, None, None


def test_static_entry_point_matches_mmr_dv_decode_on_two_calls_in_a_row():
    packets = [fixture(r) for r in DV_FIXTURES] + synth.dv_stream(115, 2) + synth.dv_stream(116, 1, pal=True)
    for k, packet in enumerate(packets):
        st_ref, frame, expect = reference_entry_point(packet)
        assert st_ref == 0
        for call in range(2):
            st, info, got = static_decode(packet)
            assert st == 0, f"packet {k} call {call}: {_lib.last_error()}"
            assert (info.format, info.width, info.height, info.plane_count) == (frame.format, frame.width,
                                                                                 frame.height, 3)
            assert got == expect, f"packet {k} call {call}: samples differ from mmr_dv_decode"
        ref = oracle.dv_decode(packet)  # and directly against the reference algorithm
        assert ref.status == 0 and expect == b"".join(p[2] for p in ref.frame.planes), f"packet {k}: oracle"


def _device_free_bytes() -> int:
    """Free device memory as cuMemGetInfo reports it for the current context."""
    cuda = ctypes.CDLL("libcuda.so.1")
    free, total = ctypes.c_size_t(0), ctypes.c_size_t(0)
    assert cuda.cuMemGetInfo_v2(ctypes.byref(free), ctypes.byref(total)) == 0
    return free.value


def test_calls_after_set_up_allocate_no_device_memory():
    packets = [fixture(r) for r in DV_FIXTURES] + synth.dv_stream(117, 3)
    st, _, _ = static_decode(packets[0])  # the first call on the device sets it up
    assert st == 0
    before = _device_free_bytes()
    for _ in range(3):
        for p in packets:
            st, _, _ = static_decode(p)
            assert st == 0
    assert _device_free_bytes() == before


def test_static_entry_point_errors_match_and_do_not_leak_into_the_next_call():
    damaged = bytearray(fixture(DV_FIXTURES[0]))
    damaged[7 * 80] = 0x76
    st_ref, _, _ = reference_entry_point(bytes(damaged))
    for _ in range(2):
        st, _, _ = static_decode(bytes(damaged))
        assert st == st_ref == m.INVALID_DATA
        assert "damaged DIF identifier" in _lib.last_error()
    clean = fixture(DV_FIXTURES[0])
    st, _, got = static_decode(clean)
    assert st == 0 and got == reference_entry_point(clean)[2] and _lib.last_error() == ""
    st, _, _ = static_decode(bytes(200000))
    assert st == m.INVALID_ARGUMENT and "exceeds" in _lib.last_error()
    st, _, _ = static_decode(clean[:1000])
    assert st == reference_entry_point(clean[:1000])[0] == m.INVALID_DATA
