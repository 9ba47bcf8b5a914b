"""Pooled batches with payloads in host memory go through device staging: each
chunk uploads its inputs, decodes device-resident (as a graph once it repeats)
and downloads its outputs while the engine takes the next chunk. Statuses,
error messages and outputs must equal the one-engine path (no staging) and the
oracle, call after call. (A failed item's buffer holds no result on either
path; its content is not compared.)"""

import ctypes

import pytest

import mmrecode_gb300 as m
import oracle
from mmrecode_gb300 import _lib, synth

pytestmark = pytest.mark.gpu

SENTINEL = 0xAB


def _packets():
    pk = [(p, m.CODEC_MJPEG, m.OUTPUT_RGB24) for p in synth.mjpeg_stream(701, 14, 640, 360, "422", 85, 40)]
    pk += [(p, m.CODEC_MJPEG, m.OUTPUT_PLANAR) for p in synth.mjpeg_stream(702, 10, 320, 240, "420", 75, 0)]
    pk += [(p, m.CODEC_MJPEG, m.OUTPUT_RGB24) for p in synth.mjpeg_stream(703, 6, 176, 144, "444", 60, 3)]
    pk += [(p, m.CODEC_DV, m.OUTPUT_PLANAR) for p in synth.dv_stream(704, 4)]
    pk += [(p, m.CODEC_DV, m.OUTPUT_RGB24) for p in synth.dv_stream(705, 2)]
    bad = bytearray(pk[3][0])
    bad[len(bad) // 2] ^= 0x5A
    bad[len(bad) // 2 + 1] = 0xFF
    pk.append((bytes(bad), m.CODEC_MJPEG, m.OUTPUT_RGB24))
    pk.append((pk[-3][0][:4000], m.CODEC_DV, m.OUTPUT_PLANAR))  # wrong DV length
    return pk


def _need(p, codec, output):
    pr = m.probe(codec, p)
    return pr.rgb_bytes if output == m.OUTPUT_RGB24 else pr.planar_bytes


class _Batch:
    """Host inputs/outputs; items in `device` read and write device memory instead."""

    def __init__(self, torch, pk, device=(), small=()):
        self.pk = pk
        self.keep, self.outs = [], []
        self.arr = (_lib.GpuItem * len(pk))()
        for i, (p, codec, output) in enumerate(pk):
            src = (ctypes.c_uint8 * len(p)).from_buffer_copy(p)
            need = max(_need(p, codec, output), 64)
            cap = need // 2 if i in small else need
            it = self.arr[i]
            it.struct_size = ctypes.sizeof(_lib.GpuItem)
            it.data, it.len, it.codec, it.output = ctypes.addressof(src), len(p), codec, output
            if i in device:
                din = torch.frombuffer(bytearray(p), dtype=torch.uint8).cuda()
                dout = torch.full((cap,), SENTINEL, dtype=torch.uint8, device="cuda")
                self.keep.append((src, din))
                it.device_data = din.data_ptr()
                it.flags = m.ITEM_OUT_DEVICE
                it.out = dout.data_ptr()
                self.outs.append(dout)
            else:
                dst = (ctypes.c_uint8 * cap)(*([SENTINEL] * cap))
                self.keep.append((src, dst))
                it.out = ctypes.addressof(dst)
                self.outs.append(dst)
            it.out_capacity = cap

    def reset(self):
        for o in self.outs:
            if isinstance(o, ctypes.Array):
                ctypes.memset(o, SENTINEL, len(o))
            else:
                o.fill_(SENTINEL)

    def payload(self, i):
        o = self.outs[i]
        return bytes(o) if isinstance(o, ctypes.Array) else o.cpu().numpy().tobytes()

    def result(self, i):
        it = self.arr[i]
        return it.status, it.message, it.out_bytes, self.payload(i)


def _oracle(p, codec, output):
    ref = oracle.jpeg_decode(p) if codec == m.CODEC_MJPEG else oracle.dv_decode(p, False)
    if ref.status:
        return ref.status, None
    return 0, oracle.rgb24(ref.frame) if output == m.OUTPUT_RGB24 else b"".join(d for (_, _, d) in ref.frame.planes)


def test_staged_pool_matches_one_engine_and_oracle_across_calls():
    torch = pytest.importorskip("torch")
    pk = _packets()
    assert len(pk) >= 2 * 16  # the pool splits it into chunks
    device, small = {1, 17, 31}, {5}
    ref = _Batch(torch, pk, device, small)
    with m.Context(engines=1) as one:
        one.decode_raw(ref.arr)
    expected = [ref.result(i) for i in range(len(pk))]
    for i, (p, codec, output) in enumerate(pk):
        st, payload = _oracle(p, codec, output)
        if i in small:
            assert expected[i][0] != 0
            continue
        assert expected[i][0] == st, (i, expected[i][1])
        if st == 0:
            assert expected[i][3][:expected[i][2]] == payload, i
    b = _Batch(torch, pk, device, small)
    with m.Context(engines=3) as pool:
        for call in range(4):  # the third and fourth calls replay the chunks' graphs
            b.reset()
            pool.decode_raw(b.arr)
            for i in range(len(pk)):
                got = b.result(i)
                assert got[:3] == expected[i][:3], (call, i, b.arr[i].message)
                if got[0] == 0:
                    assert got[3] == expected[i][3], (call, i)
            if call >= 2:
                assert pool.stats()["graph_replays"] >= 1


def test_staged_results_follow_changed_packets():
    # same headers and lengths, different entropy-coded bytes: replayed chunks
    # must decode what the host buffers hold now
    torch = pytest.importorskip("torch")
    pk = [(p, m.CODEC_MJPEG, m.OUTPUT_RGB24) for p in synth.mjpeg_stream(706, 40, 256, 192, "422", 80, 16)]
    b = _Batch(torch, pk)
    with m.Context(engines=2) as pool:
        for _ in range(3):
            pool.decode_raw(b.arr)
        for i, (p, codec, output) in enumerate(pk):
            d = bytearray(p)
            sos = d.index(b"\xff\xda")
            pos = sos + 2 + (d[sos + 2] << 8 | d[sos + 3]) + 30
            d[pos] = d[pos] ^ 0x21 if (d[pos] ^ 0x21) != 0xFF else d[pos] ^ 0x11
            ctypes.memmove(b.keep[i][0], bytes(d), len(d))
            pk[i] = (bytes(d), codec, output)
        b.reset()
        pool.decode_raw(b.arr)
        for i, (p, codec, output) in enumerate(pk):
            st, payload = _oracle(p, codec, output)
            assert b.arr[i].status == st, (i, b.arr[i].message)
            if st == 0:
                assert b.payload(i) == payload, i
