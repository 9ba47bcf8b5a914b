"""CUDA-graph replay of repeated device-resident batches: replayed results equal
direct ones and the oracle, and a replayed graph reads the current packets."""

import ctypes

import pytest

import mmrecode_gb300 as m
import oracle
from mmrecode_gb300 import _lib, synth

pytestmark = pytest.mark.gpu


def _batch(torch, packets, output):
    offs, o = [], 0
    for p in packets:
        offs.append(o)
        o += (len(p) + 255) // 256 * 256
    host = torch.zeros(o, dtype=torch.uint8, pin_memory=True)
    for p, off in zip(packets, offs):
        host.numpy()[off:off + len(p)] = memoryview(p)
    dev = host.cuda()
    need = [m.probe(m.CODEC_MJPEG, p).rgb_bytes if output == m.OUTPUT_RGB24 else m.probe(m.CODEC_MJPEG, p).planar_bytes
            for p in packets]
    outs = [torch.zeros(n, dtype=torch.uint8, device="cuda") for n in need]
    arr = (_lib.GpuItem * len(packets))()
    for i, p in enumerate(packets):
        it = arr[i]
        it.struct_size = ctypes.sizeof(_lib.GpuItem)
        it.data = host.data_ptr() + offs[i]
        it.device_data = dev.data_ptr() + offs[i]
        it.len = len(p)
        it.codec = m.CODEC_MJPEG
        it.output = output
        it.flags = m.ITEM_OUT_DEVICE
        it.out = outs[i].data_ptr()
        it.out_capacity = need[i]
    return host, dev, offs, outs, arr


def _run(ctx, arr):
    try:
        ctx.decode_raw(arr)
    except m.MmrError as e:
        raise AssertionError(f"{e}: {arr[0].message}")


def _expected(p, output):
    ref = oracle.jpeg_decode(p)
    if ref.status:
        return ref.status, None
    return 0, oracle.rgb24(ref.frame) if output == m.OUTPUT_RGB24 else b"".join(d for (_, _, d) in ref.frame.planes)


@pytest.mark.parametrize("output", [m.OUTPUT_RGB24, m.OUTPUT_PLANAR])
def test_replayed_batches_match_and_read_current_packets(output):
    torch = pytest.importorskip("torch")
    packets = synth.mjpeg_stream(601, 12, 320, 240, "422", 85, 20) + synth.mjpeg_stream(602, 4, 256, 128, "420", 70, 0)
    host, dev, offs, outs, arr = _batch(torch, packets, output)
    with m.Context(engines=1) as ctx:
        replays = []
        for _ in range(3):
            _run(ctx, arr)
            replays.append(ctx.stats()["graph_replays"])
            for i, p in enumerate(packets):
                st, payload = _expected(p, output)
                assert arr[i].status == st == 0
                assert outs[i].cpu().numpy().tobytes() == payload, i
        assert replays == [0, 1, 1]
        # same lengths and headers, different entropy-coded bytes: the plan is
        # unchanged, so the graph replays, and must decode the new bytes
        changed = []
        for i, p in enumerate(packets):
            d = bytearray(p)
            sos = d.index(b"\xff\xda")
            pos = sos + 2 + (d[sos + 2] << 8 | d[sos + 3]) + 40
            d[pos] = d[pos] ^ 0x21 if (d[pos] ^ 0x21) != 0xFF else d[pos] ^ 0x11
            changed.append(bytes(d))
            host.numpy()[offs[i]:offs[i] + len(d)] = memoryview(bytes(d))
        dev.copy_(host)
        _run(ctx, arr)
        assert ctx.stats()["graph_replays"] == 1
        for i, p in enumerate(changed):
            st, payload = _expected(p, output)
            assert arr[i].status == st, (i, arr[i].message)
            if st == 0:
                assert outs[i].cpu().numpy().tobytes() == payload, i
        ctx.set_graphs(False)
        _run(ctx, arr)
        assert ctx.stats()["graph_replays"] == 0


def test_same_lengths_and_sizes_different_geometry_never_replay_a_stale_graph():
    """Two batches in the same buffers with equal packet lengths, output sizes
    and plan size but transposed frame geometry (64x32 against 32x64 gray): each
    replays only its own captured graph, and every output equals the oracle's."""
    torch = pytest.importorskip("torch")
    import numpy as np

    rng = np.random.default_rng(7)

    def gray(w, h):
        px = rng.integers(0, 256, (h, w), dtype=np.uint8).tobytes()
        return m.encode_jpeg(m.VideoFrame(m.GRAY8, w, h, [m.Plane(px, w, w, h)], m.RANGE_FULL), 80)

    a = [gray(64, 32), gray(64, 32)]
    b = [gray(32, 64), gray(32, 64)]
    size = max(len(p) for p in a + b)
    a = [p + bytes(size - len(p)) for p in a]  # bytes after EOI are the reference's trailing data
    b = [p + bytes(size - len(p)) for p in b]
    host, dev, offs, outs, arr = _batch(torch, a, m.OUTPUT_PLANAR)

    def load(packets):
        for i, p in enumerate(packets):
            host.numpy()[offs[i]:offs[i] + len(p)] = memoryview(p)
        dev.copy_(host)

    with m.Context(engines=1) as ctx:
        replays = []
        for packets in (a, a, a, b, b, b, a, b):
            load(packets)
            _run(ctx, arr)
            replays.append(ctx.stats()["graph_replays"])
            for i, p in enumerate(packets):
                st, payload = _expected(p, m.OUTPUT_PLANAR)
                assert arr[i].status == st == 0, arr[i].message
                assert (arr[i].width, arr[i].height) == ((64, 32) if packets is a else (32, 64))
                assert outs[i].cpu().numpy().tobytes() == payload, i
        assert replays == [0, 1, 1, 0, 1, 1, 1, 1]
