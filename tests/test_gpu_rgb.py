"""RGB24 output: odd frame sizes, every subsampling, grey, DV, and device
destinations at any byte alignment, against the oracle's restatement of
terminal_preview.rs:7159-7330."""

import ctypes

import pytest

import mmrecode_gb300 as m
import oracle
from mmrecode_gb300 import _lib, synth

pytestmark = pytest.mark.gpu

SIZES = [(1, 1), (17, 9), (33, 7), (250, 3), (64, 64), (129, 65), (1000, 2)]


@pytest.fixture(scope="module")
def ctx():
    c = m.Context()
    yield c
    c.close()


def _jpeg_packets():
    pk = []
    for k, (w, h) in enumerate(SIZES):
        for sub in ("420", "422", "444"):
            pk.append(m.encode_jpeg(synth.mjpeg_frame(400 + k, 0, w, h, sub), 80, restart_interval=3 if k % 2 else 0))
        f = synth.mjpeg_frame(420 + k, 0, w, h, "444")
        pk.append(m.encode_jpeg(m.VideoFrame(m.GRAY8, w, h, [f.planes[0]], m.RANGE_FULL), 70))
    return pk


def test_odd_sizes_all_subsamplings(ctx):
    packets = _jpeg_packets()
    results = ctx.decode_batch(packets, m.CODEC_MJPEG, m.OUTPUT_RGB24)
    for i, (pkt, (r, payload)) in enumerate(zip(packets, results)):
        ref = oracle.jpeg_decode(pkt)
        assert ref.status == 0 and r.status == 0, (i, r.message, ref.message)
        assert payload == oracle.rgb24(ref.frame), i


def test_dv_rgb_limited_range(ctx):
    packets = synth.dv_stream(410, 2) + synth.dv_stream(411, 1, pal=True)
    results = ctx.decode_batch(packets, m.CODEC_DV, m.OUTPUT_RGB24)
    for i, (pkt, (r, payload)) in enumerate(zip(packets, results)):
        ref = oracle.dv_decode(pkt, False)
        assert r.status == 0, r.message
        assert payload == oracle.rgb24(ref.frame), i


def test_unaligned_device_destinations(ctx):
    torch = pytest.importorskip("torch")
    packets = _jpeg_packets()[:12] + synth.dv_stream(412, 1)
    codecs = [m.CODEC_MJPEG] * 12 + [m.CODEC_DV]
    needs = [m.probe(c, p).rgb_bytes for c, p in zip(codecs, packets)]
    offs, o = [], 0
    for k, n in enumerate(needs):
        o += 1 + k % 15  # every byte alignment
        offs.append(o)
        o += n
    dev = torch.zeros(o + 16, dtype=torch.uint8, device="cuda")
    keep = []
    items = (_lib.GpuItem * len(packets))()
    for i, p in enumerate(packets):
        src = (ctypes.c_uint8 * len(p)).from_buffer_copy(p)
        keep.append(src)
        it = items[i]
        it.struct_size = ctypes.sizeof(_lib.GpuItem)
        it.data = ctypes.addressof(src)
        it.len = len(p)
        it.codec = codecs[i]
        it.output = m.OUTPUT_RGB24
        it.flags = m.ITEM_OUT_DEVICE
        it.out = dev.data_ptr() + offs[i]
        it.out_capacity = needs[i]
    ctx.decode_raw(items)
    host = dev.cpu().numpy().tobytes()
    prev_end = 0
    for i, p in enumerate(packets):
        assert items[i].status == 0, items[i].message
        ref = oracle.jpeg_decode(p) if codecs[i] == m.CODEC_MJPEG else oracle.dv_decode(p, False)
        assert host[offs[i]:offs[i] + needs[i]] == oracle.rgb24(ref.frame), i
        assert host[prev_end:offs[i]] == bytes(offs[i] - prev_end), f"bytes before item {i} were written"
        prev_end = offs[i] + needs[i]


def _dc_frame(hm, vm, mcus_x, mcus_y, values):
    """Three-component frame of DC-only blocks; values cycles through dequantised DCs
    (4 mod 8 gives a sample exactly halfway between two integers)."""
    from helpers import encode_blocks, jpeg, stuff
    comps = [(1, hm, vm, 0), (2, 1, 1, 0), (3, 1, 1, 0)]
    pred = [0, 0, 0]
    blocks, k = [], 0
    for _ in range(mcus_x * mcus_y):
        for c, n in ((0, hm * vm), (1, 1), (2, 1)):
            for _ in range(n):
                d = values[k % len(values)]
                k += 1
                blocks.append((d - pred[c], [(0, (-1) ** k * (k % 5))] if k % 3 == 0 and k % 5 else [], True))
                pred[c] = d
    return jpeg(8 * hm * mcus_x, 8 * vm * mcus_y, comps, entropy=stuff(encode_blocks(blocks).raw_bytes()))


def test_exact_samples_inside_the_fused_conversion(ctx):
    values = [4, -4, 12, -1020, 1020, 0, 516, -516, 1, 996, -1004]
    packets = [_dc_frame(hm, vm, 9, 3, values) for hm, vm in ((1, 1), (2, 1), (2, 2))]
    results = ctx.decode_batch(packets, m.CODEC_MJPEG, m.OUTPUT_RGB24)
    for i, (pkt, (r, payload)) in enumerate(zip(packets, results)):
        ref = oracle.jpeg_decode(pkt)
        assert ref.status == 0 and r.status == 0, (i, r.message, ref.message)
        assert payload == oracle.rgb24(ref.frame), i
    stats = ctx.stats()
    assert stats["idct_exact_samples"] > 0
