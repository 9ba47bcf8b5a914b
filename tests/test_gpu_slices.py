"""Chunked entropy decoder: output and diagnostics must not depend on the slice size.

Every restart interval (the whole scan without DRI) decodes as fixed-size bit
slices that synchronise with each other. These cases sweep the slice size from
the smallest allowed (128 bits: most blocks straddle several slices) to larger
than any interval (one slice, the serial decode), on valid streams and on
corrupted restart-less streams whose first error lies deep inside a scan.
"""

import random

import pytest

import mmrecode_gb300 as m
import oracle
from mmrecode_gb300 import synth
from helpers import assert_same_decode, frame_planes_gpu, prefixed

pytestmark = pytest.mark.gpu

SLICE_SIZES = (128, 160, 256, 992, 2048, 8192, 1 << 20)


@pytest.fixture(scope="module")
def ctx():
    c = m.Context()
    yield c
    c.set_slice_bits(0)
    c.close()


def check(ctx, packets, label, output=m.OUTPUT_PLANAR):
    refs = [oracle.jpeg_decode(p) for p in packets]
    for bits in SLICE_SIZES:
        ctx.set_slice_bits(bits)
        results = ctx.decode_batch(packets, m.CODEC_MJPEG, output)
        for i, ((r, payload), ref) in enumerate(zip(results, refs)):
            tag = f"{label}[{i}] slice_bits={bits}"
            assert r.status == ref.status, f"{tag}: {r.status} {r.message} vs {ref.status} {ref.message}"
            if ref.status:
                assert r.message == prefixed(ref.status, ref.message), tag
                continue
            if output == m.OUTPUT_RGB24:
                assert payload == oracle.rgb24(ref.frame), tag
            else:
                f = m.frame_from_batch(r, payload)
                assert_same_decode(0, "", frame_planes_gpu(f), ref, tag)
    ctx.set_slice_bits(0)


def test_slice_bits_argument_checks(ctx):
    for bad in (1, 96, 100, 130, (1 << 20) + 32):
        with pytest.raises(m.MmrError) as e:
            ctx.set_slice_bits(bad)
        assert e.value.status == m.INVALID_ARGUMENT
    ctx.set_slice_bits(0)


def test_valid_streams_every_slice_size(ctx):
    packets = (synth.mjpeg_stream(301, 2, 640, 480, "420", 75, 0) +
               synth.mjpeg_stream(302, 2, 96, 64, "422", 80, 6) +
               synth.mjpeg_stream(303, 2, 208, 112, "444", 60, 1) +
               synth.mjpeg_stream(304, 1, 320, 240, "422", 95, 40))
    check(ctx, packets, "valid")


def test_dense_blocks_straddle_many_slices(ctx):
    # quality 100 with noise: most coefficients are non-zero, a block spans
    # several 128-bit slices
    packets = synth.mjpeg_stream(305, 2, 128, 96, "444", 100, 0) + synth.mjpeg_stream(306, 1, 256, 64, "420", 100, 3)
    check(ctx, packets, "dense", output=m.OUTPUT_RGB24)


def test_corruption_deep_in_restartless_scans(ctx):
    rnd = random.Random(307)
    bases = synth.mjpeg_stream(308, 2, 320, 240, "420", 85, 0) + synth.mjpeg_stream(309, 1, 320, 240, "422", 70, 0)
    packets = []
    for k in range(36):
        d = bytearray(bases[k % len(bases)])
        ds = d.index(b"\xff\xda") + 2 + (d[d.index(b"\xff\xda") + 2] << 8 | d[d.index(b"\xff\xda") + 3])
        kind = k % 4
        p = rnd.randrange(ds + (len(d) - ds) // 4, len(d) - 2)
        if kind == 0:
            d[p] = rnd.randrange(256)
        elif kind == 1:
            d = d[:p]
        elif kind == 2:
            del d[p:p + rnd.randint(1, 5)]
        else:
            d[p:p] = bytes([rnd.randrange(256) for _ in range(rnd.randint(1, 3))])
        packets.append(bytes(d))
    check(ctx, packets, "corrupt")


def test_corruption_at_slice_boundaries(ctx):
    base = synth.mjpeg_stream(310, 1, 160, 128, "420", 90, 0)[0]
    sos = base.index(b"\xff\xda")
    ds = sos + 2 + (base[sos + 2] << 8 | base[sos + 3])
    packets = []
    for off in (16, 32, 64, 127, 128, 129, 256, 1024):
        for val in (0x00, 0xFF, 0x5A):
            p = ds + off
            if p >= len(base) - 2:
                continue
            d = bytearray(base)
            d[p] = val
            packets.append(bytes(d))
    check(ctx, packets, "boundary")


def test_autotune_picks_a_size_per_class_and_output_is_unchanged():
    import ctypes
    from mmrecode_gb300 import _lib
    packets = (synth.mjpeg_stream(311, 6, 640, 480, "420", 75, 0) +
               synth.mjpeg_stream(312, 6, 480, 272, "422", 90, 30) +
               synth.mjpeg_stream(313, 6, 320, 240, "444", 60, 4))
    keep, arr = [], (_lib.GpuItem * len(packets))()
    for i, p in enumerate(packets):
        src = (ctypes.c_uint8 * len(p)).from_buffer_copy(p)
        need = m.probe(m.CODEC_MJPEG, p).planar_bytes
        dst = (ctypes.c_uint8 * need)()
        keep.append((src, dst))
        it = arr[i]
        it.struct_size = ctypes.sizeof(_lib.GpuItem)
        it.data, it.len, it.codec, it.output = ctypes.addressof(src), len(p), m.CODEC_MJPEG, m.OUTPUT_PLANAR
        it.out, it.out_capacity = ctypes.addressof(dst), need
    with m.Context(engines=2) as ctx:
        report = ctx.autotune(arr)
        assert len(report) == 3  # three restart layouts
        for r in report:
            assert r["slice_bits"] in (1024, 2048, 4096, 8192) and r["frames"] == 6
            assert r["entropy_ms"][r["slice_bits"]] == min(r["entropy_ms"].values())
        results = ctx.decode_batch(packets, m.CODEC_MJPEG, m.OUTPUT_PLANAR)
    for p, (r, payload) in zip(packets, results):
        ref = oracle.jpeg_decode(p)
        assert r.status == 0
        assert payload == b"".join(d for (_, _, d) in ref.frame.planes)


def _flat_with_texture(seed, w, h):
    """4:2:0 frame: flat grey left half (a few bits per block), noisy right half."""
    import numpy as np
    rng = np.random.default_rng(seed)
    y = np.full((h, w), 120, np.uint8)
    y[:, w // 2:] = rng.integers(0, 256, (h, w - w // 2), dtype=np.uint8)
    cw, ch = (w + 1) // 2, (h + 1) // 2
    c = np.full((ch, cw), 128, np.uint8)
    c[:, cw // 2:] = rng.integers(96, 160, (ch, cw - cw // 2), dtype=np.uint8)
    return m.VideoFrame(m.YUV420P8, w, h, [m.Plane(y.tobytes(), w, w, h), m.Plane(c.tobytes(), cw, cw, ch),
                                          m.Plane(c.copy().tobytes(), cw, cw, ch)], m.RANGE_FULL)


def test_slices_owning_more_blocks_than_their_store_holds(ctx):
    # without restart intervals a large slice of flat image owns thousands of
    # blocks: more than a slice's stored levels can hold, so the final decode
    # pass redoes it; output must not change
    packets = [m.encode_jpeg(_flat_with_texture(320 + i, 640, 480), q, True, 0) for i, q in enumerate((50, 75))]
    refs = [oracle.jpeg_decode(p) for p in packets]
    for bits in (2048, 8192, 65536, 1 << 20):
        ctx.set_slice_bits(bits)
        results = ctx.decode_batch(packets, m.CODEC_MJPEG, m.OUTPUT_PLANAR)
        for i, ((r, payload), ref) in enumerate(zip(results, refs)):
            assert r.status == ref.status == 0, (bits, i, r.message)
            f = m.frame_from_batch(r, payload)
            assert_same_decode(0, "", frame_planes_gpu(f), ref, f"flat[{i}] slice_bits={bits}")
    ctx.set_slice_bits(0)


def test_autotune_strips_and_saved_table_leave_output_unchanged(tmp_path):
    import ctypes
    from mmrecode_gb300 import _lib
    packets = (synth.mjpeg_stream(314, 4, 640, 480, "420", 75, 0) +
               synth.mjpeg_stream(315, 4, 1280, 720, "422", 90, 80) +
               synth.mjpeg_stream(316, 4, 352, 288, "444", 60, 4))
    keep, arr = [], (_lib.GpuItem * len(packets))()
    for i, p in enumerate(packets):
        src = (ctypes.c_uint8 * len(p)).from_buffer_copy(p)
        need = m.probe(m.CODEC_MJPEG, p).rgb_bytes
        dst = (ctypes.c_uint8 * need)()
        keep.append((src, dst))
        it = arr[i]
        it.struct_size = ctypes.sizeof(_lib.GpuItem)
        it.data, it.len, it.codec, it.output = ctypes.addressof(src), len(p), m.CODEC_MJPEG, m.OUTPUT_RGB24
        it.out, it.out_capacity = ctypes.addressof(dst), need
    refs = [oracle.rgb24(oracle.jpeg_decode(p).frame) for p in packets]
    with m.Context(engines=2) as ctx:
        report = ctx.autotune(arr)
        strips = [r for r in report if r["kind"] == "strip"]
        assert {r["frame_class"] >> 8 for r in strips} == {0, 1, 2}  # 4:4:4, 4:2:2, 4:2:0
        for r in strips:
            narrow, wide = (8, 16) if r["frame_class"] >> 8 == 0 else (4, 8)
            tm = r["transform_ms"]
            assert r["strip_mcus"] == (wide if tm["wide"] <= tm["narrow"] else narrow)
        path = str(tmp_path / "tuning.json")
        m.save_tuning(path, report)
        results = ctx.decode_batch(packets, m.CODEC_MJPEG, m.OUTPUT_RGB24)
    for (r, payload), ref in zip(results, refs):
        assert r.status == 0 and payload == ref
    # the other strip everywhere, installed from the saved table: same output
    table = m.load_tuning(path)
    for t in table:
        if t["kind"] == "strip":
            narrow, wide = (8, 16) if t["frame_class"] >> 8 == 0 else (4, 8)
            t["strip_mcus"] = wide if t["strip_mcus"] == narrow else narrow
    with m.Context(engines=1) as ctx:
        ctx.set_tuning(table)
        results = ctx.decode_batch(packets, m.CODEC_MJPEG, m.OUTPUT_RGB24)
        with pytest.raises(m.MmrError):
            ctx.set_tuning([{"kind": "slice", "frame_class": 1, "slice_bits": 100}])
    for (r, payload), ref in zip(results, refs):
        assert r.status == 0 and payload == ref
