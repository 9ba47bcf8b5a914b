"""Full-size workloads on the GPU, every frame against the oracle.

The benchmark's configurations at full size -- 30 VGA 4:2:0 q75 frames without
restart markers (planar), 300 1080p 4:2:2 q90 frames with a restart interval of
one MCU row (RGB24 and planar), 1000 NTSC DV25 frames (planar) and the 512
mixed MJPEG frames (320x240..3840x2160, every subsampling, quality and restart
layout; RGB24 and planar) -- decode on the GPU, and every frame's samples are
compared with the oracle's (SHA-256 per frame; the oracle runs in a process
pool over all host cores). Also: determinism across runs and batch vs
one-frame decode."""

import hashlib

import pytest

import mmrecode_gb300 as m
from helpers import oracle_digest, oracle_pool, report
from mmrecode_gb300 import synth

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


@pytest.fixture(scope="module")
def ctx():
    c = m.Context()
    yield c
    c.close()


@pytest.fixture(scope="module")
def pool():
    p = oracle_pool()
    yield p
    p.close()
    p.join()


def _sha(b):
    return hashlib.sha256(b).hexdigest() if b is not None else None


def _check_all(pool, ctx, packets, kind, codec, outputs, name):
    """Decodes with each output kind and compares every frame with the oracle."""
    ref = pool.map(oracle_digest, [(kind, p) for p in packets], chunksize=4)
    n_blocks = 0
    for output in outputs:
        res = ctx.decode_batch(packets, codec, output)
        for i, ((r, payload), (st, planar, rgb)) in enumerate(zip(res, ref)):
            assert r.status == st == 0, (i, r.message)
            want = rgb if output == m.OUTPUT_RGB24 else planar
            assert _sha(payload) == want, f"{name} frame {i} ({'rgb' if output == m.OUTPUT_RGB24 else 'planar'})"
        st = ctx.stats()
        n_blocks = max(n_blocks, st["jpeg_blocks"] + st["dv_blocks"])
    report(name, frames=len(packets), outputs=len(outputs), blocks_per_pass=n_blocks)
    return res


def test_c1_vga_420_q75_no_restart_all_30_frames(ctx, pool):
    packets = synth.mjpeg_stream(20261201, 30, 640, 480, "420", 75, 0)
    _check_all(pool, ctx, packets, "mjpeg", m.CODEC_MJPEG, [m.OUTPUT_PLANAR], "c1_vga_420")


def test_c2_1080p_422_all_300_frames(ctx, pool):
    packets = synth.mjpeg_stream(20261203, 300, 1920, 1080, "422", 90, 120)
    a = _check_all(pool, ctx, packets, "mjpeg-rgb", m.CODEC_MJPEG, [m.OUTPUT_PLANAR, m.OUTPUT_RGB24], "c2_1080p_422")
    b = ctx.decode_batch(packets, m.CODEC_MJPEG, m.OUTPUT_RGB24)
    assert [_sha(p) for _, p in a] == [_sha(p) for _, p in b]  # deterministic
    single = ctx.decode_batch([packets[95]], m.CODEC_MJPEG, m.OUTPUT_RGB24)[0]
    assert single[1] == a[95][1]


def test_c3_dv_all_1000_frames(ctx, pool):
    packets = synth.dv_stream(20261204, 1000)
    _check_all(pool, ctx, packets, "dv", m.CODEC_DV, [m.OUTPUT_PLANAR], "c3_dv25_ntsc")


def test_c4_mixed_all_512_frames(ctx, pool):
    packets, params = synth.mixed_mjpeg_stream(20261205, 512)
    _check_all(pool, ctx, packets, "mjpeg-rgb", m.CODEC_MJPEG, [m.OUTPUT_PLANAR, m.OUTPUT_RGB24], "c4_mixed")
    assert {p[3] for p in params} == {"420", "422", "444"} and {p[5] == 0 for p in params} == {True, False}
    assert max(p[1] * p[2] for p in params) > 3000 * 1800  # frames of about 4K are in the batch
