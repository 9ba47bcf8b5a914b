"""Full-size workloads on the GPU: every frame must decode, sampled frames must
equal the oracle sample for sample, and size-independent properties hold on
all frames (determinism across runs, batch vs one-frame decode, batch
composition)."""

import hashlib

import numpy as np
import pytest

import mmrecode_gb300 as m
import oracle
from mmrecode_gb300 import synth

pytestmark = [pytest.mark.gpu, pytest.mark.slow]


@pytest.fixture(scope="module")
def ctx():
    c = m.Context()
    yield c
    c.close()


def _digest(results):
    return [hashlib.sha256(p).hexdigest() if p is not None else r.status for r, p in results]


def test_mjpeg_1080p_422_300_frames_rgb(ctx):
    packets = synth.mjpeg_stream(20261203, 300, 1920, 1080, "422", 90, 120)
    a = ctx.decode_batch(packets, m.CODEC_MJPEG, m.OUTPUT_RGB24)
    assert all(r.status == 0 for r, _ in a), [r.message for r, _ in a if r.status][:3]
    b = ctx.decode_batch(packets, m.CODEC_MJPEG, m.OUTPUT_RGB24)
    assert _digest(a) == _digest(b)  # deterministic
    for i in (0, 95, 151, 299):
        ref = oracle.jpeg_decode(packets[i])
        assert a[i][1] == oracle.rgb24(ref.frame), f"frame {i}"
    single = ctx.decode_batch([packets[95]], m.CODEC_MJPEG, m.OUTPUT_RGB24)[0]
    assert single[1] == a[95][1]


def test_dv_1000_frames(ctx):
    packets = synth.dv_stream(20261204, 1000)
    res = ctx.decode_batch(packets, m.CODEC_DV)
    assert all(r.status == 0 for r, _ in res)
    for i in (0, 499, 999):
        ref = oracle.dv_decode(packets[i])
        f = m.frame_from_batch(*res[i])
        assert [p.data for p in f.planes] == [b for _, _, b in ref.frame.planes], f"frame {i}"


def test_mixed_512_frames_sampled(ctx):
    packets, params = synth.mixed_mjpeg_stream(20261205, 512)
    res = ctx.decode_batch(packets, m.CODEC_MJPEG)
    assert all(r.status == 0 for r, _ in res)
    # oracle on the smallest frames of each subsampling / restart class
    order = sorted(range(len(params)), key=lambda i: params[i][1] * params[i][2])
    seen = set()
    for i in order:
        key = (params[i][3], params[i][5] == 0, params[i][5] == 4)
        if key in seen:
            continue
        seen.add(key)
        ref = oracle.jpeg_decode(packets[i])
        f = m.frame_from_batch(*res[i])
        assert [p.data for p in f.planes] == [b for _, _, b in ref.frame.planes], f"frame {i} {params[i]}"
    assert len(seen) >= 6
