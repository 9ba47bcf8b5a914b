"""Exact transforms under volume and adversarial input.

The library evaluates the reference's binary64 transforms in fp32 and keeps a
value only when a proven error bound says it rounds like the reference; the
rest go to the binary64 reference order. These tests push well over a million
blocks through that machinery and compare every sample with the oracle:

* block level: the device functions the kernels use (idct_core.h,
  dv_idct_core.h, fdct_core.h), driven by tests/cuda/transform_harness.cu with
  the kernels' thread mappings, against orc_jpeg_idct, orc_dv_idct88 /
  orc_dv_idct248 (crates/codecs/mjpeg/src/transform.rs:86-134,
  crates/codecs/dv/src/decoder.rs:520-602) and forward_dct_quantize;
* stream level: crafted JPEG streams whose quantised coefficients are the
  adversarial blocks, through the real decoder (chunked entropy decode, planar
  IDCT + exact fix-up, fused IDCT + RGB kernel) against the oracle decoder; and
  adversarial frames through the GPU encoder against the oracle encoder.

Block kinds: dense blocks up to 2^20, quantiser-255 products with i32-range DC,
every DC value of a range (exact half-integer ties), sparse blocks, and blocks
built so that one sample (one quotient for the encoder) lies within 2^-20 of a
half-integer, also at the clamp edges -0.5 and 255.5 (tests/adversarial.py).
"""

import ctypes
import os
import zlib
import shutil
import subprocess

import numpy as np
import pytest

import adversarial
import mmrecode_gb300 as m
import oracle
from helpers import report

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "mmrecode_gb300", "csrc")


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = tmp_path_factory.mktemp("harness") / "libtransform_harness.so"
    cmd = [nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-shared", "-Xcompiler",
           "-fPIC", "-I", CSRC, os.path.join(ROOT, "tests", "cuda", "transform_harness.cu"), "-o", str(out)]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    lib = ctypes.CDLL(str(out))
    vp = ctypes.c_void_p
    lib.harness_jpeg_idct.argtypes = [vp, ctypes.c_uint64, vp, vp]
    lib.harness_dv_idct.argtypes = [vp, vp, ctypes.c_uint64, vp]
    lib.harness_fdct.argtypes = [vp, vp, vp, ctypes.c_uint64, vp, vp]
    return lib


def _first_mismatches(gpu, ref, what, extra=None):
    bad = np.nonzero((gpu != ref).reshape(len(gpu), -1).any(axis=1))[0]
    msg = [f"{what}: {len(bad)} of {len(gpu)} blocks differ"]
    for b in bad[:3]:
        msg.append(f"block {b}: gpu {gpu[b].tolist()} ref {ref[b].tolist()}" + (f" in {extra[b].tolist()}" if extra is not None else ""))
    return bad, "\n".join(msg)


def test_mjpeg_idct_blocks_match_the_reference_order(harness):
    c, kinds, near = adversarial.jpeg_idct_blocks(20261211, dense=600_000)
    gpu = np.empty((len(c), 64), np.uint8)
    exact = ctypes.c_ulonglong(0)
    assert harness.harness_jpeg_idct(c.ctypes.data, len(c), gpu.ctypes.data, ctypes.byref(exact)) == 0
    ref = oracle.jpeg_idct_many(c)
    bad, msg = _first_mismatches(gpu, ref, "MJPEG IDCT", c)
    report("mjpeg_idct_blocks", blocks=len(c), near_ties_2e20=near, exact_samples=exact.value, kinds=kinds)
    assert len(bad) == 0, msg
    assert exact.value > near  # every near tie (and more) went through the binary64 order


def test_dv_idct_blocks_match_the_reference_order(harness):
    c, modes, kinds, near = adversarial.dv_idct_blocks(20261212, n=400_000)
    gpu = np.empty((len(c), 64), np.uint8)
    assert harness.harness_dv_idct(c.ctypes.data, modes.ctypes.data, len(c), gpu.ctypes.data) == 0
    ref = np.where(modes[:, None] != 0, oracle.dv_idct248_many(c), oracle.dv_idct88_many(c))
    bad, msg = _first_mismatches(gpu, ref, "DV IDCT", c)
    report("dv_idct_blocks", blocks=len(c), blocks_248=int(modes.sum()), near_ties_2e20=near, kinds=kinds)
    assert len(bad) == 0, msg


def test_forward_dct_blocks_match_the_reference_order(harness):
    s, q, kinds, near = adversarial.fdct_blocks(20261213, n=600_000)
    rq = (1.0 / q.astype(np.float32)).astype(np.float32)  # as the encoder's host plan computes them
    gpu = np.empty((len(s), 64), np.int32)
    exact = ctypes.c_ulonglong(0)
    assert harness.harness_fdct(s.ctypes.data, q.ctypes.data, rq.ctypes.data, len(s), gpu.ctypes.data,
                                ctypes.byref(exact)) == 0
    ref = oracle.fdct_quantize_many(s, q)
    bad, msg = _first_mismatches(gpu, ref, "forward DCT", s)
    report("fdct_blocks", blocks=len(s), near_ties_2e20=near, exact_coefficients=exact.value, kinds=kinds)
    assert len(bad) == 0, msg
    assert exact.value >= near


# ------------------------------------------------------------------ streams ---

def _levels_walk(rng, n, dc_lo, dc_hi, step=2047):
    """A DC level sequence with consecutive differences within +-step."""
    d = rng.integers(-step, step + 1, n)
    out = np.empty(n, np.int64)
    v = 0
    for i in range(n):
        v = min(max(v + int(d[i]), dc_lo), dc_hi)
        out[i] = v
    return out


def _gray_blocks(rng, bw, bh, kind):
    """Quantised levels (scan order = raster of blocks) and the quantisation table."""
    n = bw * bh
    lv = np.zeros((n, 64), np.int64)
    if kind == "dense_q1":
        qt = np.ones(64, np.int64)
        lv[:, 1:] = rng.integers(-1023, 1024, (n, 63))
        lv[:, 0] = _levels_walk(rng, n, -2000, 2000)  # a restart resets the prediction to 0
    elif kind == "dense_q255":
        qt = np.full(64, 255, np.int64)
        lv[:, 1:] = rng.integers(-1023, 1024, (n, 63)) * (rng.random((n, 63)) < 0.5)
        lv[:, 0] = _levels_walk(rng, n, -8_000_000, 8_000_000)
    elif kind == "i32_dc":  # DC climbs to within one step of the largest i32 dequantised value
        qt = np.full(64, 255, np.int64)
        top = (2 ** 31 - 1) // 255
        lv[:, 0] = np.minimum(np.arange(1, n + 1) * 2047, top)
        lv[:, 1:] = rng.integers(-5, 6, (n, 63)) * (rng.random((n, 63)) < 0.3)
    elif kind == "near_ties":
        qt = np.ones(64, np.int64)
        W = adversarial.jpeg_weights()
        per = n // 8
        c, _ = adversarial.near_ties(rng, W, 8, per, 120, 300, offset=128.0)
        lv[:len(c)] = c
        lv[len(c):, 1:] = rng.integers(-200, 201, (n - len(c), 63))
        # DC differences within the category-11 limit: the DC values are at most +-720
    else:
        raise ValueError(kind)
    return lv, qt


@pytest.fixture(scope="module")
def ctx():
    c = m.Context()
    yield c
    c.close()


@pytest.mark.parametrize("kind,restart", [("dense_q1", 0), ("dense_q1", 16), ("dense_q255", 0), ("i32_dc", 0),
                                          ("near_ties", 0), ("near_ties", 8)])
def test_crafted_gray_streams_planar(ctx, kind, restart):
    """Gray frames of adversarial blocks through the real decoder (planar output:
    chunked entropy decode, planar IDCT, exact fix-up), every block against the oracle."""
    rng = np.random.default_rng(zlib.crc32(f"{kind}/{restart}".encode()))
    bw, bh = 256, 128  # 2048 x 1024: 32768 blocks per frame
    frames, blocks = [], []
    for f in range(4):
        lv, qt = _gray_blocks(rng, bw, bh, kind)
        frames.append(oracle.jpeg_write_levels(bw * 8, bh * 8, [(1, 1)], [0], [qt], lv, restart_interval=restart))
        blocks.append(lv * qt)
    res = ctx.decode_batch(frames, m.CODEC_MJPEG, m.OUTPUT_PLANAR)
    total = 0
    for f, ((r, payload), c) in enumerate(zip(res, blocks)):
        assert r.status == 0, r.message
        plane = np.frombuffer(payload, np.uint8).reshape(bh, 8, bw, 8).transpose(0, 2, 1, 3).reshape(-1, 64)
        ref = oracle.jpeg_idct_many(c.astype(np.int32))
        bad, msg = _first_mismatches(plane, ref, f"{kind} frame {f}", c)
        assert len(bad) == 0, msg
        total += len(c)
    report(f"stream_gray_{kind}_ri{restart}", blocks=total)


@pytest.mark.parametrize("sampling,restart", [((1, 1), 0), ((2, 1), 12), ((2, 2), 0)])
def test_crafted_colour_streams_rgb(ctx, sampling, restart):
    """Three-component frames of dense and near-tie blocks through the fused
    IDCT + RGB kernel, against the oracle decoder + RGB conversion."""
    rng = np.random.default_rng(sampling[0] * 10 + sampling[1] + restart)
    h, v = sampling
    w_px, h_px = 1024, 512
    mcus = (w_px // (8 * h)) * (h_px // (8 * v))
    per_mcu = h * v + 2
    W = adversarial.jpeg_weights()
    frames = []
    for f in range(3):
        n = mcus * per_mcu
        lv = np.zeros((n, 64), np.int64)
        lv[:, 1:] = rng.integers(-60, 61, (n, 63))
        c, _ = adversarial.near_ties(rng, W, 4, n // 8, 60, 200, offset=128.0)
        pick = rng.choice(n, len(c), replace=False)
        lv[pick] = c
        lv[:, 0] = np.clip(lv[:, 0], -900, 900)
        qt = [np.ones(64, np.int64), np.ones(64, np.int64)]
        frames.append(oracle.jpeg_write_levels(w_px, h_px, [(h, v), (1, 1), (1, 1)], [0, 1, 1], qt, lv,
                                               restart_interval=restart))
    res = ctx.decode_batch(frames, m.CODEC_MJPEG, m.OUTPUT_RGB24)
    for f, ((r, payload), pkt) in enumerate(zip(res, frames)):
        ref = oracle.jpeg_decode(pkt)
        assert r.status == ref.status == 0, (r.message, ref.message)
        assert payload == oracle.rgb24(ref.frame), f"frame {f}"
    report(f"stream_rgb_{h}x{v}_ri{restart}", blocks=3 * mcus * per_mcu)


def test_adversarial_frames_through_the_gpu_encoder(ctx):
    """Near-tie, noise and extreme sample blocks in frames encoded by the GPU
    encoder at q100 (unit quantisers) and q50: every byte equals the oracle encoder."""
    s, q, _, near = adversarial.fdct_blocks(20261214, n=40_000)
    keep = np.nonzero(q.max(axis=1) == 1)[0]  # blocks built for unit quantisers
    s = s[keep]
    bw = 128
    bh = len(s) // bw
    s = s[:bw * bh]
    plane = s.reshape(bh, bw, 8, 8).transpose(0, 2, 1, 3).reshape(bh * 8, bw * 8)
    f = m.VideoFrame(m.GRAY8, bw * 8, bh * 8, [m.Plane(plane.tobytes(), bw * 8, bw * 8, bh * 8)], m.RANGE_FULL)
    for quality in (100, 50):
        st, msg, got = ctx.encode_jpeg_batch([f], quality, annex_k=True, restart_interval=0)[0]
        assert st == 0, msg
        ref = oracle.jpeg_encode(oracle.FMT_GRAY8, bw * 8, bh * 8, [(bw * 8, bh * 8, plane.tobytes())], quality,
                                 annex_k=True)
        assert got == ref, f"quality {quality}"
    report("encoder_frames", blocks=2 * bw * bh)
