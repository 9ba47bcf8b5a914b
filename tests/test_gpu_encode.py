"""GPU batch JPEG encoder (mmr_gpu_jpeg_encode_batch): every output byte equals the
CPU encoder restatement's (itself byte-identical to the reference encoder's golden
stream) with the same options; statuses and messages equal too."""

import ctypes

import numpy as np
import pytest

import mmrecode_gb300 as m
import oracle
from mmrecode_gb300 import _lib, synth

from helpers import fixture, read_y4m_420

pytestmark = pytest.mark.gpu

FORMATS = {"gray": (m.GRAY8, 1, 1), "420": (m.YUV420P8, 2, 2), "422": (m.YUV422P8, 2, 1), "444": (m.YUV444P8, 1, 1)}


@pytest.fixture(scope="module")
def ctx():
    c = m.Context()
    yield c
    c.close()


def noise_frame(seed: int, w: int, h: int, sub: str, strided: bool = False) -> m.VideoFrame:
    """Uniform noise (the largest coefficients, many quotients near half-integers)."""
    fmt, sx, sy = FORMATS[sub]
    rng = np.random.default_rng(seed)
    chroma = ((w + sx - 1) // sx, (h + sy - 1) // sy)
    dims = [(w, h)] if sub == "gray" else [(w, h), chroma, chroma]
    planes = []
    for pw, ph in dims:
        a = rng.integers(0, 256, (ph, pw), dtype=np.uint8)
        if strided:  # stride wider than the plane
            wide = np.zeros((ph, pw + 7), np.uint8)
            wide[:, :pw] = a
            planes.append(m.Plane(wide.tobytes(), pw + 7, pw, ph))
        else:
            planes.append(m.Plane(a.tobytes(), pw, pw, ph))
    return m.VideoFrame(fmt, w, h, planes, m.RANGE_FULL)


def content_frame(seed: int, w: int, h: int, sub: str) -> m.VideoFrame:
    if sub == "gray":
        f = synth.mjpeg_frame(seed, 0, w, h, "444")
        return m.VideoFrame(m.GRAY8, w, h, f.planes[:1], m.RANGE_FULL)
    return synth.mjpeg_frame(seed, 0, w, h, sub)


def cpu(frame, q, annex_k=False, ri=0):
    try:
        return 0, "", m.encode_jpeg(frame, q, annex_k, ri)
    except m.MmrError as e:
        return e.status, e.message, None


def check(ctx, frames, q=75, annex_k=False, ri=0):
    got = ctx.encode_jpeg_batch(frames, q, annex_k, ri)
    for i, (f, g) in enumerate(zip(frames, got)):
        ref = cpu(f, q, annex_k, ri)
        assert g[0] == ref[0], (i, g[1], ref[1])
        assert g[1] == ref[1], i
        assert g[2] == ref[2], f"frame {i} ({f.width}x{f.height} fmt {f.format} q{q} annex {annex_k} ri {ri})"
    return got


def test_reference_golden_stream(ctx):
    frames = []
    for w, h, y, cb, cr in read_y4m_420(fixture("y4m/valid/two-frame-420.y4m")):
        cw, ch = (w + 1) // 2, (h + 1) // 2
        frames.append(m.VideoFrame(m.YUV420P8, w, h, [m.Plane(y, w, w, h), m.Plane(cb, cw, cw, ch),
                                                      m.Plane(cr, cw, cw, ch)], m.RANGE_FULL))
    got = ctx.encode_jpeg_batch(frames, 85)
    assert all(g[0] == 0 for g in got)
    assert b"".join(g[2] for g in got) == fixture("jpeg/encoded/mmrecode-q85-420.mjpg")


@pytest.mark.parametrize("sub", ["gray", "420", "422", "444"])
@pytest.mark.parametrize("q", [1, 50, 90, 100])
def test_formats_and_qualities(ctx, sub, q):
    sizes = [(1, 1), (7, 9), (17, 33), (64, 48), (250, 130)]
    frames = [noise_frame(100 * q + k, w, h, sub) for k, (w, h) in enumerate(sizes)]
    frames += [content_frame(7 + k, w, h, sub) for k, (w, h) in enumerate(sizes[2:])]
    check(ctx, frames, q)


@pytest.mark.parametrize("ri", [1, 3, 16, 1000])
def test_annex_k_and_restart_intervals(ctx, ri):
    frames = [content_frame(40 + k, w, h, sub) for k, (w, h, sub) in
              enumerate([(256, 128, "422"), (200, 136, "420"), (96, 40, "444"), (33, 17, "gray")])]
    frames.append(noise_frame(99, 130, 66, "422"))
    check(ctx, frames, 90, True, ri)
    check(ctx, frames, 60, False, ri)


def test_mixed_batch_strides_and_errors(ctx):
    good = [noise_frame(1, 64, 64, "420", strided=True), content_frame(2, 320, 240, "422"),
            noise_frame(3, 31, 29, "gray", strided=True)]
    limited = content_frame(4, 32, 32, "420")
    limited = m.VideoFrame(limited.format, limited.width, limited.height, limited.planes, m.RANGE_LIMITED)
    wrong = content_frame(5, 48, 48, "420")
    wrong = m.VideoFrame(wrong.format, 50, 48, wrong.planes, m.RANGE_FULL)  # planes do not match the size
    check(ctx, good + [limited, wrong] + good)
    got = ctx.encode_jpeg_batch(good, 0)  # quality 0
    assert {g[0] for g in got} == {m.INVALID_DATA}
    assert all(g[1] == "invalid data: JPEG quality must be between 1 and 100" for g in got)


def test_output_capacity_and_device_buffers(ctx):
    torch = pytest.importorskip("torch")
    frames = [content_frame(60 + k, 256, 144, "422") for k in range(4)]
    ref = [cpu(f, 90, True, 16)[2] for f in frames]
    lib = _lib.load()
    n = len(frames)
    items = (_lib.EncodeItem * n)()
    dev_in, dev_out = [], []
    for i, f in enumerate(frames):
        it = items[i]
        it.struct_size = ctypes.sizeof(_lib.EncodeItem)
        v = _lib.VideoFrameView()
        v.struct_size = ctypes.sizeof(_lib.VideoFrameView)
        v.format, v.range, v.width, v.height, v.plane_count = f.format, f.range, f.width, f.height, len(f.planes)
        for c, p in enumerate(f.planes):
            t = torch.frombuffer(bytearray(p.data), dtype=torch.uint8).cuda()
            dev_in.append(t)
            v.planes[c].data = ctypes.cast(t.data_ptr(), _lib.u8p)
            v.planes[c].data_len, v.planes[c].stride = len(p.data), p.stride
            v.planes[c].width, v.planes[c].height = p.width, p.height
        it.frame = v
        cap = lib.mmr_gpu_jpeg_encode_bound(f.format, f.width, f.height, 16)
        o = torch.empty(cap, dtype=torch.uint8, device="cuda")
        dev_out.append(o)
        it.out = o.data_ptr()
        it.out_capacity = cap if i != 2 else len(ref[2]) - 1  # one byte short
        it.flags = m.ITEM_OUT_DEVICE | m.ITEM_IN_DEVICE
    ctx.encode_raw(items, 90, True, 16)
    for i in range(n):
        if i == 2:
            assert items[i].status == m.INVALID_ARGUMENT
            assert items[i].message.decode() == "invalid argument: output buffer is smaller than the encoded frame"
            continue
        assert items[i].status == 0, items[i].message
        assert dev_out[i][: items[i].out_len].cpu().numpy().tobytes() == ref[i]


def test_binary64_recomputation_is_exercised(ctx):
    frames = [noise_frame(500 + k, 128, 128, "444") for k in range(4)]
    check(ctx, frames, 100)
    st = ctx.encode_stats()
    assert st["blocks"] == 4 * 3 * 16 * 16 and st["exact_coefficients"] > 0


def test_gpu_encoded_streams_decode_like_cpu_ones(ctx):
    frames = [content_frame(70 + k, 1920, 1080, "422") for k in range(2)]
    got = check(ctx, frames, 90, True, 120)
    for (_, _, data), f in zip(got, frames):
        r = oracle.jpeg_decode(data)
        assert r.status == 0 and (r.frame.width, r.frame.height) == (f.width, f.height)
