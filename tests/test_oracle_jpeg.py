"""The oracle's baseline JPEG decode (oracle/jpeg.c) against the second restatement in
tests/restatements.py, written in Python from crates/codecs/mjpeg/src/{parser,entropy,
decoder}.rs: marker parse, Huffman tables, bit reader, restart handling, block decode,
the inverse DCT and plane layout. Same status and message on every input, every sample
of every frame. Inputs: the reference fixtures, the crafted edge cases of the GPU tests,
encoder streams of every layout with Annex K and the encoder's own tables, one to many
restart intervals, and seeded mutations of their entropy-coded bytes and restart
markers. The reference's own tests pin no pixel values of a non-trivial decode, no
Annex K table decode, 4:2:2 or multi-interval restart decode."""
import numpy as np

import mmrecode_gb300 as m
import oracle
from helpers import JPEG_FIXTURES, fixture
from mmrecode_gb300 import synth
from restatements import JpegError, decode_jpeg


def compare(data, label):
    ref = oracle.jpeg_decode(data)
    try:
        fmt, w, h, planes = decode_jpeg(data)
    except JpegError as e:
        assert (ref.status, ref.message) == (e.status, e.message), f"{label}: oracle {ref.status} {ref.message!r}"
        return e.status
    assert ref.status == 0, f"{label}: oracle {ref.status} {ref.message!r}, restatement decoded"
    f = ref.frame
    assert (f.format, f.width, f.height) == (fmt, w, h), label
    assert [p[:2] for p in f.planes] == [p[:2] for p in planes], label
    for i, ((_, _, a), (_, _, b)) in enumerate(zip(planes, f.planes)):
        if a != b:
            x, y = np.frombuffer(a, np.uint8), np.frombuffer(b, np.uint8)
            raise AssertionError(f"{label}: plane {i}: {int((x != y).sum())} samples differ")
    return 0


def streams():
    out = []
    rng = np.random.default_rng(61)
    for i in range(16):
        sub = ["420", "422", "444", "gray"][i % 4]
        w, h = int(rng.integers(8, 72)), int(rng.integers(8, 56))
        q = int(rng.integers(20, 101))
        ri = [0, 1, 2, 5, 64][i % 5]
        if sub == "gray":
            frame = m.VideoFrame(m.GRAY8, w, h, [m.Plane(rng.integers(0, 256, w * h, dtype=np.uint8).tobytes(), w, w, h)],
                                 m.RANGE_FULL)
        else:
            frame = synth.mjpeg_frame(600 + i, 0, w, h, sub)
        out.append(m.encode_jpeg(frame, q, annex_k=bool(i % 2), restart_interval=ri))
    return out


def entropy_mutations(data, rng, count):
    """Byte changes inside the entropy-coded data that neither make nor remove a 0xff
    byte (the scan keeps its extent), and restart markers renumbered."""
    start = data.index(b"\xff\xda") + 2
    start += (data[start] << 8) | data[start + 1]
    end = data.rindex(b"\xff\xd9")
    out = []
    for j in range(count):
        b = bytearray(data)
        if j % 4 == 3:
            rst = [i for i in range(start, end - 1) if b[i] == 0xFF and 0xD0 <= b[i + 1] <= 0xD7]
            if rst:
                at = rst[int(rng.integers(0, len(rst)))] + 1
                b[at] = 0xD0 + (b[at] - 0xD0 + int(rng.integers(1, 8))) % 8
                out.append(bytes(b))
                continue
        for _ in range(1 + j % 3):
            at = int(rng.integers(start, end))
            if b[at] == 0xFF or b[at - 1] == 0xFF:
                continue
            v = b[at] ^ (1 << int(rng.integers(0, 8)))
            if v != 0xFF:
                b[at] = v
        out.append(bytes(b))
    return out


def test_fixtures_and_crafted_cases():
    import test_gpu_parity  # the crafted edge cases (building them needs no GPU)

    for rel in JPEG_FIXTURES:
        compare(fixture(rel), rel)
    statuses = [compare(data, name) for name, data in sorted(test_gpu_parity.crafted_cases().items())]
    assert statuses.count(0) >= 8 and statuses.count(2) >= 10 and statuses.count(3) >= 3, statuses


def test_encoder_streams_and_entropy_mutations():
    rng = np.random.default_rng(62)
    outcomes = {}
    for i, s in enumerate(streams()):
        assert compare(s, f"stream {i}") == 0
        for j, d in enumerate(entropy_mutations(s, rng, 24)):
            st = compare(d, f"stream {i} mutation {j}")
            outcomes[st] = outcomes.get(st, 0) + 1
    assert outcomes.get(0, 0) > 20 and outcomes.get(2, 0) > 100, outcomes


def test_benchmark_frames():
    """The first frame of the 1080p 4:2:2 q90 workload (restart interval 120 MCUs,
    135 intervals) and of the 640x480 4:2:0 q75 one (no restart markers)."""
    compare(synth.mjpeg_stream(20261203, 1, 1920, 1080, "422", 90, 120, annex_k=True)[0], "1080p 4:2:2")
    compare(synth.mjpeg_stream(20261201, 1, 640, 480, "420", 75, 0, annex_k=True)[0], "640x480 4:2:0")
