"""The host-side header probe (mmr_gpu_probe, mmrecode_gb300/csrc/engine.cu probe_packet)
against the oracle's full decode, on CPU. The probe sizes every output buffer of the
batch, session and server paths before the GPU sees a packet, so: wherever the oracle
decodes a packet, the probe reports that frame's format, size and plane geometry
(decode_jpeg + into_video_frame, crates/codecs/mjpeg/src/decoder.rs:69-167; DV
detect_profile, crates/codecs/dv/src/profile.rs:87-127); wherever the probe already
fails, the oracle fails with the same status. Inputs: synthetic MJPEG streams of
several layouts and sizes with seeded mutations of their marker segments, and NTSC
and PAL DV frames with flipped header bits, wrong lengths and payload damage."""
import numpy as np

import mmrecode_gb300 as m
import oracle
from mmrecode_gb300 import synth


def check(codec, data, label, stats):
    ref = oracle.jpeg_decode(data) if codec == m.CODEC_MJPEG else oracle.dv_decode(data)
    pr = m.probe(codec, data)
    stats[(ref.status, pr.status)] = stats.get((ref.status, pr.status), 0) + 1
    if ref.status == 0:
        f = ref.frame
        assert pr.status == 0, label
        assert (pr.format, pr.range, pr.width, pr.height, pr.plane_count) == \
            (f.format, f.range, f.width, f.height, len(f.planes)), label
        for c, (w, h, _) in enumerate(f.planes):
            assert (pr.plane_width[c], pr.plane_height[c]) == (w, h), f"{label}: plane {c}"
        assert pr.planar_bytes == sum(w * h for w, h, _ in f.planes), label
        assert pr.rgb_bytes == f.width * f.height * 3, label
    elif pr.status != 0:
        assert pr.status == ref.status, f"{label}: probe {pr.status}, oracle {ref.status} {ref.message}"


def test_mjpeg_probe_agrees_with_the_decode():
    rng = np.random.Generator(np.random.PCG64(9))
    packets = []
    for i, (w, h, sub, q, ri) in enumerate([(64, 48, "420", 75, 0), (80, 40, "422", 90, 5), (48, 48, "444", 50, 3),
                                            (33, 17, "420", 95, 1), (120, 64, "422", 60, 0), (1, 1, "444", 80, 0),
                                            (17, 250, "420", 70, 2)]):
        packets += synth.mjpeg_stream(400 + i, 1, w, h, sub, q, ri, annex_k=bool(i % 2))
    stats = {}
    for i, p in enumerate(packets):
        check(m.CODEC_MJPEG, p, f"stream {i}", stats)
        head = max(16, int(oracle.jpeg_parse(p)[2]["data_offset"]) or len(p))
        for j in range(200):
            b = bytearray(p)
            op, at = j % 4, int(rng.integers(0, min(head, len(p))))
            if op == 0:
                b[at] ^= 1 << int(rng.integers(0, 8))
            elif op == 1:
                b = b[:at]
            elif op == 2:
                del b[at]
            else:
                b.insert(at, b[at])
            check(m.CODEC_MJPEG, bytes(b), f"stream {i} mutation {j} (op {op} at {at})", stats)
    # decodes, header failures the probe sees, and failures only the decode finds
    assert stats.get((0, 0), 0) > 100 and stats.get((2, 2), 0) > 100 and stats.get((2, 0), 0) > 0, stats


def test_dv_probe_agrees_with_the_decode():
    rng = np.random.Generator(np.random.PCG64(10))
    stats = {}
    for i, p in enumerate(synth.dv_stream(500, 1) + synth.dv_stream(501, 1, pal=True)):
        for j in range(60):
            b = bytearray(p)
            op = j % 6
            if op == 0:
                b[0] ^= 1 << int(rng.integers(5, 8))  # DIF section type of the first block
            elif op == 1:
                b[3] ^= 0x80  # the 525/625 flag (profile.rs:37-58)
            elif op == 2:
                b = b[:int(rng.integers(0, len(b)))]
            elif op == 3:
                b += bytes(int(rng.integers(1, 100)))
            elif op == 4:
                b[int(rng.integers(0, 80 * 150))] ^= 1 << int(rng.integers(0, 8))  # first DIF sequence
            check(m.CODEC_DV, bytes(b), f"frame {i} mutation {j} (op {op})", stats)
    assert stats.get((0, 0), 0) >= 40 and stats.get((2, 2), 0) >= 80, stats
