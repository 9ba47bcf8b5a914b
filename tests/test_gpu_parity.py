"""GPU decode vs the oracle: identical status, message and every sample.

Covers the reference fixtures, seeded synthetic streams of every benchmark
shape (at sizes the oracle decodes in seconds), crafted edge cases of the
entropy decoder and marker handling, seeded corruption, DV damage and
concealment, RGB output and batch composition."""

import hashlib
import json
import os
import random
import subprocess

import numpy as np
import pytest

import mmrecode_gb300 as m
import oracle
from mmrecode_gb300 import _lib, synth
from helpers import (DV_FIXTURES, GOLDEN, JPEG_FIXTURES, SIMPLE_AC, SIMPLE_DC, assert_same_decode,
                     dv_restamped, encode_blocks, fixture, frame_planes_gpu, jpeg, prefixed, stuff, report)

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def ctx():
    c = m.Context()
    yield c
    c.close()


def gpu_single(codec, data):
    try:
        f = m.decode_jpeg(data) if codec == m.CODEC_MJPEG else m.decode_dv(data)
        return 0, "", frame_planes_gpu(f), f
    except m.MmrError as e:
        return e.status, e.message, [], None


def check_single(codec, data, label, conceal=False):
    ref = oracle.jpeg_decode(data) if codec == m.CODEC_MJPEG else oracle.dv_decode(data, conceal)
    st, msg, planes, frame = gpu_single(codec, data)
    assert_same_decode(st, msg, planes, ref, label)
    if ref.status:
        assert msg == prefixed(ref.status, ref.message), label
    return ref


def check_batch(ctx, codec, packets, label, output=m.OUTPUT_PLANAR, conceal=False):
    results = ctx.decode_batch(packets, codec, output, conceal)
    for i, (pkt, (r, payload)) in enumerate(zip(packets, results)):
        ref = oracle.jpeg_decode(pkt) if codec == m.CODEC_MJPEG else oracle.dv_decode(pkt, conceal)
        assert r.status == ref.status, f"{label}[{i}]: {r.status} {r.message} vs {ref.status} {ref.message}"
        if ref.status:
            assert r.message == prefixed(ref.status, ref.message), f"{label}[{i}]"
            continue
        if output == m.OUTPUT_RGB24:
            assert payload == oracle.rgb24(ref.frame), f"{label}[{i}] rgb"
        else:
            f = m.frame_from_batch(r, payload)
            assert_same_decode(0, "", frame_planes_gpu(f), ref, f"{label}[{i}]")
        if conceal:
            assert r.concealed_segments == len(ref.concealed)


# ------------------------------------------------------------------ fixtures

@pytest.mark.parametrize("rel", JPEG_FIXTURES)
def test_jpeg_fixtures_single(rel):
    check_single(m.CODEC_MJPEG, fixture(rel), rel)


@pytest.mark.parametrize("rel", DV_FIXTURES)
def test_dv_fixtures_single(rel):
    check_single(m.CODEC_DV, fixture(rel), rel)


def test_fixtures_match_pinned_oracle_checksums():
    pinned = json.load(open(os.path.join(GOLDEN, "oracle_outputs.json")))
    for rel in JPEG_FIXTURES + DV_FIXTURES:
        codec = m.CODEC_MJPEG if rel.startswith("jpeg") else m.CODEC_DV
        st, msg, planes, _ = gpu_single(codec, fixture(rel))
        assert st == pinned[rel]["status"], rel
        if st == 0:
            assert [[w, h, hashlib.sha256(b).hexdigest()] for w, h, b in planes] == pinned[rel]["planes"], rel


def test_fixtures_batch_planar_and_rgb(ctx):
    jp = [fixture(r) for r in JPEG_FIXTURES]
    dv = [fixture(r) for r in DV_FIXTURES]
    for out in (m.OUTPUT_PLANAR, m.OUTPUT_RGB24):
        check_batch(ctx, m.CODEC_MJPEG, jp, "jpeg fixtures", out)
        check_batch(ctx, m.CODEC_DV, dv, "dv fixtures", out)


def test_c_caller_smoke(tmp_path):
    exe = tmp_path / "smoke_decode"
    subprocess.run(["gcc", "-std=c11", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "smoke_decode.c"), "-o", str(exe), _lib.LIB_PATH,
                    f"-Wl,-rpath,{os.path.dirname(_lib.LIB_PATH)}"], check=True)
    for codec, rel in [("mjpeg", "jpeg/valid/baseline-420.jpg"), ("dv", DV_FIXTURES[0])]:
        out = subprocess.run([str(exe), codec, os.path.join(GOLDEN, rel)], capture_output=True, text=True, check=True).stdout
        data = fixture(rel)
        ref = oracle.jpeg_decode(data) if codec == "mjpeg" else oracle.dv_decode(data)

        def fnv(b):
            h = 1469598103934665603
            for x in b:
                h = ((h ^ x) * 1099511628211) & (2 ** 64 - 1)
            return f"{h:016x}"
        for i, (w, h, b) in enumerate(ref.frame.planes):
            assert f"plane {i} {w}x{h} {fnv(b)}" in out, out


# ------------------------------------------------------------------ synthetic workloads (small counts)

def test_mjpeg_640x480_420_q75_no_restart(ctx):
    packets = synth.mjpeg_stream(101, 3, 640, 480, "420", 75, 0)
    check_batch(ctx, m.CODEC_MJPEG, packets, "640x480")
    check_single(m.CODEC_MJPEG, packets[0], "640x480 single")


def test_mjpeg_1080p_422_q90_restart_row_rgb(ctx):
    packets = synth.mjpeg_stream(102, 2, 1920, 1080, "422", 90, 120)
    check_batch(ctx, m.CODEC_MJPEG, packets, "1080p rgb", m.OUTPUT_RGB24)
    check_batch(ctx, m.CODEC_MJPEG, packets[:1], "1080p planar")


@pytest.mark.parametrize("pal", [False, True])
def test_dv_synthetic_88_and_248(ctx, pal):
    packets = synth.dv_stream(103, 3, pal=pal)
    check_batch(ctx, m.CODEC_DV, packets, "dv")
    check_batch(ctx, m.CODEC_DV, packets[:1], "dv rgb", m.OUTPUT_RGB24)


def _dv_content(kind: str, pal: bool, seed: int):
    """Frames that push the DV encoder's bits through every spill level: noise as
    strong as the encoder still fits (blocks overflow into the macroblock and segment
    pools), flat (nothing spills), one-sample checkerboards and 8-sample stripes
    (every block dense or one-sided)."""
    w, h = 720, (576 if pal else 480)
    cw, ch = (360, 288) if pal else (180, 480)
    rng = np.random.Generator(np.random.PCG64(seed))
    yy, xx = np.mgrid[0:h, 0:w]
    cy, cx = np.mgrid[0:ch, 0:cw]
    if kind == "noise":
        planes = [128 + rng.integers(-12, 13, (h, w)), 128 + rng.integers(-12, 13, (ch, cw)),
                  128 + rng.integers(-12, 13, (ch, cw))]
    elif kind == "flat":
        planes = [np.full((h, w), 120), np.full((ch, cw), 100), np.full((ch, cw), 150)]
    elif kind == "checker":
        planes = [16 + 219 * ((yy + xx) & 1), 16 + 224 * ((cy + cx) & 1), 240 - 224 * ((cy + cx) & 1)]
    else:  # stripes
        planes = [16 + 219 * ((xx >> 3) & 1), 16 + 224 * ((cy >> 3) & 1), 128 + 0 * cx]
    planes = [np.asarray(p, dtype=np.uint8) for p in planes]
    fmt = m.YUV420P8 if pal else m.YUV411P8
    return m.VideoFrame(fmt, w, h, [m.Plane(planes[0].tobytes(), w, w, h), m.Plane(planes[1].tobytes(), cw, cw, ch),
                                    m.Plane(planes[2].tobytes(), cw, cw, ch)], m.RANGE_LIMITED)


@pytest.mark.parametrize("pal", [False, True])
def test_dv_spill_levels_extreme_content(ctx, pal):
    packets = []
    for i, kind in enumerate(("noise", "flat", "checker", "stripes")):
        frame = _dv_content(kind, pal, 120 + i)
        for mode in (m.DV_MODE_88, m.DV_MODE_ACTIVITY):
            try:
                packets.append(m.encode_dv(frame, mode))
            except m.MmrError:  # the encoder's own limit (a segment over its budget): no stream
                pass
    assert len(packets) >= 6
    check_batch(ctx, m.CODEC_DV, packets, "dv extreme")
    # the same with damaged payload bytes: errors inside the pools, with and without concealment
    rng = np.random.Generator(np.random.PCG64(130 + pal))
    bad = []
    for pkt in packets[:4]:
        b = bytearray(pkt)
        for _ in range(40):
            dif = int(rng.integers(0, len(b) // 80))
            if (dif % 150) >= 6:  # video DIF blocks keep their headers intact
                b[dif * 80 + int(rng.integers(4, 80))] ^= 1 << int(rng.integers(0, 8))
        bad.append(bytes(b))
    check_batch(ctx, m.CODEC_DV, bad, "dv extreme damaged")
    check_batch(ctx, m.CODEC_DV, bad, "dv extreme damaged conceal", conceal=True)
    report("dv spill levels", frames=len(packets) + 2 * len(bad))


@pytest.mark.parametrize("pal", [False, True])
def test_dv_every_class_quantiser_and_mode(ctx, pal):
    """Frames whose macroblock quantisation numbers and block classes and modes are set
    at random (helpers.dv_restamped): the dequantisation through every QUANT_SHIFTS
    row, class offset and the class-3 shift (decoder.rs:290-310), 8-8 and 2-4-8 blocks
    of every class mixed in each macroblock."""
    rng = np.random.Generator(np.random.PCG64(140 + pal))
    packets = [dv_restamped(f, rng) for f in synth.dv_stream(141 + pal, 2, pal=pal)]
    check_batch(ctx, m.CODEC_DV, packets, "dv restamped")
    check_batch(ctx, m.CODEC_DV, packets[:1], "dv restamped rgb", m.OUTPUT_RGB24)
    report("dv classes and quantisers", frames=len(packets))


def test_mixed_sizes_subsampling_quality_restart(ctx):
    rng = np.random.Generator(np.random.PCG64(104))
    packets = []
    for i in range(10):
        w = int(rng.integers(1, 40)) * 8 + int(rng.integers(0, 8))
        h = int(rng.integers(1, 30)) * 8 + int(rng.integers(0, 8))
        sub = ["420", "422", "444"][i % 3]
        q = int(rng.integers(50, 96))
        _, sx, sy = synth.SUBSAMPLING[sub]
        row = (w + 8 * sx - 1) // (8 * sx)
        ri = [0, row, 4, 1][i % 4]
        packets.append(m.encode_jpeg(synth.mjpeg_frame(104, i, w, h, sub), q, annex_k=bool(i % 2), restart_interval=ri))
    gray = m.VideoFrame(m.GRAY8, 37, 21, [m.Plane(bytes(range(37 * 21 % 256)) * 4, 37, 37, 21)], m.RANGE_FULL)
    gray.planes[0] = m.Plane(bytes((x * 7) % 256 for x in range(37 * 21)), 37, 37, 21)
    packets.append(m.encode_jpeg(gray, 60, restart_interval=3))
    check_batch(ctx, m.CODEC_MJPEG, packets, "mixed")
    check_batch(ctx, m.CODEC_MJPEG, packets, "mixed rgb", m.OUTPUT_RGB24)


# ------------------------------------------------------------------ crafted edge cases

def _gray(w=16, h=8, blocks=None, **kw):
    blocks = blocks if blocks is not None else [(5, [(0, 3), (2, -2)], True), (-3, [], True)]
    return jpeg(w, h, [(1, 1, 1, 0)], entropy=stuff(encode_blocks(blocks).raw_bytes()), **kw)


def crafted_cases():
    cases = {}
    cases["ok"] = _gray()
    # ZRL landing exactly on index 64 ends the block without EOB (decoder.rs:527-531)
    cases["zrl_to_64"] = _gray(16, 8, [(0, [(0, 1)] * 47 + [(0xF0, 0)], False), (1, [], True)])
    cases["run_to_64"] = _gray(8, 8, [(0, [(0, 1)] + [(0xF0, 0)] * 3 + [(14, 1)], False)])
    cases["last_coefficient_63"] = _gray(16, 8, [(0, [(0, 1)] + [(0xF0, 0)] * 3 + [(13, 1)], False), (2, [], True)])
    cases["zrl_past_64"] = _gray(8, 8, [(0, [(0, 1)] * 50 + [(0xF0, 0)], False)])
    cases["run_past_63"] = _gray(8, 8, [(0, [(0, 1)] * 60 + [(5, 1)], False)])
    cases["dc_category_12"] = jpeg(8, 8, [(1, 1, 1, 0)], dht=[(0, 0, [0, 0, 0, 13] + [0] * 12, list(range(13))),
                                                             (1, 0, *SIMPLE_AC)],
                                   entropy=bytes([0b11000000, 0xFF, 0x00]))
    # AC table whose second 2-bit code (01) is the symbol 0x30 (run 3, size 0): DC 0000, AC 01
    cases["ac_zero_size"] = jpeg(8, 8, [(1, 1, 1, 0)], dht=[(0, 0, *SIMPLE_DC), (1, 0, [0, 4] + [0] * 14, [0x00, 0x30, 0xF0, 0x01])],
                                 entropy=bytes([0b00000111]))
    cases["ac_category_11"] = jpeg(8, 8, [(1, 1, 1, 0)], dht=[(0, 0, *SIMPLE_DC),
                                                             (1, 0, [0, 0, 0, 0, 0, 0, 0, 3] + [0] * 8, [0, 0x0B, 0x01])],
                                   entropy=bytes([0x00, 0x1F, 0xFF, 0x00]))  # DC 0000, AC 00000001 -> size 11
    cases["truncated_data"] = _gray(8, 8, [(0, [(0, 5)] * 30, True)])[:-40] + b"\xff\xd9"
    cases["no_code_16_bits"] = jpeg(8, 8, [(1, 1, 1, 0)], dht=[(0, 0, [1] + [0] * 15, [0]), (1, 0, [1] + [0] * 15, [0])],
                                    entropy=bytes([0b01111111, 0xFF, 0x00, 0xFF, 0x00, 0xFF, 0x00]))
    # restart handling (entropy.rs:111-134)
    blocks = [(3, [(0, 1)], True), (4, [], True), (-2, [(1, 2)], True), (1, [], True)]
    parts = [stuff(encode_blocks([b]).raw_bytes()) for b in blocks]
    rst = lambda n: bytes([0xFF, 0xD0 + n])
    cases["restart_ok"] = jpeg(32, 8, [(1, 1, 1, 0)], dri=1, entropy=parts[0] + rst(0) + parts[1] + rst(1) + parts[2] + rst(2) + parts[3])
    cases["restart_fill_ff"] = jpeg(32, 8, [(1, 1, 1, 0)], dri=1, entropy=parts[0] + b"\xff\xff\xd0" + parts[1] + rst(1) + parts[2] + rst(2) + parts[3])
    cases["restart_wrong_number"] = jpeg(32, 8, [(1, 1, 1, 0)], dri=1, entropy=parts[0] + rst(0) + parts[1] + rst(5) + parts[2] + rst(2) + parts[3])
    cases["restart_missing"] = jpeg(32, 8, [(1, 1, 1, 0)], dri=1, entropy=parts[0] + rst(0) + parts[1] + parts[2] + rst(2) + parts[3])
    cases["restart_extra_data"] = jpeg(32, 8, [(1, 1, 1, 0)], dri=1, entropy=parts[0] + b"\x12" + rst(0) + parts[1] + rst(1) + parts[2] + rst(2) + parts[3])
    cases["restart_stuffed_before"] = jpeg(32, 8, [(1, 1, 1, 0)], dri=1, entropy=parts[0] + b"\xff\x00" + rst(0) + parts[1] + rst(1) + parts[2] + rst(2) + parts[3])
    cases["restart_trailing_extra"] = jpeg(32, 8, [(1, 1, 1, 0)], dri=1, entropy=parts[0] + rst(0) + parts[1] + rst(1) + parts[2] + rst(2) + parts[3] + rst(3) + b"\x55" + rst(4))
    cases["restart_inside_data"] = jpeg(32, 8, [(1, 1, 1, 0)], dri=2, entropy=parts[0] + rst(0) + parts[1] + rst(1) + parts[2] + parts[3])
    cases["rst_in_unrestarted_scan"] = jpeg(32, 8, [(1, 1, 1, 0)], entropy=parts[0] + rst(0) + parts[1] + parts[2] + parts[3])
    cases["ri_larger_than_image"] = jpeg(32, 8, [(1, 1, 1, 0)], dri=100, entropy=b"".join(parts))
    # markers and structure
    cases["second_scan"] = cases["ok"][:-2] + jpeg(16, 8, [(1, 1, 1, 0)], entropy=b"\x00")[2:]
    cases["app14_rgb_in_tail"] = jpeg(16, 16, [(1, 2, 2, 0), (2, 1, 1, 0), (3, 1, 1, 0)],
                                      entropy=stuff(encode_blocks([(1, [], True)] * 6).raw_bytes()),
                                      tail=b"\xff\xee\x00\x0eAdobe\x00\x64\x00\x00\x00\x00\x00\xff\xd9")
    cases["sof_after_sos"] = jpeg(16, 8, [(1, 1, 1, 0)], sof=False, entropy=stuff(encode_blocks([(2, [], True)] * 2).raw_bytes()),
                                  tail=b"\xff\xc0\x00\x0b\x08\x00\x08\x00\x10\x01\x01\x11\x00\xff\xd9")
    cases["missing_quant"] = _gray(quant={1: [1] * 64})
    cases["missing_ac_table"] = jpeg(8, 8, [(1, 1, 1, 0)], dht=[(0, 0, *SIMPLE_DC)], entropy=b"\x00")
    cases["oversubscribed"] = jpeg(8, 8, [(1, 1, 1, 0)], dht=[(0, 0, [3] + [0] * 15, [0, 1, 2]), (1, 0, *SIMPLE_AC)], entropy=b"\x00")
    cases["quant16"] = jpeg(8, 8, [(1, 1, 1, 0)], quant={}, extra_before_sos=b"\xff\xdb\x00\x83\x10" + b"\x00\x01" * 64, entropy=b"\x00")
    cases["dnl_height"] = jpeg(8, 0, [(1, 1, 1, 0)], entropy=b"\x00")
    cases["dup_ids_panic"] = jpeg(8, 8, [(1, 1, 1, 0), (1, 1, 1, 0)], scan=[(1, 0, 0), (5, 0, 0)], entropy=b"\x00")
    cases["four_components"] = jpeg(16, 16, [(1, 1, 1, 0), (2, 1, 1, 0), (3, 1, 1, 0), (4, 1, 1, 0)],
                                    entropy=stuff(encode_blocks([(i % 5 - 2, [(0, 1)], True) for i in range(16)]).raw_bytes()))
    cases["two_components"] = jpeg(16, 8, [(1, 2, 1, 0), (2, 1, 1, 0)],
                                   entropy=stuff(encode_blocks([(1, [], True)] * 3).raw_bytes()))
    cases["sampling_3_1_1"] = jpeg(24, 8, [(1, 3, 1, 0), (2, 1, 1, 0), (3, 1, 1, 0)],
                                   entropy=stuff(encode_blocks([(2, [(0, 1)], True)] * 5).raw_bytes()))
    cases["odd_size_420"] = jpeg(17, 9, [(1, 2, 2, 0), (2, 1, 1, 0), (3, 1, 1, 0)],
                                 entropy=stuff(encode_blocks([(i % 3, [(1, -1)], True) for i in range(24)]).raw_bytes()))
    # pred grows by 2047 per block; pred * 255 leaves i32 after 4114 blocks (decoder.rs:511-514)
    cases["dc_dequant_overflow"] = jpeg(8 * 4200, 8, [(1, 1, 1, 0)], quant={0: [255] * 64},
                                        entropy=stuff(encode_blocks([(2047, [], True)] * 4200).raw_bytes()))
    cases["empty"] = b""
    cases["soi_only"] = b"\xff\xd8"
    cases["eoi_no_scan"] = b"\xff\xd8\xff\xd9"
    return cases


@pytest.mark.parametrize("name", sorted(crafted_cases()))
def test_crafted_edge_case(name):
    data = crafted_cases()[name]
    check_single(m.CODEC_MJPEG, data, name)


def test_crafted_cases_in_one_batch(ctx):
    cases = crafted_cases()
    check_batch(ctx, m.CODEC_MJPEG, [cases[k] for k in sorted(cases)], "crafted batch")


def test_idct_ties_and_clamps_through_streams(ctx):
    # DC-only blocks over a range of dequantised DC values, including the x.5 ties (dc = 4 mod 8)
    # consecutive differences stay within DC category 11 (|diff| <= 2047)
    blocks = [(d, [], True) for d in [4, -4, 0, 1, 8, 12, -1024, 0, 1020, 1023, 0, -1023, 0, 2047, 2043, 20]]
    diffs, prev = [], 0
    for d, a, e in blocks:
        diffs.append((d - prev, a, e))
        prev = d
    data = jpeg(8 * len(blocks), 8, [(1, 1, 1, 0)], entropy=stuff(encode_blocks(diffs).raw_bytes()))
    check_single(m.CODEC_MJPEG, data, "dc ladder")
    # dense blocks of large alternating coefficients with quantiser 255 (saturating samples)
    acs = [(0, ((-1) ** k) * (500 + k)) for k in range(40)]
    data = jpeg(8, 8, [(1, 1, 1, 0)], quant={0: [255] * 64}, entropy=stuff(encode_blocks([(3, acs, True)]).raw_bytes()))
    check_single(m.CODEC_MJPEG, data, "dense saturating")


def _pad_entropy(packet: bytes, pad: int) -> bytes:
    """Inserts `pad` zero bytes after the last MCU's data (ignored by the decoder) before EOI."""
    return packet[:-2] + bytes(pad) + packet[-2:]


def test_terminator_on_scan_tile_boundaries(ctx):
    # The marker scan works on 4096-byte tiles starting at the 16-byte boundary below the
    # first entropy byte; a terminator on a tile's first byte (or one byte either side)
    # must still yield the right token and restart-marker totals.
    packets = []
    for base in synth.mjpeg_stream(113, 2, 160, 120, "420", 85, 0) + synth.mjpeg_stream(114, 1, 160, 128, "422", 85, 10):
        st, _, info = oracle.jpeg_parse(base)
        ds = info["data_offset"]
        term = ds + info["data_length"]
        need = (4096 - (term - (ds & ~15)) % 4096) % 4096
        for delta in (-1, 0, 1, 4096):
            if need + delta >= 0:
                packets.append(_pad_entropy(base, need + delta))
    check_batch(ctx, m.CODEC_MJPEG, packets, "tile boundary")


# ------------------------------------------------------------------ seeded corruption

def test_corrupted_mjpeg_streams_match_oracle(ctx):
    rnd = random.Random(105)
    bases = synth.mjpeg_stream(106, 2, 96, 64, "420", 80, 0) + synth.mjpeg_stream(107, 2, 96, 64, "422", 80, 6)
    bases.append(fixture("jpeg/valid/baseline-420.jpg"))
    packets = []
    for k in range(120):
        d = bytearray(bases[k % len(bases)])
        kind = k % 4
        if kind == 0:
            for _ in range(rnd.randint(1, 4)):
                d[rnd.randrange(len(d))] = rnd.randrange(256)
        elif kind == 1:
            d = d[: rnd.randrange(len(d))]
        elif kind == 2:
            p = rnd.randrange(len(d))
            d[p:p] = bytes([0xFF, rnd.choice([0x00, 0xD0 + rnd.randrange(8), 0xD9, 0xFF, 0xC4])])
        else:
            p = rnd.randrange(len(d))
            del d[p:p + rnd.randint(1, 8)]
        packets.append(bytes(d))
    check_batch(ctx, m.CODEC_MJPEG, packets, "corrupt")


def test_corrupted_dv_frames_match_oracle(ctx):
    rnd = random.Random(108)
    base = synth.dv_stream(109, 1)[0]
    packets = []
    for k in range(12):
        d = bytearray(base)
        for _ in range(rnd.randint(1, 40)):
            d[rnd.randrange(len(d))] = rnd.randrange(256)
        packets.append(bytes(d))
    check_batch(ctx, m.CODEC_DV, packets, "dv corrupt")
    check_batch(ctx, m.CODEC_DV, packets, "dv corrupt concealed", conceal=True)


# dv/tests/reference_vectors.rs:48-64 damaged_video_segment_can_be_reported_and_concealed
def test_dv_damage_reported_and_concealed(ctx):
    damaged = bytearray(fixture(DV_FIXTURES[0]))
    damaged[7 * 80] = 0x76
    check_single(m.CODEC_DV, bytes(damaged), "damaged")
    (r, payload), = ctx.decode_batch([bytes(damaged)], m.CODEC_DV, conceal=True)
    ref = oracle.dv_decode(bytes(damaged), conceal=True)
    assert r.status == 0 and r.concealed_segments == 1 and ref.concealed == [(0, 0)]
    assert_same_decode(0, "", frame_planes_gpu(m.frame_from_batch(r, payload)), ref, "concealed")


# ------------------------------------------------------------------ composition

def test_same_alone_and_in_the_mix(ctx):
    jp = synth.mjpeg_stream(110, 3, 320, 240, "422", 85, 20) + [fixture("jpeg/valid/baseline-420.jpg")]
    dv = synth.dv_stream(111, 2)
    alone = [ctx.decode_batch([p], m.CODEC_MJPEG)[0] for p in jp] + [ctx.decode_batch([p], m.CODEC_DV)[0] for p in dv]
    mixed = ctx.decode_batch(jp + dv, [m.CODEC_MJPEG] * len(jp) + [m.CODEC_DV] * len(dv))
    for (ra, pa), (rb, pb) in zip(alone, mixed):
        assert ra.status == rb.status == 0 and pa == pb


def test_trait_decoder_batched_matches_single():
    packets = synth.mjpeg_stream(112, 5, 64, 48, "420", 70, 0)
    packets.insert(2, b"\xff\xd8garbage")
    single, batched = m.MjpegDecoder(), m.MjpegDecoder(batch=3)
    for d in (single, batched):
        d.configure(m.CodecDescriptor(m.MJPEG_CODEC_NAME))
    out_s, out_b = [], []
    for i, p in enumerate(packets):
        try:
            single.send_packet(m.Packet(p, pts=i))
            out_s.append(single.receive_frame())
        except m.MmrError as e:
            out_s.append(e.status)
        batched.send_packet(m.Packet(p, pts=i))
    batched.flush()
    while True:
        try:
            f = batched.receive_frame()
        except m.MmrError as e:
            out_b.append(e.status)
            continue
        if f is None:
            break
        out_b.append(f)
    assert len(out_s) == len(out_b)
    for a, b in zip(out_s, out_b):
        if isinstance(a, int):
            assert a == b
        else:
            assert a.pts == b.pts and [p.data for p in a.planes] == [p.data for p in b.planes]
