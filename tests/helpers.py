"""Shared test helpers: fixtures, Y4M reading, a JPEG assembler for crafted
edge-case streams, and GPU-vs-oracle comparison."""

from __future__ import annotations

import os
import struct

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# counts the parity tests report (frames, blocks, near ties, exact-path samples);
# tests/conftest.py prints them in the terminal summary
REPORTS: list = []


def report(name: str, **counts) -> None:
    REPORTS.append((name, counts))


def fixture(rel: str) -> bytes:
    with open(os.path.join(GOLDEN, rel), "rb") as f:
        return f.read()


JPEG_FIXTURES = [
    "jpeg/valid/baseline-420.jpg",
    "jpeg/valid/minimal-gray.jpg",
    "jpeg/valid/unknown-app-marker.jpg",
    "jpeg/valid/restart-interval.jpg",
    "jpeg/parser/stuffed-restarts.jpg",
    "jpeg/invalid/invalid-length.jpg",
    "jpeg/invalid/missing-eoi.jpg",
    "jpeg/invalid/truncated-marker.jpg",
    "jpeg/encoded/mmrecode-q85-420.mjpg",
]
DV_FIXTURES = ["dv/valid/dv25-525-60-one-frame.dv", "dv/valid/dv25-625-50-one-frame.dv"]


def read_y4m_420(data: bytes):
    """Frames of a 4:2:0 Y4M stream as (Y, Cb, Cr) byte strings (crates/containers/y4m)."""
    header, rest = data.split(b"\n", 1)
    fields = header.split()
    w = int([f for f in fields if f.startswith(b"W")][0][1:])
    h = int([f for f in fields if f.startswith(b"H")][0][1:])
    cw, ch = (w + 1) // 2, (h + 1) // 2
    frames = []
    while rest.startswith(b"FRAME"):
        _, rest = rest.split(b"\n", 1)
        y, rest = rest[: w * h], rest[w * h:]
        cb, rest = rest[: cw * ch], rest[cw * ch:]
        cr, rest = rest[: cw * ch], rest[cw * ch:]
        frames.append((w, h, y, cb, cr))
    return frames



def dv_restamped(frame, rng):
    """Every macroblock's quantisation number (byte 3, low nibble) and every block's
    mode bit and class (bits 9..11 of its region) set at random: the VLC parse is
    unchanged, the dequantisation runs through every QUANT_SHIFTS row, class offset
    and class-3 shift, and 8-8 and 2-4-8 blocks mix in every macroblock."""
    b = bytearray(frame)  # frames of intact DIF structure (120000 or 144000 bytes)
    starts = np.cumsum((0, 112, 112, 112, 112, 80))
    for seq in range(len(frame) // 12000):
        for vn in range(135):
            base = (seq * 150 + 7 + (vn // 15) * 16 + vn % 15) * 80
            b[base + 3] = (b[base + 3] & 0xF0) | int(rng.integers(0, 16))
            for start in starts:
                for off, bit in zip(range(9, 12), rng.integers(0, 2, 3)):
                    pos = 32 + int(start) + off
                    mask = 0x80 >> (pos & 7)
                    b[base + pos // 8] = (b[base + pos // 8] & ~mask) | (mask if bit else 0)
    return bytes(b)

# ------------------------------------------------------------------ JPEG assembly

class BitWriter:
    def __init__(self):
        self.bits: list[int] = []

    def put(self, value: int, count: int):
        for s in range(count - 1, -1, -1):
            self.bits.append((value >> s) & 1)

    def raw_bytes(self, pad_bit: int = 1) -> bytes:
        b = list(self.bits)
        while len(b) % 8:
            b.append(pad_bit)
        return bytes(int("".join(map(str, b[i:i + 8])), 2) for i in range(0, len(b), 8))


def stuff(data: bytes) -> bytes:
    out = bytearray()
    for x in data:
        out.append(x)
        if x == 0xFF:
            out.append(0)
    return bytes(out)


def segment(marker: int, payload: bytes) -> bytes:
    return bytes([0xFF, marker]) + struct.pack(">H", len(payload) + 2) + payload


def canonical_codes(counts, symbols):
    """symbol -> (code, length) of a canonical table (entropy.rs:18-55)."""
    codes, code, k = {}, 0, 0
    for length in range(1, 17):
        for _ in range(counts[length - 1]):
            codes.setdefault(symbols[k], (code, length))
            code += 1
            k += 1
        code <<= 1
    return codes


SIMPLE_DC = ([0, 0, 0, 12] + [0] * 12, list(range(12)))
SIMPLE_AC = ([0] * 7 + [162] + [0] * 8, [0x00, 0xF0] + [(r << 4) | s for r in range(16) for s in range(1, 11)])


def jpeg(width, height, comps, scan=None, quant=None, dht=None, dri=None, entropy=b"", tail=b"\xff\xd9",
         jfif=True, extra_before_sos=b"", sof=True):
    """Assembles SOI [JFIF] DQT SOF0 DHT [DRI] ... SOS entropy tail.

    comps: list of (id, h, v, tq); scan: list of (selector, td, ta) (default: all comps, tables 0);
    quant: {id: 64 zigzag values}; dht: list of (class, id, counts, symbols)."""
    quant = quant or {0: [1] * 64, 1: [1] * 64, 2: [1] * 64, 3: [1] * 64}
    dht = dht if dht is not None else [(0, 0, *SIMPLE_DC), (1, 0, *SIMPLE_AC)]
    scan = scan if scan is not None else [(c[0], 0, 0) for c in comps]
    out = b"\xff\xd8"
    if jfif:
        out += segment(0xE0, b"JFIF\x00\x01\x02\x00\x00\x01\x00\x01\x00\x00")
    for q, vals in quant.items():
        out += segment(0xDB, bytes([q]) + bytes(vals))
    if sof:
        p = bytes([8]) + struct.pack(">HH", height, width) + bytes([len(comps)])
        for cid, h, v, tq in comps:
            p += bytes([cid, (h << 4) | v, tq])
        out += segment(0xC0, p)
    for cls, tid, counts, symbols in dht:
        out += segment(0xC4, bytes([(cls << 4) | tid]) + bytes(counts) + bytes(symbols))
    if dri is not None:
        out += segment(0xDD, struct.pack(">H", dri))
    out += extra_before_sos
    p = bytes([len(scan)])
    for sel, td, ta in scan:
        p += bytes([sel, (td << 4) | ta])
    p += bytes([0, 63, 0])
    out += segment(0xDA, p)
    return out + entropy + tail


def encode_blocks(blocks, dc_table=SIMPLE_DC, ac_table=SIMPLE_AC):
    """Entropy-codes blocks given as (dc_diff, [(run, level), ...], eob) into a BitWriter."""
    dcc = canonical_codes(*dc_table)
    acc = canonical_codes(*ac_table)
    w = BitWriter()
    for dc, acs, eob in blocks:
        cat = abs(dc).bit_length()
        code, n = dcc[cat]
        w.put(code, n)
        if cat:
            w.put(dc if dc >= 0 else dc + (1 << cat) - 1, cat)
        for run, level in acs:
            if level == 0:  # raw symbol
                code, n = acc[run]
                w.put(code, n)
                continue
            cat = abs(level).bit_length()
            code, n = acc[(run << 4) | cat]
            w.put(code, n)
            w.put(level if level >= 0 else level + (1 << cat) - 1, cat)
        if eob:
            code, n = acc[0x00]
            w.put(code, n)
    return w


# ------------------------------------------------------------------ comparison

def frame_planes_gpu(frame):
    return [(p.width, p.height, bytes(p.data)) for p in frame.planes]


def assert_same_decode(gpu_status, gpu_message, gpu_planes, ref, label=""):
    """GPU result vs oracle Result: identical status, message and every sample."""
    assert gpu_status == ref.status, f"{label}: status {gpu_status} != oracle {ref.status} ({ref.message}) [{gpu_message}]"
    if ref.status == 0:
        assert len(gpu_planes) == len(ref.frame.planes), label
        for i, ((gw, gh, gb), (rw, rh, rb)) in enumerate(zip(gpu_planes, ref.frame.planes)):
            assert (gw, gh) == (rw, rh), f"{label}: plane {i} dims"
            if gb != rb:
                a = np.frombuffer(gb, np.uint8).astype(int)
                b = np.frombuffer(rb, np.uint8).astype(int)
                bad = np.nonzero(a != b)[0]
                raise AssertionError(f"{label}: plane {i}: {len(bad)} samples differ, first at {bad[0]} "
                                     f"(gpu {a[bad[0]]}, oracle {b[bad[0]]})")


def prefixed(status: int, message: str) -> str:
    """The C ABI's message for an oracle (Rust-level) diagnostic (crates/core/src/error.rs:18-27)."""
    prefix = {1: "invalid argument: ", 2: "invalid data: ", 3: "unsupported: ", 4: "invalid state: "}
    return prefix.get(status, "") + message


# ---------------------------------------------------------------- oracle pool

def oracle_digest(job):
    """(kind, packet) -> (status, SHA-256 of the oracle's planar frame, of its RGB24 or None).
    kind: "mjpeg", "mjpeg-rgb" (also the RGB digest), "dv". Runs in pool workers."""
    import hashlib

    import oracle

    kind, packet = job
    r = oracle.dv_decode(packet) if kind == "dv" else oracle.jpeg_decode(packet)
    if r.status != 0:
        return r.status, None, None
    planar = hashlib.sha256(b"".join(p[2] for p in r.frame.planes)).hexdigest()
    rgb = hashlib.sha256(oracle.rgb24(r.frame)).hexdigest() if kind == "mjpeg-rgb" else None
    return 0, planar, rgb


def oracle_pool():
    """A process pool for the oracle, started with spawn (safe after CUDA is initialised)."""
    import multiprocessing as mp

    return mp.get_context("spawn").Pool(os.cpu_count() or 4)
