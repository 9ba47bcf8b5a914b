"""The marker parser shared by the host and the device (mmrecode_gb300/csrc/jpeg_syntax.h:
the prefix up to the first SOS, the first scan's end, the tail) against the oracle's
restatement of parse_jpeg (crates/codecs/mjpeg/src/parser.rs:18-81), on CPU: the same
outcome (status) and error offset for every input, and for valid streams the same frame size,
component count, scan count and entropy-data offset. Inputs: synthetic streams of
several layouts and restart intervals, the golden JPEG fixtures, and seeded
mutations of their marker segments (byte flips, truncations, dropped and doubled
bytes)."""
import ctypes
import re
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from mmrecode_gb300 import synth

ROOT = Path(__file__).resolve().parents[1]


class ParseOut(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("kind", ctypes.c_uint32), ("offset", ctypes.c_uint32),
                ("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("ncomp", ctypes.c_uint32),
                ("dri", ctypes.c_uint32), ("scan_count", ctypes.c_uint32), ("data_offset", ctypes.c_uint32),
                ("ended_at_eoi", ctypes.c_uint32)]


@pytest.fixture(scope="module")
def parse():
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    out_dir = Path(__import__("tempfile").mkdtemp(prefix="syntax"))
    so = out_dir / "syntax_harness.so"
    subprocess.run([gxx, "-O1", "-shared", "-fPIC", "-std=c++17", f"-I{ROOT / 'mmrecode_gb300' / 'csrc'}",
                    "-o", str(so), str(ROOT / "tests" / "cuda" / "syntax_harness.cpp")], check=True)
    lib = ctypes.CDLL(str(so))
    lib.mmr_test_parse_jpeg.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(ParseOut)]

    def run(data: bytes) -> ParseOut:
        out = ParseOut()
        lib.mmr_test_parse_jpeg(data, len(data), ctypes.byref(out))
        return out
    return run


def streams():
    out = []
    for i, (w, h, sub, q, ri) in enumerate([(64, 48, "420", 75, 0), (80, 40, "422", 90, 5), (48, 48, "444", 50, 3),
                                            (33, 17, "420", 95, 1), (120, 64, "422", 60, 0)]):
        out += synth.mjpeg_stream(300 + i, 1, w, h, sub, q, ri, annex_k=bool(i % 2))
    for rel in sorted((ROOT / "tests" / "golden" / "jpeg").rglob("*")):
        if rel.is_file() and rel.suffix.lower() in (".jpg", ".jpeg", ".mjpg"):
            out.append(rel.read_bytes())
    return out


def check(parse, data: bytes, label: str):
    got = parse(data)
    st, msg, info = oracle.jpeg_parse(data)
    assert got.status == st, f"{label}: {got.status} (kind {got.kind} at {got.offset}) vs {st} {msg}"
    at = re.search(r"0x([0-9a-f]{8})", msg)
    if st and at:  # the byte offset the reference reports
        assert got.offset == int(at.group(1), 16), f"{label}: offset {got.offset:#010x} vs {msg}"
    if st == 0:
        assert (got.width, got.height, got.ncomp) == (info["width"], info["height"], info["component_count"]), label
        assert got.scan_count == info["scan_count"], label
        if info["scan_count"]:
            assert got.data_offset == info["data_offset"], label
    return st


def test_valid_streams(parse):
    packets = streams()
    assert len(packets) >= 5
    for i, p in enumerate(packets):
        assert check(parse, p, f"valid[{i}]") == 0 or i >= 5  # fixtures may hold errors on purpose


def test_mutated_marker_segments(parse):
    rng = np.random.Generator(np.random.PCG64(7))
    outcomes = {}
    for i, p in enumerate(streams()):
        _, _, info = oracle.jpeg_parse(p)
        head = max(16, int(info["data_offset"]) or len(p))  # mutate the marker segments before the scan
        for j in range(120):
            b = bytearray(p)
            op = j % 4
            at = int(rng.integers(0, min(head, len(b))))
            if op == 0:
                b[at] ^= 1 << int(rng.integers(0, 8))
            elif op == 1:
                b = b[:at]
            elif op == 2:
                del b[at]
            else:
                b.insert(at, b[at])
            st = check(parse, bytes(b), f"mutated[{i}.{j}] op {op} at {at}")
            outcomes[st] = outcomes.get(st, 0) + 1
    assert len(outcomes) >= 2 and outcomes.get(0, 0) > 50 and outcomes.get(2, 0) > 50, outcomes
