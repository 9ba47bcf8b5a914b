"""The engine's Huffman lookup records (mmrecode_gb300/csrc/huffman_lut.h) checked entry by
entry against a canonical decode written here from the JPEG rules (entropy.rs:18-70
builds the canonical code; decoder.rs:501-546 the symbol checks; receive_extend
entropy.rs:168-182): the 9-bit code table, the 11-bit whole-symbol / code-only table
and the two-symbol table of the sync passes. Tables come from the oracle encoder's
streams (Annex K and the reference encoder's own tables) and from seeded random
canonical codes with codes up to 16 bits."""
import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle

ROOT = Path(__file__).resolve().parents[1]
FB = 11
K_EOB, K_CODE = 1 << 12, 1 << 13
K_PAIR = K_EOB | K_CODE


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no g++")
    so = tmp_path_factory.mktemp("lut") / "lut_harness.so"
    subprocess.run([gxx, "-O1", "-shared", "-fPIC", "-std=c++17", f"-I{ROOT / 'mmrecode_gb300' / 'csrc'}",
                    "-o", str(so), str(ROOT / "tests" / "cuda" / "lut_harness.cpp")], check=True)
    lib = ctypes.CDLL(str(so))
    lib.mmr_test_lut_size.restype = ctypes.c_size_t
    lib.mmr_test_build_lut.argtypes = [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_size_t]
    return lib


def build(lib, key: bytes, ac: bool):
    size = lib.mmr_test_lut_size()
    buf = (ctypes.c_uint8 * size)()
    assert lib.mmr_test_build_lut(key, len(key), 1 if ac else 0, buf, size) == 0
    raw = bytes(buf)
    fast = np.frombuffer(raw, dtype=np.uint16, count=512, offset=0)
    fastv = np.frombuffer(raw, dtype=np.uint32, count=1 << FB, offset=1024)
    fastp = np.frombuffer(raw, dtype=np.uint32, count=1 << FB, offset=1024 + 4 * (1 << FB))
    return fast, fastv, fastp


def codes_of(key: bytes):
    """(length, code) -> symbol of the canonical code (JPEG Annex C)."""
    counts, syms = key[:16], key[16:]
    out, code, k = {}, 0, 0
    for length in range(1, 17):
        for _ in range(counts[length - 1]):
            out[(length, code)] = syms[k]
            code += 1
            k += 1
        code <<= 1
    return out


def first_code(codes, bits: int, nbits: int, max_len: int):
    """The code at the top of an nbits-wide bit string, of at most max_len bits."""
    for length in range(1, min(max_len, nbits) + 1):
        sym = codes.get((length, bits >> (nbits - length)))
        if sym is not None:
            return length, sym
    return None


def extend(v: int, size: int) -> int:
    return v + 1 - (1 << size) if size and v < (1 << (size - 1)) else v


def whole(codes, bits: int, nbits: int, ac: bool):
    """(entry kind, total bits, advance, eob, value) of the symbol at the top of bits,
    as the fast tables record it, or None where they leave it to the slow path."""
    found = first_code(codes, bits, nbits, FB)
    if found is None:
        return None
    length, sym = found
    if ac:
        if sym == 0x00:
            size, adv, eob = 0, 0, True
        elif sym == 0xF0:
            size, adv, eob = 0, 16, False
        else:
            size, adv, eob = sym & 15, (sym >> 4) + 1, False
            if not 1 <= size <= 10:
                return None
    else:
        size, adv, eob = sym, 1, False
        if size > 11:
            return None
    if length + size > nbits:
        return ("code", length, adv, eob, size)
    mag = (bits >> (nbits - length - size)) & ((1 << size) - 1) if size else 0
    return ("whole", length + size, adv, eob, extend(mag, size))


def expected_fastv(codes, x: int, ac: bool) -> int:
    w = whole(codes, x, FB, ac)
    if w is None:
        return 0
    kind, total, adv, eob, v = w
    if kind == "code":
        return (v << 16) | K_CODE | (adv << 5) | total  # (v holds the size, total the code length)
    return (((v & 0xFFFF) << 16) | (K_EOB if eob else 0) | (adv << 5) | total) & 0xFFFFFFFF


def expected_fastp(codes, x: int, ac: bool, single: int) -> int:
    if not ac:
        return single
    w1 = whole(codes, x, FB, ac)
    if w1 is None or w1[0] != "whole" or w1[3]:
        return single
    _, l1, adv1, _, v1 = w1
    if l1 + 2 > FB or not -64 <= v1 <= 63:
        return single
    rest = FB - l1
    w2 = whole(codes, x & ((1 << rest) - 1), rest, ac)
    if w2 is None or w2[0] != "whole":
        return single
    _, l2, adv2, eob2, v2 = w2
    if not -32 <= v2 <= 31:
        return single
    adv2 = 0 if eob2 else adv2
    return (((v2 & 63) << 26) | ((v1 & 127) << 19) | (adv2 << 14) | K_PAIR | (adv1 << 5) | (l1 + l2)) & 0xFFFFFFFF


def check_table(lib, key: bytes, ac: bool):
    fast, fastv, fastp = build(lib, key, ac)
    codes = codes_of(key)
    for x in range(512):
        found = first_code(codes, x, 9, 9)
        want = (found[0] << 8) | found[1] if found else 0
        assert int(fast[x]) == want, (x, int(fast[x]), want)
    pairs = 0
    for x in range(1 << FB):
        want = expected_fastv(codes, x, ac)
        assert int(fastv[x]) == want, (ac, x, hex(int(fastv[x])), hex(want))
        wantp = expected_fastp(codes, x, ac, want)
        assert int(fastp[x]) == wantp, (ac, x, hex(int(fastp[x])), hex(wantp))
        pairs += int(wantp) != int(want)
    return pairs


def dht_tables(jpeg: bytes):
    """(key, is_ac) of every DHT table in a JPEG stream."""
    out, i = [], 2
    while i + 4 <= len(jpeg) and jpeg[i] == 0xFF:
        marker = jpeg[i + 1]
        length = (jpeg[i + 2] << 8) | jpeg[i + 3]
        seg = jpeg[i + 4:i + 2 + length]
        if marker == 0xC4:
            p = 0
            while p < len(seg):
                tc = seg[p] >> 4
                n = sum(seg[p + 1:p + 17])
                out.append((bytes(seg[p + 1:p + 17 + n]), tc == 1))
                p += 17 + n
        if marker == 0xDA:
            break
        i += 2 + length
    return out


def test_tables_of_the_encoders_streams(harness):
    rng = np.random.default_rng(11)
    w, h = 64, 48
    planes = [(w, h, rng.integers(0, 256, (h, w), dtype=np.uint8).tobytes()),
              (w // 2, h // 2, rng.integers(0, 256, (h // 2, w // 2), dtype=np.uint8).tobytes()),
              (w // 2, h // 2, rng.integers(0, 256, (h // 2, w // 2), dtype=np.uint8).tobytes())]
    seen, pairs = set(), 0
    for annex_k in (True, False):
        for quality in (50, 90, 100):
            jpeg = oracle.jpeg_encode(2, w, h, planes, quality, annex_k=annex_k)  # 4:2:0
            for key, ac in dht_tables(jpeg):
                if (key, ac) in seen:
                    continue
                seen.add((key, ac))
                pairs += check_table(harness, key, ac)
    assert len(seen) >= 4
    assert pairs > 0  # the AC tables do hold pairs


def random_key(rng, nsym: int, ac: bool) -> bytes:
    """A canonical code with nsym symbols and lengths up to 16 (Kraft sum <= 1)."""
    lengths = sorted(int(x) for x in rng.integers(2, 17, nsym))
    while sum(2.0 ** -x for x in lengths) > 1.0:  # lengthen the shortest codes until they fit
        i = next(j for j, x in enumerate(lengths) if x < 16)
        lengths[i] += 1
        lengths.sort()
    lengths = np.array(lengths)
    counts = [int((lengths == length).sum()) for length in range(1, 17)]
    if ac:  # valid symbols, then ones the decoder rejects (size 11..15, zero size but not EOB/ZRL)
        pool = [0x00, 0xF0] + [(r << 4) | s for r in range(16) for s in range(1, 11)]
        pool += [(r << 4) | s for r in (0, 3) for s in range(11, 16)] + [r << 4 for r in (1, 7, 14)]
    else:  # sizes 12..15 are rejected
        pool = list(range(16))
    syms = list(rng.choice(pool, size=min(nsym, len(pool)), replace=False))
    return bytes(counts) + bytes(int(s) for s in syms)


@pytest.mark.parametrize("seed", range(6))
def test_random_canonical_codes(harness, seed):
    rng = np.random.default_rng(100 + seed)
    check_table(harness, random_key(rng, 16, False), False)
    check_table(harness, random_key(rng, int(rng.integers(20, 160)), True), True)
