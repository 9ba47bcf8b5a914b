"""Second restatements of reference algorithms, written in Python/numpy from the
reference source for the CPU tests that pin the oracle: the four binary64 transforms
with the reference's operation order (binary64 products and sums, never fused; Rust's
round half away from zero) and the DV25 video decode (crates/codecs/dv/src/decoder.rs).
Test infrastructure only."""
import math
import re
from pathlib import Path

import numpy as np

import adversarial

FRAC = 0.7071067811865476  # std::f64::consts::FRAC_1_SQRT_2


def rust_round(x):
    """f64::round: half away from zero (x - trunc(x) is exact in binary64)."""
    t = np.trunc(x)
    f = x - t
    return t + np.where(np.abs(f) >= 0.5, np.sign(x), 0.0)


def to_u8(x):
    return np.clip(rust_round(x), 0.0, 255.0).astype(np.uint8)


def jpeg_idct(c):
    M = adversarial.idct_matrix()
    c = np.asarray(c, np.float64)
    t = np.zeros((len(c), 64))
    for v in range(8):
        for x in range(8):
            for u in range(8):
                t[:, v * 8 + x] = t[:, v * 8 + x] + M[x, u] * c[:, v * 8 + u]
    out = np.zeros((len(c), 64), np.uint8)
    for y in range(8):
        for x in range(8):
            s = np.zeros(len(c))
            for v in range(8):
                s = s + M[y, v] * t[:, v * 8 + x]
            out[:, y * 8 + x] = to_u8(s + 128.0)
    return out


def fdct_quantize(samples, quant):
    M = adversarial.idct_matrix()
    s = np.asarray(samples, np.float64)
    q = np.asarray(quant, np.float64)
    t = np.zeros((len(s), 64))
    for y in range(8):
        for u in range(8):
            for x in range(8):
                t[:, y * 8 + u] = t[:, y * 8 + u] + M[x, u] * (s[:, y * 8 + x] - 128.0)
    out = np.zeros((len(s), 64), np.int32)
    for v in range(8):
        for u in range(8):
            value = np.zeros(len(s))
            for y in range(8):
                value = value + M[y, v] * t[:, y * 8 + u]
            out[:, v * 8 + u] = rust_round(value / q[:, v * 8 + u]).astype(np.int32)
    return out


def cos16(a, b):
    return math.cos(float(a) * float(b) * math.pi / 16.0)


def cos8(a, b):
    return math.cos(float(a) * float(b) * math.pi / 8.0)


def dv_idct88(c):
    c = np.asarray(c, np.float64)
    out = np.zeros((len(c), 64), np.uint8)
    for y in range(8):
        for x in range(8):
            s = np.zeros(len(c))
            for v in range(8):
                for u in range(8):
                    cu = FRAC if u == 0 else 1.0
                    cv = FRAC if v == 0 else 1.0
                    s = s + cu * cv * c[:, v * 8 + u] * cos16(2 * x + 1, u) * cos16(2 * y + 1, v)
            out[:, y * 8 + x] = to_u8(s / 4.0)
    return out


def dv_idct248(c):
    c = np.asarray(c, np.float64)
    b = np.zeros((len(c), 64))
    for pair in range(4):
        for u in range(8):
            first, second = c[:, pair * 16 + u], c[:, pair * 16 + 8 + u]
            b[:, pair * 16 + u] = first + second
            b[:, pair * 16 + 8 + u] = first - second
    h = np.zeros((len(c), 64))
    for row in range(8):
        for x in range(8):
            s = np.zeros(len(c))
            for u in range(8):
                cu = FRAC if u == 0 else 1.0
                s = s + cu * b[:, row * 8 + u] * cos16(2 * x + 1, u)
            h[:, row * 8 + x] = s / 2.0
    out = np.zeros((len(c), 64), np.uint8)
    for field in range(2):
        for y in range(4):
            for x in range(8):
                s = np.zeros(len(c))
                for v in range(4):
                    cv = FRAC if v == 0 else 1.0
                    s = s + cv * h[:, (v * 2 + field) * 8 + x] * cos8(2 * y + 1, v)
                out[:, (y * 2 + field) * 8 + x] = to_u8(s / 2.0)
    return out


# ------------------------------------------------------------------ DV25 video decode

_CSRC = Path(__file__).resolve().parents[1] / "mmrecode_gb300" / "csrc" / "tables.h"


def _table(name):
    """An initializer list of the library's tables.h (the reference's tables.rs data)."""
    text = _CSRC.read_text()
    body = re.search(r"#define " + name + r"\s+\\?\s*\{([^}]*)\}", text).group(1)
    return [int(v) for v in re.findall(r"-?\d+", body.replace("\\", " "))]


ZIGZAG_88 = _table("MMR_ZIGZAG_INIT")
ZIGZAG_248 = _table("MMR_DV_ZIGZAG_248_INIT")
QUANT_SHIFTS = [_table("MMR_DV_QUANT_SHIFTS_INIT")[4 * i:4 * i + 4] for i in range(22)]
QUANT_OFFSET = _table("MMR_DV_QUANT_OFFSET_INIT")
IWEIGHT_88 = _table("MMR_DV_IWEIGHT_88_INIT")
IWEIGHT_248 = _table("MMR_DV_IWEIGHT_248_INIT")
BLOCK_BITS = (112, 112, 112, 112, 80, 80)  # decoder.rs:15


class DvError(Exception):
    pass


class _Block:
    __slots__ = ("c", "pos", "mode", "cls", "q", "partial", "complete")

    def __init__(self, q, cls, mode):
        self.c = [0] * 64
        self.pos, self.mode, self.cls, self.q = 0, mode, cls, q
        self.partial, self.complete = "", False


class DvVideo:
    """decode_video_with_options (decoder.rs:87-150) for frames whose DIF structure is
    intact. vlc: the code list of vlc_entries (decoder.rs:319-354) as (code, length, run,
    level). Bits are strings of '0'/'1' (bytes_to_bits, :603-611)."""

    def __init__(self, vlc):
        self.codes = {(length, code): (run, level) for code, length, run, level in vlc}
        self.lengths = sorted({length for _, length, _, _ in vlc})  # first match by length (:312-317)

    def decode_vlc(self, bits, pos):
        n = len(bits) - pos
        for length in self.lengths:
            if length > n:
                return None
            hit = self.codes.get((length, int(bits[pos:pos + length], 2)))
            if hit is not None:
                return length, hit[0], hit[1]
        return None

    @staticmethod
    def inverse_factor(block, position):  # inverse_factor_for_encoding (:290-310)
        q = block.q + QUANT_OFFSET[block.cls]
        area = 0 if position <= 5 else 1 if position <= 20 else 2 if position <= 42 else 3
        weight = IWEIGHT_248[position] if block.mode else IWEIGHT_88[position]
        return weight << (QUANT_SHIFTS[q][area] + 1 + (1 if block.cls == 3 else 0))

    def consume_ac(self, block, bits_in):  # :245-284
        if block.complete:
            return bits_in
        bits = block.partial + bits_in
        block.partial = ""
        cursor = 0
        while True:
            hit = self.decode_vlc(bits, cursor)
            if hit is not None:
                length, run, level = hit
                cursor += length
                block.pos += run + 1
                if block.pos >= 64:
                    block.complete = True
                    return bits[cursor:]
                if level != 0:
                    scan = ZIGZAG_248 if block.mode else ZIGZAG_88
                    block.c[scan[block.pos]] = (level * self.inverse_factor(block, block.pos) + 8192) >> 14
            elif len(bits) - cursor < 16:
                block.partial += bits[cursor:]
                return ""
            else:
                raise DvError("invalid DV variable-length coefficient code")

    def consume_pool(self, blocks, pool):  # :225-243
        for block in blocks:
            if not block.complete and pool:
                pool = self.consume_ac(block, pool)
        return pool

    def decode_macroblock(self, data):  # :193-223
        q = data[3] & 0x0F
        payload = "".join(format(b, "08b") for b in data[4:80])
        cursor, blocks, mb_pool = 0, [], ""
        for count in BLOCK_BITS:
            region = payload[cursor:cursor + count]
            cursor += count
            dc = int(region[:9], 2)
            if region[0] == "1":
                dc -= 1 << 9  # signed_bits (:618-625)
            block = _Block(q, int(region[10:12], 2), region[9] != "0")
            block.c[0] = dc * 4 + 1024
            left = self.consume_ac(block, region[12:])
            if block.complete:
                mb_pool += left
            blocks.append(block)
        return blocks, self.consume_pool(blocks, mb_pool)

    @staticmethod
    def coordinates(pal, sequences, sequence, slot):  # macroblock_coordinates (:395-422)
        off, shuf3, lstart = (2, 6, 8, 0, 4), (18, 9, 27, 0, 36), (9, 4, 13, 0, 18)
        serpent1 = [0, 1, 2, 2, 1, 0] * 4 + [0, 1, 2]
        serpent2 = [0, 1, 2, 3, 4, 5, 5, 4, 3, 2, 1, 0] * 2 + [0, 1, 2, 3, 4, 5]
        out = []
        for mb in range(5):
            if pal:
                x = shuf3[mb] + slot // 3
                y = serpent1[slot] + ((sequence + off[mb]) % sequences) * 3
                out.append((x * 2, y * 2))
            else:
                row = (sequence + off[mb]) % sequences
                k = slot + (3 if mb in (1, 2) else 0)
                x = lstart[mb] + k // 6
                y = serpent2[k] + row * 6
                if x > 21:
                    y = y * 2 - row * 6
                out.append((x * 4, y))
        return out

    def decode(self, data, conceal=False):
        """(planes [(w, h, bytes)], concealed [(sequence, slot)]) or DvError."""
        pal = len(data) == 144000
        sequences, width, height = (12, 720, 576) if pal else (10, 720, 480)
        cw, ch = (360, 288) if pal else (180, 480)
        planes = [np.full((height, width), 16, np.uint8), np.full((ch, cw), 128, np.uint8),
                  np.full((ch, cw), 128, np.uint8)]
        concealed, segments = [], []
        for sequence in range(sequences):
            for slot in range(27):
                try:
                    segments.append((sequence, slot, self.decode_segment(data, sequence, slot)))
                except DvError:
                    if not conceal:
                        raise
                    concealed.append((sequence, slot))
        # the transforms of every placed block in one batch, then placement (:425-505)
        blocks = [b for _, _, mbs in segments for mb in mbs for b in mb]
        coeffs = np.array([b.c for b in blocks], np.int64).reshape(-1, 64)
        modes = np.array([b.mode for b in blocks], bool)
        pixels = np.zeros((len(blocks), 64), np.uint8)
        if modes.any():
            pixels[modes] = dv_idct248(coeffs[modes])
        if (~modes).any():
            pixels[~modes] = dv_idct88(coeffs[~modes])
        k = 0
        for sequence, slot, mbs in segments:
            for (mb_x, mb_y), mb in zip(self.coordinates(pal, sequences, sequence, slot), mbs):
                px = [pixels[k + i].reshape(8, 8) for i in range(6)]
                k += 6
                x, y = mb_x * 8, mb_y * 8
                if pal:
                    for i, (dx, dy) in enumerate(((0, 0), (8, 0), (0, 8), (8, 8))):
                        planes[0][y + dy:y + dy + 8, x + dx:x + dx + 8] = px[i]
                    planes[2][y // 2:y // 2 + 8, x // 2:x // 2 + 8] = px[4]
                    planes[1][y // 2:y // 2 + 8, x // 2:x // 2 + 8] = px[5]
                elif mb_x < 88:
                    for i in range(4):
                        planes[0][y:y + 8, x + 8 * i:x + 8 * i + 8] = px[i]
                    planes[2][y:y + 8, x // 4:x // 4 + 8] = px[4]
                    planes[1][y:y + 8, x // 4:x // 4 + 8] = px[5]
                else:
                    for i, (dx, dy) in enumerate(((0, 0), (8, 0), (0, 8), (8, 8))):
                        planes[0][y + dy:y + dy + 8, x + dx:x + dx + 8] = px[i]
                    for p, b in ((2, px[4]), (1, px[5])):  # put_split_chroma (:488-503)
                        planes[p][y:y + 8, x // 4:x // 4 + 4] = b[:, :4]
                        planes[p][y + 8:y + 16, x // 4:x // 4 + 4] = b[:, 4:]
        return [(p.shape[1], p.shape[0], p.tobytes()) for p in planes], concealed

    def decode_segment(self, data, sequence, slot):  # :152-191
        mbs, pool = [], ""
        for mb in range(5):
            vn = slot * 5 + mb
            index = sequence * 150 + 7 + (vn // 15) * 16 + vn % 15
            blocks, overflow = self.decode_macroblock(data[index * 80:index * 80 + 80])
            pool += overflow
            mbs.append(blocks)
        for block in (b for blocks in mbs for b in blocks):  # consume_pool_for_macroblocks (:215-223)
            if not block.complete and pool:
                pool = self.consume_ac(block, pool)
        if any(not b.complete for blocks in mbs for b in blocks):
            raise DvError(f"DV video segment {slot} in sequence {sequence} has incomplete coefficients")
        return mbs


# ------------------------------------------------------------------ baseline JPEG decode

class JpegError(Exception):
    def __init__(self, status, message):
        super().__init__(message)
        self.status, self.message = status, message


INVALID_DATA, UNSUPPORTED, INTERNAL = 2, 3, 100
_NAMES = {0x01: "TEM", 0xC0: "SOF0", 0xC4: "DHT", 0xD8: "SOI", 0xD9: "EOI", 0xDA: "SOS", 0xDB: "DQT",
          0xDC: "DNL", 0xDD: "DRI", 0xFE: "COM"}


def _marker_name(code):  # syntax.rs:73-99
    if 0xD0 <= code <= 0xD7:
        return f"RST{code - 0xD0}"
    if 0xE0 <= code <= 0xEF:
        return "APP"
    return _NAMES.get(code, "UNKNOWN")


def _bad(offset, message):  # parser.rs jpeg_error / invalid
    return JpegError(INVALID_DATA, f"JPEG at byte 0x{offset:08x}: {message}")


def _read_marker(data, pos):  # parser.rs:93-110
    if pos >= len(data) or data[pos] != 0xFF:
        raise _bad(pos, "expected JPEG marker prefix 0xff")
    code_at = pos + 1
    while code_at < len(data) and data[code_at] == 0xFF:
        code_at += 1
    if code_at >= len(data):
        raise _bad(code_at, "truncated marker")
    if data[code_at] == 0x00:
        raise _bad(code_at, "stuffed 0xff byte outside entropy-coded data")
    return pos, data[code_at], code_at + 1


def _scan_entropy(data, start):  # parser.rs:373-414
    pos = start
    while pos < len(data):
        if data[pos] != 0xFF:
            pos += 1
            continue
        marker_at = pos
        pos += 1
        while pos < len(data) and data[pos] == 0xFF:
            pos += 1
        if pos >= len(data):
            raise _bad(pos, "truncated marker in entropy-coded data")
        code = data[pos]
        pos += 1
        if code == 0x00 or 0xD0 <= code <= 0xD7:
            continue
        return (start, marker_at - start), (marker_at, code, pos)
    raise _bad(len(data), "entropy-coded scan has no terminating marker")


def _segment(code, p, base, seg):  # parse_segment_data and the segment parsers (parser.rs:112-371)
    if code == 0xC0:
        if len(p) < 6:
            raise _bad(base, "SOF0 payload is too short")
        n = p[5]
        if n == 0:
            raise _bad(base + 5, "SOF0 must declare at least one component")
        if len(p) != 6 + 3 * n:
            raise _bad(base + 5, f"SOF0 declares {n} components but has {len(p)} bytes")
        if p[0] != 8:
            raise _bad(base, "baseline SOF0 sample precision must be 8 bits")
        height, width = (p[1] << 8) | p[2], (p[3] << 8) | p[4]
        if width == 0:
            raise _bad(base + 3, "SOF0 width must be non-zero")
        comps = []
        for i in range(n):
            o = 6 + 3 * i
            hs, vs = p[o + 1] >> 4, p[o + 1] & 15
            if not (1 <= hs <= 4 and 1 <= vs <= 4):
                raise _bad(base + o + 1, "sampling factors must be between 1 and 4")
            if p[o + 2] > 3:
                raise _bad(base + o + 2, "quantization table selector must be 0 through 3")
            comps.append((p[o], hs, vs, p[o + 2]))
        seg["frame"] = (width, height, comps)
    elif code == 0xDB:
        tables, pos = [], 0
        while pos < len(p):
            spec = p[pos]
            pos += 1
            if spec >> 4 > 1:
                raise _bad(base + pos - 1, "DQT precision must be 0 or 1")
            if spec & 15 > 3:
                raise _bad(base + pos - 1, "DQT table identifier must be 0 through 3")
            size = 1 + (spec >> 4)
            if len(p) - pos < 64 * size:
                raise _bad(base + pos, "truncated DQT values")
            vals = [p[pos + i] if size == 1 else (p[pos + 2 * i] << 8) | p[pos + 2 * i + 1] for i in range(64)]
            pos += 64 * size
            tables.append((spec & 15, spec >> 4, vals))
        if not tables:
            raise _bad(base, "DQT must contain at least one table")
        seg["dqt"] = tables
    elif code == 0xC4:
        tables, pos = [], 0
        while pos < len(p):
            spec = p[pos]
            pos += 1
            if spec >> 4 > 1:
                raise _bad(base + pos - 1, "DHT class must be 0 or 1")
            if spec & 15 > 3:
                raise _bad(base + pos - 1, "DHT table identifier must be 0 through 3")
            if pos + 16 > len(p):
                raise _bad(base + pos, "truncated DHT code counts")
            counts = list(p[pos:pos + 16])
            pos += 16
            if pos + sum(counts) > len(p):
                raise _bad(base + pos, "truncated DHT symbols")
            symbols = list(p[pos:pos + sum(counts)])
            pos += sum(counts)
            tables.append((spec >> 4, spec & 15, counts, symbols))
        if not tables:
            raise _bad(base, "DHT must contain at least one table")
        seg["dht"] = tables
    elif code == 0xDD:
        if len(p) != 2:
            raise _bad(base, "DRI payload must contain exactly two bytes")
        seg["dri"] = (p[0] << 8) | p[1]
    elif code == 0xDA:
        if not p:
            raise _bad(base, "SOS payload is empty")
        n = p[0]
        if n == 0:
            raise _bad(base, "SOS must select at least one component")
        if len(p) != 1 + 2 * n + 3:
            raise _bad(base, f"SOS declares {n} components but has {len(p)} bytes")
        comps = []
        for i in range(n):
            o = 1 + 2 * i
            if p[o + 1] >> 4 > 3 or p[o + 1] & 15 > 3:
                raise _bad(base + o + 1, "Huffman table selectors must be 0 through 3")
            comps.append((p[o], p[o + 1] >> 4, p[o + 1] & 15))
        t = 1 + 2 * n
        seg["sos"] = (comps, p[t], p[t + 1], p[t + 2] >> 4, p[t + 2] & 15)
    elif code == 0xE0 and p[:5] == b"JFIF\0":
        if len(p) < 14:
            raise _bad(base, "JFIF APP0 payload is too short")
        if len(p) != 14 + 3 * p[12] * p[13]:
            raise _bad(base + 12, "JFIF thumbnail dimensions do not match payload size")
        seg["jfif"] = True
    elif 0xE0 <= code <= 0xEF:
        seg["app"] = (code - 0xE0, bytes(p))


def parse_jpeg(data):
    """parse_jpeg (parser.rs:18-81): the segment list and the entropy scans."""
    soi_at, code, pos = _read_marker(data, 0)
    if code != 0xD8 or soi_at != 0:
        raise _bad(soi_at, "expected SOI as the first marker")
    segments, scans, pending = [], [], None
    while True:
        at, code, after = pending if pending else _read_marker(data, pos)
        pending = None
        pos = after
        if code == 0xD9:
            return segments, scans
        if code in (0x01, 0xD8) or 0xD0 <= code <= 0xD7:
            continue
        if pos + 2 > len(data):
            raise _bad(pos, "truncated segment length")
        length = (data[pos] << 8) | data[pos + 1]
        if length < 2:
            raise _bad(pos, "segment length must include its two length bytes")
        start, end = pos + 2, pos + length
        if end > len(data):
            raise _bad(start, f"truncated {_marker_name(code)} payload")
        seg = {"offset": at}
        _segment(code, data[start:end], start, seg)
        segments.append(seg)
        pos = end
        if code == 0xDA:
            scan, pending = _scan_entropy(data, pos)
            pos = pending[2]
            scans.append(scan)


def _huffman(cls_id, counts, symbols):  # HuffmanDecoder::new (entropy.rs:18-55)
    total = sum(counts)
    if total == 0 or total != len(symbols):
        raise JpegError(INVALID_DATA, f"JPEG Huffman table {cls_id} has inconsistent symbol counts")
    codes, code, k = {}, 0, 0
    for length in range(1, 17):
        if code + counts[length - 1] > 1 << length:
            raise JpegError(INVALID_DATA, f"JPEG Huffman table {cls_id} is oversubscribed at length {length}")
        for _ in range(counts[length - 1]):
            codes[(length, code)] = symbols[k]
            k += 1
            code += 1
        code <<= 1
    return codes


class _Reader:  # EntropyReader (entropy.rs:72-166)
    def __init__(self, data, base):
        self.data, self.base, self.pos, self.byte, self.left = data, base, 0, 0, 0

    def error(self, message):
        return JpegError(INVALID_DATA, f"JPEG entropy at byte 0x{self.base + self.pos:08x}: {message}")

    def data_byte(self):
        if self.pos >= len(self.data):
            raise self.error("unexpected end of entropy-coded data")
        b = self.data[self.pos]
        self.pos += 1
        if b != 0xFF:
            return b
        while self.pos < len(self.data) and self.data[self.pos] == 0xFF:
            self.pos += 1
        if self.pos >= len(self.data):
            raise self.error("truncated entropy marker")
        code = self.data[self.pos]
        self.pos += 1
        if code == 0x00:
            return 0xFF
        raise self.error(f"unexpected marker 0xff{code:02x} inside coded block")

    def bit(self):
        if self.left == 0:
            self.byte, self.left = self.data_byte(), 8
        self.left -= 1
        return (self.byte >> self.left) & 1

    def bits(self, n):
        v = 0
        for _ in range(n):
            v = (v << 1) | self.bit()
        return v

    def restart(self, expected):
        self.left = 0
        marker_at = self.base + self.pos
        if self.pos >= len(self.data) or self.data[self.pos] != 0xFF:
            raise self.error("expected restart marker at MCU boundary")
        self.pos += 1
        while self.pos < len(self.data) and self.data[self.pos] == 0xFF:
            self.pos += 1
        if self.pos >= len(self.data):
            raise self.error("truncated restart marker")
        code = self.data[self.pos]
        self.pos += 1
        if code != 0xD0 + expected:
            raise JpegError(INVALID_DATA, f"JPEG at byte 0x{marker_at:08x}: expected RST{expected}, found marker 0x{code:02x}")

    def decode(self, codes):  # HuffmanDecoder::decode (entropy.rs:57-70)
        v = 0
        for length in range(1, 17):
            v = (v << 1) | self.bit()
            sym = codes.get((length, v))
            if sym is not None:
                return sym
        raise self.error("no Huffman code matches the next 16 bits")

    def extend(self, size):  # receive_extend (entropy.rs:168-182)
        if size == 0:
            return 0
        if size > 15:
            raise self.error("coefficient magnitude contains more than 15 bits")
        v = self.bits(size)
        return v + 1 - (1 << size) if v < 1 << (size - 1) else v


def _i32(v, reader, message):
    if not -(1 << 31) <= v < 1 << 31:
        raise reader.error(message)
    return v


def _block(reader, dc, ac, q, pred):  # decode_block (decoder.rs:495-548); returns (coefficients, prediction)
    c = [0] * 64
    size = reader.decode(dc)
    if size > 11:
        raise reader.error("baseline DC coefficient category exceeds 11")
    pred = _i32(pred + reader.extend(size), reader, "DC prediction overflow")
    c[0] = _i32(pred * q[0], reader, "dequantized DC coefficient overflow")
    k = 1
    while k < 64:
        sym = reader.decode(ac)
        run, size = sym >> 4, sym & 15
        if size == 0:
            if run == 0:
                break
            if run != 15:
                raise reader.error("invalid zero-size AC Huffman symbol")
            k += 16
            if k > 64:
                raise reader.error("AC zero run exceeds the end of the block")
            continue
        if size > 10:
            raise reader.error("baseline AC coefficient category exceeds 10")
        k += run
        if k >= 64:
            raise reader.error("AC coefficient run exceeds the end of the block")
        v = reader.extend(size)
        c[ZIGZAG_88[k]] = _i32(v * q[k], reader, "dequantized AC coefficient overflow")
        k += 1
    return c, pred


def decode_jpeg(data):
    """decode_jpeg + into_video_frame (decoder.rs:69-167, 169-493): (format, width,
    height, [(w, h, bytes)]) or JpegError with the reference's status and message."""
    segments, scans = parse_jpeg(data)
    frame = next((s["frame"] for s in segments if "frame" in s), None)
    if frame is None:
        raise JpegError(INVALID_DATA, "JPEG has no baseline SOF0 frame header")
    if len(scans) != 1:
        raise JpegError(UNSUPPORTED, f"baseline decoder currently requires exactly one scan, found {len(scans)}")
    sos = [s for s in segments if "sos" in s]
    if not sos:
        raise JpegError(INVALID_DATA, "JPEG has entropy data without an SOS header")
    if len(sos) > 1:
        raise JpegError(UNSUPPORTED, "baseline decoder currently supports only one SOS header")
    scan_at, (scomps, ss, se, ah, al) = sos[0]["offset"], sos[0]["sos"]
    width, height, comps = frame
    if height == 0:
        raise JpegError(UNSUPPORTED, "JPEG height supplied by a DNL marker is not supported yet")
    if len(scomps) != len(comps):
        raise JpegError(UNSUPPORTED, "non-interleaved or partial-component JPEG scans are not supported yet")
    if ss != 0 or se != 63 or ah != 0 or al != 0:
        raise JpegError(UNSUPPORTED, "scan parameters are not baseline sequential")
    for cid, _, _, _ in comps:
        if sum(1 for sel, _, _ in scomps if sel == cid) != 1:
            raise JpegError(INVALID_DATA, f"JPEG scan must select frame component {cid} exactly once")
    if len(comps) == 1:  # infer_color_model (decoder.rs:169-194)
        model = "gray"
    else:
        adobe = next((a[1][11] for s in segments if "app" in s for a in [s["app"]]
                      if a[0] == 14 and len(a[1]) >= 12 and a[1][:5] == b"Adobe"), None)
        jfif = any("jfif" in s for s in segments)
        model = {(3, 0): "rgb", (3, 1): "ycbcr", (4, 0): "cmyk", (4, 2): "ycck"}.get((len(comps), adobe))
        if model is None:
            model = "ycbcr" if len(comps) == 3 and adobe is None and jfif else "unknown"
    quant, dcs, acs, ri = [None] * 4, [None] * 4, [None] * 4, 0  # DecodeTables::collect (:263-299)
    for s in segments:
        if s["offset"] >= scan_at:
            break
        for tid, precision, vals in s.get("dqt", []):
            quant[tid] = (precision, vals)
        for cls, tid, counts, symbols in s.get("dht", []):
            (acs if cls else dcs)[tid] = _huffman(tid, counts, symbols)
        ri = s.get("dri", ri)
    hmax, vmax = max(c[1] for c in comps), max(c[2] for c in comps)
    states = []
    for cid, hs, vs, tq in comps:  # make_component_states (:421-461)
        if quant[tq] is None:
            raise JpegError(INVALID_DATA, f"JPEG component {cid} references missing quantization table {tq}")
        if quant[tq][0] != 0:
            raise JpegError(UNSUPPORTED, "16-bit quantization tables are not allowed in baseline JPEG")
        states.append({"hs": hs, "vs": vs, "q": quant[tq][1], "w": -(-width * hs // hmax),
                       "h": -(-height * vs // vmax), "pred": 0})
    decoders = []
    for sel, td, ta in scomps:  # make_scan_decoders (:463-493)
        index = next((i for i, c in enumerate(comps) if c[0] == sel), None)
        if index is None:  # `.expect` panics (:470-474); the C ABI contains it (capi/src/lib.rs:572-588)
            raise JpegError(INTERNAL, "panic contained at MMRecode C API boundary")
        if dcs[td] is None:
            raise JpegError(INVALID_DATA, f"JPEG scan references missing DC Huffman table {td}")
        if acs[ta] is None:
            raise JpegError(INVALID_DATA, f"JPEG scan references missing AC Huffman table {ta}")
        decoders.append((index, dcs[td], acs[ta]))
    inter = len(comps) > 1
    mcu_w, mcu_h = (hmax * 8, vmax * 8) if inter else (8, 8)
    cols, rows = -(-width // mcu_w), -(-height // mcu_h)
    (start, length) = scans[0]
    reader = _Reader(data[start:start + length], start)
    number, blocks = 0, []
    for mcu in range(cols * rows):  # reconstruct (:318-402)
        if mcu > 0 and ri and mcu % ri == 0:
            reader.restart(number)
            number = (number + 1) & 7
            for st in states:
                st["pred"] = 0
        mx, my = mcu % cols, mcu // cols
        for index, dc, ac in decoders:
            st = states[index]
            br, bc = (st["vs"], st["hs"]) if inter else (1, 1)
            for by in range(br):
                for bx in range(bc):
                    c, st["pred"] = _block(reader, dc, ac, st["q"], st["pred"])
                    blocks.append((index, (mx * bc + bx) * 8, (my * br + by) * 8, c))
    planes = [np.zeros((st["h"], st["w"]), np.uint8) for st in states]
    if blocks:
        pixels = jpeg_idct(np.array([b[3] for b in blocks], np.int64))
        for (index, x, y, _), px in zip(blocks, pixels):  # write_block (:550-565)
            p = planes[index]
            h, w = min(8, p.shape[0] - y), min(8, p.shape[1] - x)
            if h > 0 and w > 0:
                p[y:y + h, x:x + w] = px.reshape(8, 8)[:h, :w]
    dims = [(p.shape[1], p.shape[0]) for p in planes]  # standard_pixel_format (:100-126)
    if model == "gray" and len(planes) == 1 and dims[0] == (width, height):
        fmt = 1
    else:
        if model != "ycbcr" or len(planes) != 3 or dims[0] != (width, height) or dims[1] != dims[2]:
            raise JpegError(UNSUPPORTED, "JPEG components do not map directly to a shared planar pixel format")
        half_w, half_h = -(-width // 2), -(-height // 2)
        fmt = {(width, height): 4, (half_w, height): 3, (half_w, half_h): 2}.get(dims[1])
        if fmt is None:
            raise JpegError(UNSUPPORTED, "JPEG chroma sampling is not 4:2:0, 4:2:2, or 4:4:4")
    return fmt, width, height, [(p.shape[1], p.shape[0], p.tobytes()) for p in planes]
