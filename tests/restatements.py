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
