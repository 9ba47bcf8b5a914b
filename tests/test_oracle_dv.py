"""The oracle's DV25 video decode (oracle/dv.c) against the second restatement in
tests/restatements.py, written in Python from crates/codecs/dv/src/decoder.rs:87-611:
segment and macroblock decode with the three spill levels, dequantisation, the 8-8 and
2-4-8 transforms, macroblock coordinates and placement. Frames from the encoder (NTSC
and PAL, both mode policies) and copies with damaged payload bytes, decoded with and
without concealment: the same status and message, the same concealed segments and
every sample. The reference's own tests pin only frame sizes and one damaged vector."""
import numpy as np
import pytest

import mmrecode_gb300 as m
import oracle
from mmrecode_gb300 import synth
from helpers import dv_restamped
from restatements import DvError, DvVideo


@pytest.fixture(scope="module")
def dv():
    return DvVideo(oracle.dv_vlc_entries())


def compare(dv, data, conceal, label):
    ref = oracle.dv_decode(data, conceal)
    try:
        planes, concealed = dv.decode(data, conceal)
    except DvError as e:
        assert ref.status == m.INVALID_DATA and ref.message == str(e), f"{label}: {ref.status} {ref.message} / {e}"
        return "error"
    assert ref.status == 0, f"{label}: oracle {ref.status} {ref.message}"
    assert ref.concealed == concealed, label
    for i, ((w, h, got), (rw, rh, want)) in enumerate(zip(planes, ref.frame.planes)):
        assert (w, h) == (rw, rh), f"{label}: plane {i}"
        if got != want:
            a, b = np.frombuffer(got, np.uint8), np.frombuffer(want, np.uint8)
            bad = np.nonzero(a != b)[0]
            raise AssertionError(f"{label}: plane {i}: {bad.size} samples differ, first at {bad[0]}")
    return "concealed" if concealed else "ok"


def damaged(frame, rng, count):
    """Payload bytes (4..79 of video DIF blocks) changed; identifiers stay intact."""
    b = bytearray(frame)
    sequences = len(frame) // 12000
    for _ in range(count):
        seq, vn = int(rng.integers(0, sequences)), int(rng.integers(0, 135))
        index = seq * 150 + 7 + (vn // 15) * 16 + vn % 15
        b[index * 80 + int(rng.integers(4, 80))] ^= int(rng.integers(1, 256))
    return bytes(b)


@pytest.mark.parametrize("pal", [False, True], ids=["ntsc", "pal"])
def test_dv_decode_two_restatements_agree(dv, pal):
    rng = np.random.default_rng(51 + pal)
    frames = synth.dv_stream(520 + pal, 1, pal=pal) + synth.dv_stream(530 + pal, 1, pal=pal, mode=m.DV_MODE_88)
    outcomes = []
    for i, f in enumerate(frames):
        outcomes.append(compare(dv, f, False, f"frame {i}"))
        outcomes.append(compare(dv, dv_restamped(f, rng), False, f"frame {i} restamped"))
        for j, count in enumerate((1, 4, 40)):
            d = damaged(f, rng, count)
            for conceal in (False, True):
                outcomes.append(compare(dv, d, conceal, f"frame {i} damage {j} conceal {conceal}"))
    assert "ok" in outcomes and "error" in outcomes and "concealed" in outcomes, outcomes
