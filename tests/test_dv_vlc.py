"""The engine's two-level DV VLC lookup table (mmrecode_gb300/csrc/dv_vlc.h) checked for
every 16-bit window against the oracle's restatement of decoder.rs:319-354
vlc_entries (canonical codes from VLC_LEN, sign bits appended): code length, run and
level of the code at the top of the window."""
import ctypes
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle

ROOT = Path(__file__).resolve().parents[1]
L1 = 10  # level-1 bits (kDvVlcL1Bits)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    gxx = shutil.which("g++")
    cuda_inc = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda")) / "include"
    if not gxx or not (cuda_inc / "cuda_runtime.h").exists():
        pytest.skip("no g++ or CUDA headers")
    so = tmp_path_factory.mktemp("vlc") / "vlc_harness.so"
    subprocess.run([gxx, "-O1", "-shared", "-fPIC", "-std=c++17", f"-I{ROOT / 'mmrecode_gb300' / 'csrc'}",
                    f"-I{cuda_inc}", "-o", str(so), str(ROOT / "tests" / "cuda" / "vlc_harness.cpp")], check=True)
    lib = ctypes.CDLL(str(so))
    lib.mmr_test_dv_vlc_capacity.restype = ctypes.c_size_t
    lib.mmr_test_fill_dv_vlc.restype = ctypes.c_size_t
    lib.mmr_test_fill_dv_vlc.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
    return lib


def test_every_window_decodes_like_the_oracle(harness):
    cap = harness.mmr_test_dv_vlc_capacity()
    table = np.zeros(cap, np.uint32)
    used = harness.mmr_test_fill_dv_vlc(table.ctypes.data, cap)
    assert 1 << L1 <= used <= cap

    entries = oracle.dv_vlc_entries()
    assert len(entries) == 746
    by_len = {}
    for code, length, run, level in entries:
        by_len.setdefault(length, {})[code] = (run, level)

    w = np.arange(1 << 16, dtype=np.uint32)
    e = table[w >> (16 - L1)]
    second = (e & 0x80000000) != 0
    e = np.where(second, table[(e & 0xFFFF) + (w & ((1 << (16 - L1)) - 1))], e)
    got_len = e & 31
    got_run = (e >> 5) & 127
    got_level = ((e >> 12) & 511).astype(np.int32) - 256

    want_len = np.zeros(1 << 16, np.uint32)
    want_run = np.zeros(1 << 16, np.uint32)
    want_level = np.zeros(1 << 16, np.int32)
    for x in range(1 << 16):
        for length in sorted(by_len):
            hit = by_len[length].get(x >> (16 - length))
            if hit is not None:
                want_len[x], (want_run[x], want_level[x]) = length, hit
                break
    assert (want_len > 0).all()  # the code is complete: every window starts with a code
    bad = np.nonzero((got_len != want_len) | (got_run != want_run) | (got_level != want_level))[0]
    assert bad.size == 0, [(int(x), int(got_len[x]), int(want_len[x])) for x in bad[:5]]


def test_too_small_a_table_is_refused(harness):
    table = np.zeros(1 << L1, np.uint32)
    assert harness.mmr_test_fill_dv_vlc(table.ctypes.data, (1 << L1) - 1) == 0
    assert harness.mmr_test_fill_dv_vlc(table.ctypes.data, 1 << L1) == 0  # no room for a level-2 block
