"""The C-ABI library without a GPU: symbols, versions, argument checks, probe.

Mirrors crates/capi/src/lib.rs:1210-1441 (C boundary tests) and
crates/capi/tests/header.rs (the C header compiles under C11 -Werror)."""

import ctypes
import glob
import os
import re
import shutil
import subprocess
import threading

import pytest

import mmrecode_gb300 as m
from mmrecode_gb300 import _lib, synth
from helpers import fixture

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        names += re.findall(r"MMR_API\s+[\w\s\*]+?\b(mmr_\w+)\s*\(", open(h).read())
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_functions()
    assert len(names) >= 24
    for name in names:
        assert hasattr(lib, name), name
    assert set(names) == set(_lib.SIGNATURES), "bindings and headers disagree"
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = {l.split()[-1] for l in out.splitlines() if " T " in l}
    assert set(names) <= exported


def test_versions():
    assert m.abi_version() == 1
    assert len(m.version()) > 0


def _frame():
    f = _lib.VideoFrameC()
    f.struct_size = ctypes.sizeof(_lib.VideoFrameC)
    return f


# lib.rs:1353-1370 invalid_argument_sets_thread_local_diagnostic
def test_null_data_with_length_is_invalid_argument():
    lib = _lib.load()
    f = _frame()
    assert lib.mmr_mjpeg_decode(None, 4, ctypes.byref(f)) == m.INVALID_ARGUMENT
    required = lib.mmr_last_error_message(None, 0)
    buf = ctypes.create_string_buffer(required)
    assert lib.mmr_last_error_message(buf, required) == required
    assert "data is null" in buf.value.decode()
    small = ctypes.create_string_buffer(4)
    lib.mmr_last_error_message(small, 4)
    assert small.value == buf.value[:3]
    assert lib.mmr_dv_decode(None, 4, ctypes.byref(f)) == m.INVALID_ARGUMENT
    assert lib.mmr_mjpeg_decode(None, 0, None) == m.INVALID_ARGUMENT
    assert "out_frame is null" in _lib.last_error()


# lib.rs:1426-1435 rejects_an_incompatible_output_structure
def test_struct_size_mismatch_leaves_frame_untouched():
    lib = _lib.load()
    f = _lib.VideoFrameC()
    f.struct_size = 0
    f.width = 1234
    data = fixture("jpeg/valid/baseline-420.jpg")
    assert lib.mmr_mjpeg_decode(data, len(data), ctypes.byref(f)) == m.INVALID_ARGUMENT
    assert f.struct_size == 0 and f.width == 1234


def test_last_error_is_thread_local():
    lib = _lib.load()
    lib.mmr_mjpeg_decode(None, 4, ctypes.byref(_frame()))
    seen = []
    t = threading.Thread(target=lambda: seen.append(_lib.last_error()))
    t.start()
    t.join()
    assert seen == [""] and "data is null" in _lib.last_error()


def test_frame_and_buffer_free_are_null_safe_and_idempotent():
    lib = _lib.load()
    lib.mmr_video_frame_free(None)
    f = _frame()
    lib.mmr_video_frame_free(ctypes.byref(f))
    lib.mmr_video_frame_free(ctypes.byref(f))
    assert f.struct_size == ctypes.sizeof(_lib.VideoFrameC) and f.plane_count == 0
    lib.mmr_buffer_free(None)
    b = _lib.Buffer()
    lib.mmr_buffer_free(ctypes.byref(b))
    assert b.struct_size == ctypes.sizeof(_lib.Buffer)


def test_entries_outside_this_library_report_unsupported():
    lib = _lib.load()
    b = _lib.Buffer()
    b.struct_size = ctypes.sizeof(_lib.Buffer)
    n = ctypes.c_size_t(7)
    assert lib.mmr_mpeg2_picture_count(b"x", 1, ctypes.byref(n)) == m.UNSUPPORTED and n.value == 0
    assert lib.mmr_mpegts_mux_mpeg2(b"x", 1, ctypes.byref(b)) == m.UNSUPPORTED
    assert "outside this library" in _lib.last_error()


def test_encode_argument_checks():
    lib = _lib.load()
    b = _lib.Buffer()
    b.struct_size = ctypes.sizeof(_lib.Buffer)
    assert lib.mmr_mjpeg_encode(None, 75, ctypes.byref(b)) == m.INVALID_ARGUMENT
    v = _lib.VideoFrameView()
    v.struct_size = ctypes.sizeof(_lib.VideoFrameView)
    v.format, v.range, v.width, v.height, v.plane_count = 1, 1, 8, 8, 1
    v.planes[0].data_len, v.planes[0].stride, v.planes[0].width, v.planes[0].height = 10, 8, 8, 8
    buf = (ctypes.c_uint8 * 10)()
    v.planes[0].data = ctypes.cast(buf, _lib.u8p)
    assert lib.mmr_mjpeg_encode(ctypes.byref(v), 75, ctypes.byref(b)) == m.INVALID_ARGUMENT
    assert "plane 0 needs 64 bytes but data_len is 10" in _lib.last_error()
    v.format = 9
    assert lib.mmr_mjpeg_encode(ctypes.byref(v), 75, ctypes.byref(b)) == m.INVALID_ARGUMENT
    assert "unknown pixel format 9" in _lib.last_error()


def test_probe_reports_geometry_from_headers():
    info = m.probe(m.CODEC_MJPEG, fixture("jpeg/valid/baseline-420.jpg"))
    assert (info.status, info.format, info.width, info.height, info.plane_count) == (0, m.YUV420P8, 16, 16, 3)
    assert info.planar_bytes == 16 * 16 + 2 * 8 * 8 and info.rgb_bytes == 16 * 16 * 3
    info = m.probe(m.CODEC_DV, fixture("dv/valid/dv25-625-50-one-frame.dv"))
    assert (info.format, info.width, info.height, info.plane_width[1], info.plane_height[1]) == (m.YUV420P8, 720, 576, 360, 288)
    info = m.probe(m.CODEC_MJPEG, fixture("jpeg/invalid/invalid-length.jpg"))
    assert info.status == m.INVALID_DATA
    p = synth.mjpeg_stream(5, 1, 1920, 1080, "422", 90, 120)[0]
    info = m.probe(m.CODEC_MJPEG, p)
    assert (info.format, info.plane_width[1], info.plane_height[1]) == (m.YUV422P8, 960, 1080)


def _reference_smoke() -> str:
    """The reference's own C smoke program, where the reference checkout is present
    (its location is the fixture script's, tests/golden/make_fixtures.py)."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_fixtures", os.path.join(ROOT, "tests", "golden",
                                                                                "make_fixtures.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return os.path.join(mod.REFERENCE, "crates", "capi", "tests", "smoke.c")


REFERENCE_SMOKE = _reference_smoke()
REFERENCE_HEADER = os.path.join(os.path.dirname(os.path.dirname(REFERENCE_SMOKE)), "include", "mmrecode.h")


def _declarations(path):
    """#define lines and C statements (typedefs, prototypes) of a header, with
    comments dropped and whitespace normalised."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    defines = sorted(re.sub(r"\s+", " ", l.strip()) for l in text.splitlines() if l.strip().startswith("#define"))
    body = re.sub(r"\s+", " ", "\n".join(l for l in text.splitlines() if not l.strip().startswith("#")))
    body = re.sub(r"\s*([(),;{}*\[\]])\s*", r"\1", body)
    return defines, sorted(x.strip() for x in body.split(";") if x.strip())


@pytest.mark.skipif(not os.path.exists(REFERENCE_HEADER), reason="reference checkout absent")
def test_v1_header_declares_what_the_reference_header_declares():
    """include/mmrecode.h against crates/capi/include/mmrecode.h: the same macros, types
    and prototypes (only comments and line breaks differ), so callers compile unchanged."""
    assert _declarations(os.path.join(ROOT, "include", "mmrecode.h")) == _declarations(REFERENCE_HEADER)


@pytest.mark.skipif(not os.path.exists(REFERENCE_SMOKE) or not shutil.which("gcc"), reason="reference smoke.c absent")
def test_reference_smoke_c_compiles_and_links_unchanged(tmp_path):
    exe = tmp_path / "smoke"
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), REFERENCE_SMOKE,
           "-o", str(exe), _lib.LIB_PATH, f"-Wl,-rpath,{os.path.dirname(_lib.LIB_PATH)}"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr


def test_session_c_caller_compiles(tmp_path):
    """tests/c/session_decode.c, a C caller of the decoder session API, compiles with
    every warning as an error and links (it runs on a GPU)."""
    src = os.path.join(ROOT, "tests", "c", "session_decode.c")
    exe = tmp_path / "session_decode"
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), src, "-o", str(exe),
           _lib.LIB_PATH, f"-Wl,-rpath,{os.path.dirname(_lib.LIB_PATH)}"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    usage = subprocess.run([str(exe)], capture_output=True, text=True)  # no arguments: usage, exit 2
    assert usage.returncode == 2 and "usage" in usage.stderr


def test_own_c_smoke_compiles(tmp_path):
    src = os.path.join(ROOT, "tests", "c", "smoke_decode.c")
    exe = tmp_path / "smoke_decode"
    cmd = ["gcc", "-std=c11", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), src, "-o", str(exe),
           _lib.LIB_PATH, f"-Wl,-rpath,{os.path.dirname(_lib.LIB_PATH)}"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr


@pytest.mark.parametrize("compiler,std", [("gcc", "-std=c11"), ("g++", "-std=c++17")])
def test_gpu_header_is_clean_c_and_cpp(tmp_path, compiler, std):
    """include/mmrecode_gpu.h for C and C++ callers: it compiles with every warning as an
    error, and every function it declares links against the library."""
    names = declared_functions()
    src = tmp_path / ("use_gpu_header.c" if compiler == "gcc" else "use_gpu_header.cpp")
    body = ",\n    ".join(f"(void (*)(void))&{n}" for n in names)
    src.write_text('#include "mmrecode_gpu.h"\n#include <stdio.h>\n\n'
                   f"static void (*const entries[])(void) = {{\n    {body}\n}};\n\n"
                   "int main(void) {\n"
                   "    printf(\"%zu\\n\", sizeof entries / sizeof entries[0]);\n"
                   "    return 0;\n}\n")
    exe = tmp_path / "use_gpu_header"
    flags = ["-Wall", "-Wextra", "-Werror", "-pedantic"] + (["-Wno-cast-function-type"] if compiler == "g++" else [])
    cmd = [compiler, std, *flags, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe), _lib.LIB_PATH,
           f"-Wl,-rpath,{os.path.dirname(_lib.LIB_PATH)}"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and int(out.stdout) == len(names)
