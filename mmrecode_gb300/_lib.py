"""ctypes binding of libmmrecode_gpu.so (include/mmrecode.h, include/mmrecode_gpu.h).

The library is built in-tree by ``mmrecode_gb300.build.build()``. Loading never
falls back to anything else: a missing library raises.
"""

from __future__ import annotations

import ctypes
import os

from . import build as _build

LIB_PATH = _build.LIB

u8p = ctypes.POINTER(ctypes.c_uint8)


class PlaneView(ctypes.Structure):
    _fields_ = [("data", u8p), ("data_len", ctypes.c_size_t), ("stride", ctypes.c_size_t),
                ("width", ctypes.c_size_t), ("height", ctypes.c_size_t)]


class VideoFrameView(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("format", ctypes.c_uint32), ("range", ctypes.c_uint32),
                ("width", ctypes.c_size_t), ("height", ctypes.c_size_t), ("plane_count", ctypes.c_size_t),
                ("planes", PlaneView * 3)]


class OwnedPlane(ctypes.Structure):
    _fields_ = [("data", u8p), ("data_len", ctypes.c_size_t), ("stride", ctypes.c_size_t),
                ("width", ctypes.c_size_t), ("height", ctypes.c_size_t)]


class VideoFrameC(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("format", ctypes.c_uint32), ("range", ctypes.c_uint32),
                ("width", ctypes.c_size_t), ("height", ctypes.c_size_t), ("plane_count", ctypes.c_size_t),
                ("planes", OwnedPlane * 3)]


class DeviceFrame(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("format", ctypes.c_uint32), ("range", ctypes.c_uint32),
                ("width", ctypes.c_size_t), ("height", ctypes.c_size_t), ("plane_count", ctypes.c_size_t),
                ("planes", ctypes.c_void_p * 3), ("plane_width", ctypes.c_size_t * 3),
                ("plane_height", ctypes.c_size_t * 3), ("buffer", ctypes.c_void_p), ("buffer_bytes", ctypes.c_size_t)]


class Buffer(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("data", u8p), ("len", ctypes.c_size_t)]


class GpuConfig(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("device", ctypes.c_int32), ("flags", ctypes.c_uint32),
                ("engines", ctypes.c_uint32)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("device", ctypes.c_int32), ("engines", ctypes.c_uint32),
                ("max_batch", ctypes.c_uint32), ("pad", ctypes.c_uint32), ("memory_budget", ctypes.c_uint64)]


class ServerStats(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t)] + [(n, ctypes.c_uint64) for n in (
        "submitted", "completed", "failed", "rejected", "batches", "in_flight", "queued")] + [
        (n, ctypes.c_double) for n in ("p50_ms", "p99_ms", "max_ms", "mean_ms", "frames_per_s", "window_s")] + [
        ("peak_budget_bytes", ctypes.c_uint64)]


class FrameInfo(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("status", ctypes.c_int32), ("format", ctypes.c_uint32),
                ("range", ctypes.c_uint32), ("width", ctypes.c_size_t), ("height", ctypes.c_size_t),
                ("plane_count", ctypes.c_size_t), ("plane_width", ctypes.c_size_t * 3),
                ("plane_height", ctypes.c_size_t * 3), ("planar_bytes", ctypes.c_size_t),
                ("rgb_bytes", ctypes.c_size_t)]


class GpuItem(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("data", ctypes.c_void_p), ("device_data", ctypes.c_void_p),
                ("len", ctypes.c_size_t), ("codec", ctypes.c_uint32), ("output", ctypes.c_uint32),
                ("flags", ctypes.c_uint32), ("out", ctypes.c_void_p), ("out_capacity", ctypes.c_size_t),
                ("status", ctypes.c_int32), ("format", ctypes.c_uint32), ("range", ctypes.c_uint32),
                ("width", ctypes.c_size_t), ("height", ctypes.c_size_t), ("plane_count", ctypes.c_size_t),
                ("plane_offset", ctypes.c_size_t * 3), ("plane_width", ctypes.c_size_t * 3),
                ("plane_height", ctypes.c_size_t * 3), ("out_bytes", ctypes.c_size_t),
                ("concealed_segments", ctypes.c_uint32), ("message", ctypes.c_char * 200)]


class BatchStats(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t)] + [(n, ctypes.c_double) for n in (
        "total_ms", "upload_ms", "scan_ms", "entropy_ms", "idct_ms", "dv_ms", "rgb_ms", "download_ms")] + [
        (n, ctypes.c_uint64) for n in ("input_bytes", "output_bytes", "jpeg_blocks", "dv_blocks", "rgb_pixels",
                                      "idct_exact_samples")] + [
        ("launches", ctypes.c_uint32)] + [
        (n, ctypes.c_double) for n in ("slice_spec_ms", "slice_sync_ms", "slice_decode_ms")] + [
        ("graph_replays", ctypes.c_uint32), ("slices", ctypes.c_uint64), ("slices_redone", ctypes.c_uint64),
        ("dv_segment_ms", ctypes.c_double), ("dv_idct_ms", ctypes.c_double),
        ("slices_redone_whole", ctypes.c_uint64)]


class TuneEntry(ctypes.Structure):
    _fields_ = [("frame_class", ctypes.c_uint32), ("slice_bits", ctypes.c_uint32), ("frames", ctypes.c_uint32),
                ("kind", ctypes.c_uint32), ("entropy_ms", ctypes.c_double * 4), ("strip_mcus", ctypes.c_uint32),
                ("pad", ctypes.c_uint32), ("transform_ms", ctypes.c_double * 2)]


class JpegEncodeOptions(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("quality", ctypes.c_uint8), ("annex_k_huffman", ctypes.c_uint8),
                ("restart_interval", ctypes.c_uint16)]


class EncodeItem(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("frame", VideoFrameView), ("flags", ctypes.c_uint32),
                ("out", ctypes.c_void_p), ("out_capacity", ctypes.c_size_t), ("status", ctypes.c_int32),
                ("out_len", ctypes.c_size_t), ("message", ctypes.c_char * 200)]


class EncodeStats(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("device_ms", ctypes.c_double), ("blocks", ctypes.c_uint64),
                ("exact_coefficients", ctypes.c_uint64), ("bytes_out", ctypes.c_uint64)]


class StreamInfo(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("kind", ctypes.c_uint32), ("frame_status", ctypes.c_int32),
                ("frame_count", ctypes.c_size_t), ("y4m_bytes", ctypes.c_size_t), ("candidates", ctypes.c_uint64),
                ("upload_ms", ctypes.c_double), ("scan_ms", ctypes.c_double), ("message", ctypes.c_char * 512)]


class StreamResult(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_size_t), ("status", ctypes.c_int32), ("frames_written", ctypes.c_size_t),
                ("bytes_written", ctypes.c_size_t), ("message", ctypes.c_char * 512)]


# Every function the headers declare, with its ctypes signature.
SIGNATURES = {
    "mmr_abi_version": ([], ctypes.c_uint32),
    "mmr_version": ([], ctypes.c_char_p),
    "mmr_last_error_message": ([ctypes.c_char_p, ctypes.c_size_t], ctypes.c_size_t),
    "mmr_mjpeg_decode": ([ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(VideoFrameC)], ctypes.c_int32),
    "mmr_dv_decode": ([ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(VideoFrameC)], ctypes.c_int32),
    "mmr_mpeg2_picture_count": ([ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int32),
    "mmr_mpeg2_decode_picture": ([ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.POINTER(VideoFrameC)],
                                 ctypes.c_int32),
    "mmr_video_frame_free": ([ctypes.POINTER(VideoFrameC)], None),
    "mmr_mjpeg_encode": ([ctypes.POINTER(VideoFrameView), ctypes.c_uint8, ctypes.POINTER(Buffer)], ctypes.c_int32),
    "mmr_dv_encode": ([ctypes.POINTER(VideoFrameView), ctypes.POINTER(Buffer)], ctypes.c_int32),
    "mmr_mpeg2_encode": ([ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.POINTER(Buffer)], ctypes.c_int32),
    "mmr_mpegts_mux_mpeg2": ([ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(Buffer)], ctypes.c_int32),
    "mmr_mpegts_mux_mpeg2_mp2": ([ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                                 ctypes.POINTER(Buffer)], ctypes.c_int32),
    "mmr_mpegts_demux_mpeg2": ([ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(Buffer)], ctypes.c_int32),
    "mmr_mpegts_demux_mp2": ([ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(Buffer)], ctypes.c_int32),
    "mmr_buffer_free": ([ctypes.POINTER(Buffer)], None),
    "mmr_gpu_context_create": ([ctypes.POINTER(GpuConfig), ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int32),
    "mmr_gpu_context_destroy": ([ctypes.c_void_p], None),
    "mmr_gpu_probe": ([ctypes.c_uint32, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(FrameInfo)], ctypes.c_int32),
    "mmr_gpu_decode_batch": ([ctypes.c_void_p, ctypes.POINTER(GpuItem), ctypes.c_size_t], ctypes.c_int32),
    "mmr_gpu_last_batch_ms": ([ctypes.c_void_p], ctypes.c_double),
    "mmr_gpu_last_batch_launches": ([ctypes.c_void_p], ctypes.c_uint32),
    "mmr_gpu_set_slice_bits": ([ctypes.c_void_p, ctypes.c_uint32], ctypes.c_int32),
    "mmr_gpu_set_graphs": ([ctypes.c_void_p, ctypes.c_int], ctypes.c_int32),
    "mmr_gpu_autotune": ([ctypes.c_void_p, ctypes.POINTER(GpuItem), ctypes.c_size_t, ctypes.POINTER(TuneEntry),
                         ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)], ctypes.c_int32),
    "mmr_gpu_set_tuning": ([ctypes.c_void_p, ctypes.POINTER(TuneEntry), ctypes.c_size_t], ctypes.c_int32),
    "mmr_gpu_last_batch_stats": ([ctypes.c_void_p, ctypes.POINTER(BatchStats)], ctypes.c_int32),
    "mmr_mjpeg_encode_ex": ([ctypes.POINTER(VideoFrameView), ctypes.POINTER(JpegEncodeOptions), ctypes.POINTER(Buffer)],
                            ctypes.c_int32),
    "mmr_dv_encode_ex": ([ctypes.POINTER(VideoFrameView), ctypes.c_uint32, ctypes.POINTER(Buffer)], ctypes.c_int32),
    "mmr_dv_decode_static": ([ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                              ctypes.POINTER(FrameInfo)], ctypes.c_int32),
    "mmr_gpu_server_create": ([ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int32),
    "mmr_gpu_server_destroy": ([ctypes.c_void_p], None),
    "mmr_gpu_server_submit": ([ctypes.c_void_p, ctypes.POINTER(GpuItem), ctypes.POINTER(ctypes.c_uint64)],
                              ctypes.c_int32),
    "mmr_gpu_server_wait": ([ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int64, ctypes.POINTER(GpuItem),
                            ctypes.POINTER(ctypes.c_double)], ctypes.c_int32),
    "mmr_gpu_server_stats_get": ([ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ServerStats)], ctypes.c_int32),
    "mmr_gpu_server_set_slice_bits": ([ctypes.c_void_p, ctypes.c_uint32], ctypes.c_int32),
    "mmr_gpu_server_set_tuning": ([ctypes.c_void_p, ctypes.POINTER(TuneEntry), ctypes.c_size_t], ctypes.c_int32),
    "mmr_gpu_decoder_create": ([ctypes.c_uint32, ctypes.POINTER(ctypes.c_void_p)], ctypes.c_int32),
    "mmr_gpu_decoder_destroy": ([ctypes.c_void_p], None),
    "mmr_gpu_decoder_configure": ([ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p], ctypes.c_int32),
    "mmr_gpu_decoder_send_packet": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint64],
                                    ctypes.c_int32),
    "mmr_gpu_decoder_receive_frame": ([ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(VideoFrameC),
                                       ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int)], ctypes.c_int32),
    "mmr_gpu_decoder_flush": ([ctypes.c_void_p], ctypes.c_int32),
    "mmr_gpu_decoder_set_output": ([ctypes.c_void_p, ctypes.c_uint32], ctypes.c_int32),
    "mmr_gpu_decoder_receive_device_frame": ([ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(DeviceFrame),
                                              ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int)],
                                             ctypes.c_int32),
    "mmr_gpu_device_frame_release": ([ctypes.POINTER(DeviceFrame)], None),
    "mmr_gpu_server_replay": ([ctypes.c_void_p, ctypes.POINTER(GpuItem), ctypes.c_size_t,
                              ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_int64)], ctypes.c_int32),
    "mmr_gpu_stream_open": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_char_p,
                            ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(StreamInfo)], ctypes.c_int32),
    "mmr_gpu_stream_frame": ([ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_uint64),
                             ctypes.POINTER(ctypes.c_uint64)], ctypes.c_int32),
    "mmr_gpu_stream_decode_y4m": ([ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(StreamResult)],
                                  ctypes.c_int32),
    "mmr_gpu_stream_close": ([ctypes.c_void_p], None),
    "mmr_gpu_jpeg_encode_bound": ([ctypes.c_uint32, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_uint16], ctypes.c_size_t),
    "mmr_gpu_jpeg_encode_batch": ([ctypes.c_void_p, ctypes.POINTER(JpegEncodeOptions), ctypes.POINTER(EncodeItem),
                                  ctypes.c_size_t], ctypes.c_int32),
    "mmr_gpu_last_encode_stats": ([ctypes.c_void_p, ctypes.POINTER(EncodeStats)], ctypes.c_int32),
}

_lib = None


def load() -> ctypes.CDLL:
    """Loads the in-tree library, building it first if it is missing."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            _build.build()
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"libmmrecode_gpu.so is missing at {LIB_PATH}")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = res
        _lib = lib
    return _lib


def last_error() -> str:
    lib = load()
    n = lib.mmr_last_error_message(None, 0)
    buf = ctypes.create_string_buffer(n)
    lib.mmr_last_error_message(buf, n)
    return buf.value.decode("utf-8", "replace")
