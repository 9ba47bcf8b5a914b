"""Continuous-batching server: results in the mix equal results alone (and the
oracle), corrupt requests fail alone, the memory budget is enforced, and
latency statistics are reported."""

import random
import threading

import pytest

import mmrecode_gb300 as m
import oracle
from mmrecode_gb300 import synth

pytestmark = pytest.mark.gpu


def _mix():
    pk = []
    pk += [(p, m.CODEC_MJPEG, m.OUTPUT_RGB24) for p in synth.mjpeg_stream(501, 6, 1280, 720, "422", 85, 80)]
    pk += [(p, m.CODEC_MJPEG, m.OUTPUT_PLANAR) for p in synth.mjpeg_stream(502, 4, 640, 480, "420", 75, 0)]
    pk += [(p, m.CODEC_MJPEG, m.OUTPUT_RGB24) for p in synth.mjpeg_stream(503, 3, 352, 288, "444", 60, 4)]
    pk += [(p, m.CODEC_DV, m.OUTPUT_PLANAR) for p in synth.dv_stream(504, 4)]
    pk += [(p, m.CODEC_DV, m.OUTPUT_RGB24) for p in synth.dv_stream(505, 2)]
    bad = bytearray(pk[0][0])
    bad[len(bad) // 2] ^= 0x5A
    bad[len(bad) // 2 + 1] = 0xFF
    pk.append((bytes(bad), m.CODEC_MJPEG, m.OUTPUT_RGB24))
    pk.append((pk[-2][0][:5000], m.CODEC_DV, m.OUTPUT_PLANAR))  # wrong DV length
    return pk


def _expected(packet, codec, output):
    ref = oracle.jpeg_decode(packet) if codec == m.CODEC_MJPEG else oracle.dv_decode(packet, False)
    if ref.status:
        return ref.status, None
    if output == m.OUTPUT_RGB24:
        return 0, oracle.rgb24(ref.frame)
    return 0, b"".join(data for (_, _, data) in ref.frame.planes)


def test_mixed_requests_from_many_threads_match_alone_and_oracle():
    pk = _mix()
    rng = random.Random(506)
    order = list(range(len(pk))) * 3
    rng.shuffle(order)
    results = {}
    with m.Server(engines=3, max_batch=8) as srv:
        lock = threading.Lock()

        def client(idx):
            for i in idx:
                p, codec, output = pk[i]
                t = srv.submit(p, codec, output)
                r, payload, lat = srv.wait(t)
                assert lat > 0
                with lock:
                    results.setdefault(i, []).append((r.status, r.message, payload))

        threads = [threading.Thread(target=client, args=(order[k::6],)) for k in range(6)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        st = srv.stats()
        assert st["completed"] == len(order) and st["submitted"] == len(order)
        assert st["p99_ms"] >= st["p50_ms"] > 0
        assert st["batches"] >= 1
    with m.Context() as ctx:
        alone = ctx.decode_batch([p for p, _, _ in pk], [c for _, c, _ in pk], [o for _, _, o in pk])
    for i, (p, codec, output) in enumerate(pk):
        exp_status, exp_payload = _expected(p, codec, output)
        ra, pa = alone[i]
        assert ra.status == exp_status, i
        for status, message, payload in results[i]:
            assert status == exp_status, (i, message)
            assert message == ra.message, i
            assert payload == pa, i
            if exp_status == 0:
                assert payload == exp_payload, i


def test_memory_budget_refuses_oversized_requests_and_caps_batches():
    small = synth.mjpeg_stream(507, 6, 320, 240, "420", 75, 0)
    big = synth.mjpeg_stream(508, 1, 3840, 2160, "422", 90, 240)[0]
    budget = 3 * 4_000_000  # three engines, 4 MB each
    with m.Server(engines=3, max_batch=64, memory_budget=budget) as srv:
        with pytest.raises(m.MmrError) as e:
            srv.submit(big, m.CODEC_MJPEG, m.OUTPUT_RGB24)
        assert e.value.status == m.INVALID_ARGUMENT
        tickets = [srv.submit(p, m.CODEC_MJPEG, m.OUTPUT_PLANAR) for p in small]
        for t, p in zip(tickets, small):
            r, payload, _ = srv.wait(t)
            assert r.status == 0
            ref = oracle.jpeg_decode(p)
            assert payload == b"".join(d for (_, _, d) in ref.frame.planes)
        st = srv.stats()
        assert st["rejected"] == 1
        assert 0 < st["peak_budget_bytes"] <= budget


def test_unknown_ticket_and_timeout():
    with m.Server(engines=1) as srv:
        with pytest.raises(m.MmrError) as e:
            srv.wait(12345, timeout_s=0.0)
        assert e.value.status == m.INVALID_ARGUMENT
        p = synth.mjpeg_stream(509, 1, 64, 64, "420", 75, 0)[0]
        t = srv.submit(p)
        r, payload, lat = srv.wait(t, timeout_s=30.0)
        assert r.status == 0 and payload
        st = srv.stats(reset=True)
        assert st["completed"] == 1
        st = srv.stats()
        assert st["p50_ms"] == 0 and st["completed"] == 0  # new window


def test_open_loop_replay_returns_every_result():
    import ctypes
    from mmrecode_gb300 import _lib
    pk = synth.mjpeg_stream(510, 5, 320, 240, "422", 80, 20) + synth.dv_stream(511, 2)
    codecs = [m.CODEC_MJPEG] * 5 + [m.CODEC_DV] * 2
    n = 21
    keep, arr = [], (_lib.GpuItem * n)()
    for i in range(n):
        p, c = pk[i % 7], codecs[i % 7]
        src = (ctypes.c_uint8 * len(p)).from_buffer_copy(p)
        need = m.probe(c, p).planar_bytes
        dst = (ctypes.c_uint8 * need)()
        keep.append((src, dst))
        it = arr[i]
        it.struct_size = ctypes.sizeof(_lib.GpuItem)
        it.data, it.len, it.codec, it.output = ctypes.addressof(src), len(p), c, m.OUTPUT_PLANAR
        it.out, it.out_capacity = ctypes.addressof(dst), need
    arrivals = [0.0005 * i for i in range(n)]
    with m.Server(engines=2, max_batch=4) as srv:
        lat, lag = srv.replay(arr, arrivals)
    assert len(lat) == n and all(x > 0 for x in lat)
    for i in range(n):
        assert arr[i].status == 0, arr[i].message
        p, c = pk[i % 7], codecs[i % 7]
        ref = oracle.jpeg_decode(p) if c == m.CODEC_MJPEG else oracle.dv_decode(p, False)
        assert ctypes.string_at(keep[i][1], arr[i].out_bytes) == b"".join(d for (_, _, d) in ref.frame.planes), i


def test_installed_tuning_table_leaves_results_unchanged():
    pk = synth.mjpeg_stream(512, 4, 640, 480, "422", 85, 40) + synth.mjpeg_stream(513, 4, 352, 288, "444", 70, 0)
    table = [{"kind": "slice", "frame_class": (lay << 8) | b, "slice_bits": 1024} for lay in range(3) for b in range(20)]
    table += [{"kind": "strip", "frame_class": (v << 8) | b, "strip_mcus": 4 if v else 8}
              for v in range(3) for b in range(1, 9)]
    with m.Server(engines=2, max_batch=4) as srv:
        srv.set_tuning(table)
        tickets = [srv.submit(p, m.CODEC_MJPEG, m.OUTPUT_RGB24) for p in pk]
        for t, p in zip(tickets, pk):
            r, payload, _ = srv.wait(t)
            assert r.status == 0, r.message
            assert payload == oracle.rgb24(oracle.jpeg_decode(p).frame)
        with pytest.raises(m.MmrError):
            srv.set_tuning([{"kind": "slice", "frame_class": 0, "slice_bits": 7}])
