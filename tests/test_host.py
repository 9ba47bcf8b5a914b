"""Host-side Decoder-trait logic that needs no GPU: configuration and state errors.

Mirrors crates/codecs/mjpeg/src/codec.rs:290-378 (trait wrapper tests) and
the state checks of crates/codecs/dv/src/codec.rs:20-56."""

import pytest

import mmrecode_gb300 as m


@pytest.mark.parametrize("cls,name", [(m.MjpegDecoder, m.MJPEG_CODEC_NAME), (m.DvDecoder, m.DV_CODEC_NAME)])
def test_decoder_requires_configuration(cls, name):
    d = cls()
    for call in (lambda: d.send_packet(m.Packet(b"")), d.receive_frame, d.flush):
        with pytest.raises(m.MmrError) as e:
            call()
        assert e.value.status == m.INVALID_STATE
    with pytest.raises(m.MmrError) as e:
        d.configure(m.CodecDescriptor("video/other"))
    assert e.value.status == m.INVALID_DATA
    with pytest.raises(m.MmrError):
        d.configure(m.CodecDescriptor(name, "audio"))
    d.configure(m.CodecDescriptor(name))
    assert d.receive_frame() is None
    d.flush()


def test_batched_decoder_queues_until_full():
    d = m.MjpegDecoder(batch=4)
    d.configure(m.CodecDescriptor(m.MJPEG_CODEC_NAME))
    d._run_pending = lambda: pytest.fail("decoded before the batch was full")
    for _ in range(3):
        d.send_packet(m.Packet(b"\xff\xd8"))
    assert d.receive_frame() is None


def test_tuning_table_json_round_trip(tmp_path):
    import mmrecode_gb300 as m
    table = [{"kind": "slice", "frame_class": 269, "slice_bits": 4096, "frames": 12,
              "entropy_ms": {"1024": 1.5, "2048": 1.2, "4096": 1.1, "8192": 1.3}},
             {"kind": "strip", "frame_class": 263, "strip_mcus": 4, "frames": 6,
              "transform_ms": {"narrow": 0.2, "wide": 0.25}}]
    path = str(tmp_path / "t.json")
    m.save_tuning(path, table)
    assert m.load_tuning(path) == table
    (tmp_path / "bad.json").write_text('{"classes": []}')
    import pytest
    with pytest.raises(ValueError):
        m.load_tuning(str(tmp_path / "bad.json"))
