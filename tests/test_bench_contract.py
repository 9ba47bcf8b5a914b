"""bench.py's reference arm on CPU: one JSON line on stdout with the keys and types of
the benchmark contract, the headline configuration (300 frames of 1920x1080 4:2:2 q90,
restart interval 120 MCUs, RGB24), a CPU baseline that names its cores and sample, and
an end-to-end figure with no host-device bytes. The arm times the oracle restatement of
the reference decoder (decode + RGB24 of every frame) on all host cores."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=900, cwd=ROOT)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.strip()]
    assert len(lines) == 1, p.stdout[-2000:]
    line = json.loads(lines[0])
    for key, kind in (("metric", str), ("value", float), ("unit", str), ("n_gpus", int), ("steps", int),
                      ("warmup", int), ("ms_per_step", float), ("higher_is_better", bool), ("scaling", str),
                      ("dtype", str), ("data", str), ("config", dict), ("cpu_baseline", dict), ("e2e", dict)):
        assert isinstance(line[key], kind), key
    assert line["impl"] == "reference" and line["vs_baseline"] is None
    assert (line["n_gpus"], line["steps"], line["warmup"], line["unit"]) == (1, 1, 0, "frames/s")
    assert line["value"] > 0 and abs(line["ms_per_step"] - 300 * 1000 / line["value"]) < 1e-6 * line["ms_per_step"]
    c = line["config"]
    assert c["workload"] == "mjpeg-1080p-422-q90-ri120mcu-rgb24"
    assert (c["frames_per_gpu"], c["width"], c["height"], c["subsampling"], c["quality"],
            c["restart_interval_mcus"], c["output"]) == (300, 1920, 1080, "422", 90, 120, "rgb24")
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == (os.cpu_count() or 1) and cb["value"] == line["value"]
    assert "300 frames" in cb["sample"]
    assert line["e2e"] == {"value": line["value"], "unit": "frames/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
