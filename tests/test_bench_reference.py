"""bench.py's reference arm (libmceliece itself on the host cores, the oracle port where its sources
are absent) prints one JSON line with the main arm's metric, unit and workload, and an e2e entry without
host-device traffic; it needs no GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_reference_arm_line():
    import bench

    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0",
                          "--set", "348864", "--n", "4096"], cwd=ROOT, capture_output=True, text=True, timeout=600,
                         check=True)
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.metric_name("348864")
    assert line["unit"] == "KEM ops/s (enc+dec, 50/50)" and line["higher_is_better"] is True
    assert line["config"]["workload"] == bench.workload("348864", 4096, 0.10)
    assert line["value"] > 0
    from oracle import pyref
    assert line["cpu_baseline"]["kind"] == ("reference" if pyref.available() else "port")
    assert line["config"]["n_per_gpu"] == 4096
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
