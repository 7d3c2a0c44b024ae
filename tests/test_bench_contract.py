"""bench.py's reference arm (the host CPU implementation of the path) prints
the one JSON line the benchmark contract asks for; it needs no GPU."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    out = subprocess.run(
        [sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1",
         "--cpu-seconds", "1", "--pairs", "128"],
        cwd=ROOT, capture_output=True, text=True, timeout=300, check=True).stdout
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out
    r = json.loads(lines[0])
    assert r["impl"] == "reference"
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config"):
        assert key in r, key
    assert r["unit"] == "GCUPS" and r["value"] > 0 and r["higher_is_better"] is True
    assert r["steps"] == 1 and r["warmup"] == 1
    assert "workload" in r["config"]
    cb = r["cpu_baseline"]
    assert cb["value"] == r["value"] and cb["cores"] >= 1 and cb["kind"] in ("reference", "port")
    assert cb["sample"]
    e = r["e2e"]
    assert e["value"] == r["value"] and e["unit"] == r["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
