"""bench.py --impl reference on the host cores: the reference arm of the
benchmark contract prints one JSON line with the engine arm's metric, unit and
direction, the oracle port as its `cpu_baseline`, and an `e2e` block with no
host-device traffic (it never touches a GPU, so it runs here)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, r.stdout
    j = json.loads(lines[0])
    assert j["impl"] == "reference"
    sys.path.insert(0, ROOT)
    import bench
    assert j["metric"] == bench.METRIC
    assert j["unit"] == "Mrays/s" and j["higher_is_better"] is True
    assert j["steps"] == 1 and j["warmup"] >= 3 and j["n_gpus"] == 1
    assert j["value"] > 0 and j["ms_per_step"] > 0
    cb = j["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == j["value"]
    e2e = j["e2e"]
    assert e2e["value"] == j["value"] and e2e["unit"] == j["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
