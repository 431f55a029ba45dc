"""bench.py's reference arm runs on the CPU (the C oracle on the host cores) and prints the one JSON
line the measurement contract asks for: the same metric, unit and workload as the GPU arm, with
impl = reference, a cpu_baseline describing the run and an e2e object without device copies; a
requested warm-up below 3 steps is raised to 3."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_json_line(built):
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0"],
                         cwd=ROOT, check=True, capture_output=True, text=True, timeout=600).stdout
    lines = [l for l in out.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out
    r = json.loads(lines[0])
    import bench
    assert r["impl"] == "reference"
    assert r["metric"] == bench.METRIC and r["unit"] == bench.UNIT and r["higher_is_better"] is True
    assert r["steps"] == 1 and r["warmup"] == 3 and r["n_gpus"] == 1   # at least 3 warm-up steps, always
    assert r["value"] > 0 and r["ms_per_step"] > 0
    cb = r["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == r["value"] and cb["sample"]
    e2e = r["e2e"]
    assert e2e["value"] == r["value"] and e2e["unit"] == r["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert "batched sweep" in r["config"]["workload"] and r["data"] == "synthetic"
