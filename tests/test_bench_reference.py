"""bench.py's reference arm on CPU: the oracle timed on the host cores after
the same warm-up as the GPU arm (at least 20 steps), printed as one JSON line
with the arm's keys, without the product library loaded. Runs the
49,600-particle dam break (configuration 0) to stay quick."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--config", "0", "--steps", "2", "--warmup", "3", "--cpu-steps", "1"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "particle-steps/s" and d["higher_is_better"] is True
    # the GPU arm warms up max(--warmup, 20) steps; so does this arm
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 20
    assert d["config"]["particles"] == 49600
    assert d["config"]["steps_timed"] == "21..21"
    assert d["config"]["gpu_arm_steps_timed"] == "21..22"
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert "steps 21..21" in cb["sample"]
    # the oracle only: the product library is never mapped into the arm
    assert "oracle/liboracle.so" in d["libraries_loaded"]
    assert not any("libfluidsph" in f for f in d["libraries_loaded"]), d["libraries_loaded"]
    assert d["e2e"] == {"value": d["value"], "unit": "particle-steps/s",
                        "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
