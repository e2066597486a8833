"""bench.py's reference arm runs on the host cores and prints one JSON line
with the keys the bench contract names. This arm needs no GPU, so the
contract is checked here on a 2-option sample."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_the_contract_line():
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "1", "--ref-sample", "2"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, p.stdout[-2000:]
    out = json.loads(lines[0])
    assert out["impl"] == "reference"
    if "unavailable" in out:
        return
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "config", "cpu_baseline", "e2e"):
        assert key in out, key
    assert out["value"] > 0 and out["higher_is_better"] is True
    assert out["steps"] == 1 and out["warmup"] == 1
    assert "workload" in out["config"]
    cb = out["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["value"] == out["value"]
    assert cb["unit"] == out["unit"] and cb["sample"]
    e2e = out["e2e"]
    assert e2e["value"] == out["value"] and e2e["unit"] == out["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
