"""bench.py's reference arm runs on the host cores (no GPU) and prints the
contract's JSON line: the same metric, unit and workload as the GPU arm's
default, impl "reference", a cpu_baseline describing the run and an e2e
entry with no host-device copies."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "1"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.strip().splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "F+X engine antenna-samples/s" and d["unit"] == "antenna-samples/s"
    assert d["higher_is_better"] is True and d["value"] > 0
    assert d["config"]["workload"] == "c3_array256"
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["e2e"]["value"] == d["value"]
