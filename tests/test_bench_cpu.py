"""bench.py's reference arm (CPU): one JSON line in the bench contract's shape.

`bench.py --impl reference` times the oracle port of the reference CPU path on the host cores; the GB300 arm
needs a GPU and is checked on the GPU machine.  This checks the reference line's keys and the rules it must
keep: at least three warm-up frames, and cpu_baseline / e2e describing the same measurement.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line():
    res = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1"],
                         cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, res.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "integrated_mpix_per_s" and d["unit"] == "Mpix/s"
    assert d["higher_is_better"] is True and d["value"] > 0
    assert d["steps"] >= 1 and d["warmup"] >= 3  # the bench's warm-up rule, even when fewer are asked for
    assert d["data"] == "synthetic" and "workload" in d["config"]
    cpu = d["cpu_baseline"]
    assert cpu["value"] == d["value"] and cpu["unit"] == d["unit"] and cpu["cores"] >= 1
    assert cpu["kind"] in ("reference", "port") and cpu["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
