"""bench.py's reference arm on the CPU: the oracle's serial restatements on the
host cores, one JSON line with the GPU arm's metric and the reference keys."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("workload, metric_start, unit", [
    ("rt", "RT MRays/s", "MRays/s"),
    ("bfs", "BFS traversals/s", "traversals/s"),
    ("served-bfs", "served BFS traversals/s", "traversals/s"),
])
def test_reference_arm_line(workload, metric_start, unit):
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", workload, "--steps", "1"],
                       cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"].startswith(metric_start) and d["unit"] == unit
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["kind"] == "port"
    assert d["e2e"] == {"value": d["value"], "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
