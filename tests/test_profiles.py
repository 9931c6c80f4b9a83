"""The committed ncu summaries under profiles/: the bench reads its roofline traffic
from one of them, and every capture they record was taken without locking the
GPU's clocks."""
import glob
import os
import re
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def test_bench_reads_headline_traffic():
    import bench
    pv = bench.profile_values(bench.TB_PROFILE)
    for k in ("dram_bytes_per_launch", "l2_atomic_requests_per_launch", "l2_red_requests_per_launch",
              "ops_per_launch"):
        assert k in pv and pv[k] > 0, (k, pv)
    # the headline launch: 262144 threads x 128 balanced iterations, enqueue + dequeue
    assert pv["ops_per_launch"] == 262144 * 128 * 2


def test_profile_values_absent_file():
    import bench
    assert bench.profile_values("no_such_profile.md") == {}


def test_every_ncu_command_keeps_clocks():
    files = glob.glob(os.path.join(ROOT, "profiles", "*.md")) + glob.glob(os.path.join(ROOT, "profiles", "*.txt"))
    assert files
    for f in files:
        text = open(f).read()
        # join continued command lines, then look at each ncu invocation
        joined = re.sub(r"\\\s*\n\s*", " ", text)
        for m in re.finditer(r"(?m)^\s*ncu\s+--.*$", joined):
            assert "--clock-control none" in m.group(0), (os.path.basename(f), m.group(0))
