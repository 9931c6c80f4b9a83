"""Race detection on the CPU restatements of the four queues: the oracle's
ThreadSanitizer build runs histories (alternating and split) and FIFO drains of
every queue with 8 host threads, and the stalled-thread helping case of G-WFQ;
ThreadSanitizer must report nothing and every history must still check
linearizable."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
from oracle import lib
for kind in ("gwfq", "glfq", "wfq", "sfq"):
    for mode in (0, 1):
        h = lib.cpu_history(kind, 8, 32, mode=mode)
        assert lib.check(h) == "Linearizable (FIFO)", (kind, mode)
    r = lib.cpu_fifo_check(kind, 8, 64)
    assert r["verified"] and r["dup"] == 0 and r["missing"] == 0, (kind, r)
import numpy as np
st = np.zeros(4, np.uint64)
assert lib.lib().oracle_gwf_stalled_helping(8, 64, 1, st.ctypes.data) == 1, st
print("ok")
"""


def test_queue_ports_race_free():
    try:
        tsan = subprocess.run(["gcc", "-print-file-name=libtsan.so"], capture_output=True, text=True).stdout.strip()
    except OSError:
        pytest.skip("no gcc")
    if not tsan or not os.path.isabs(tsan) or not os.path.exists(tsan):
        pytest.skip("no ThreadSanitizer runtime")
    from oracle import build
    lib = build.build(sanitize="thread")
    env = dict(os.environ, LD_PRELOAD=tsan, GCQ_ORACLE_LIBRARY=lib, TSAN_OPTIONS="exitcode=66")
    r = subprocess.run([sys.executable, "-c", SCRIPT], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    if "unexpected memory mapping" in r.stderr or "FATAL: ThreadSanitizer" in r.stderr:
        pytest.skip("ThreadSanitizer cannot run in this environment")
    assert "WARNING: ThreadSanitizer" not in r.stderr, r.stderr[-4000:]
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), (r.returncode, r.stderr[-2000:])
