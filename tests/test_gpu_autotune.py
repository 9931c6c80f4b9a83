"""The autotuner (gcq_tb_autotune): every candidate is a real throughput run of a
fresh queue; the returned best point is the fastest one measured."""
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,cap,threads", [("gwfq", 16, 16384), ("sfq", 14, 2048)])
def test_autotune_small(gcq, kind, cap, threads):
    r = gcq.autotune(kind, cap, threads, mode=0, ms_per_point=15.0, passes=1)
    best, table = r["best"], r["table"]
    measured = [p for p in table if p["status"] == 0]
    assert len(measured) >= 4
    assert best["succ_mops"] > 0
    assert best["succ_mops"] == max(p["succ_mops"] for p in measured)
    assert threads % best["block"] == 0
    # the default point (block 256, chunk 128) is measured first
    assert (table[0]["block"], table[0]["chunk_ops"]) == (256, 128)
