"""Correctness at the sizes the benchmarks time.

The throughput bench times G-WFQ and G-LFQ balanced at 262144 threads with
capacity 2^20, G-WFQ split at 65536 threads, SFQ at 32768 threads with length
2^16 and YMC at 65536 threads.  The chunk kernel only counts operations, so these
tests run the same queues, at the same sizes, through checks that look at the
values:

* the reference's FIFO mode (produce, then drain; throughout_bench.cpp:456-767),
  with ops per thread capped to capacity / threads as the reference caps it
  (:627-653): exactly once, and per producer in order;
* the same check with producers and consumers running at once, in the split
  kernel's roles (gcq_fifo_check_split);
* split-mode histories of 16384 threads through the oracle's O(n log n) pattern
  scan (sound: every pattern it reports is a violation; complete for the value
  patterns when no dequeue reports empty).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,cap,threads", [("gwfq", 20, 262144), ("glfq", 20, 262144),
                                               ("sfq", 16, 32768), ("wfq", 0, 65536)])
def test_fifo_drain_at_bench_size(gcq, kind, cap, threads):
    with gcq.Queue(kind, cap, threads) as q:
        r = q.fifo_check(threads=threads, ops_per_thread=32)
        assert r["verified"] == 1, r
        if kind != "wfq":
            assert r["ops_per_thread"] == min(32, (1 << cap) // threads)
        assert r["in_count"] == r["out_count"] == threads * r["ops_per_thread"]
        assert q.error_word() & ~gcq.ERR_POOL == 0


@pytest.mark.parametrize("kind,cap,threads", [("gwfq", 20, 65536), ("glfq", 20, 65536), ("gwfq", 15, 16384),
                                               ("glfq", 15, 16384), ("sfq", 16, 32768), ("wfq", 0, 8192)])
@pytest.mark.parametrize("pct", [50, 25])
def test_fifo_split_concurrent(gcq, kind, cap, threads, pct):
    """Split roles at the timed split size: consumers take tokens while producers
    still make them; every token comes out once and each producer's tokens come out
    in the order it made them."""
    with gcq.Queue(kind, cap, threads) as q:
        r = q.fifo_check_split(threads=threads, producer_percent=pct, ops_per_producer=32)
        assert r["verified"] == 1, r
        assert r["in_count"] == r["out_count"] > 0
        assert q.error_word() & ~gcq.ERR_POOL == 0


def test_fifo_split_rejects_non_resident(gcq):
    # producers and consumers wait for each other: every thread must be resident
    with gcq.Queue("glfq", 20, 1 << 20) as q:
        with pytest.raises(gcq.GcqError) as e:
            q.fifo_check_split(threads=1 << 20, producer_percent=50, ops_per_producer=4)
        assert e.value.status == gcq.EUNSUPPORTED


@pytest.mark.parametrize("kind,cap", [("gwfq", 15), ("glfq", 15), ("sfq", 16), ("wfq", 0)])
def test_split_history_16384_threads_patterns(gcq, oracle_lib, kind, cap):
    threads = 16384
    with gcq.Queue(kind, cap, threads) as q:
        recs = q.history(threads=threads, ops=16, block=256, mode=1, producer_percent=50)
        assert len(recs) == threads * 16
        rep = oracle_lib.patterns(recs)
        assert not rep["violations"], rep
        assert q.error_word() & ~gcq.ERR_POOL == 0


@pytest.mark.parametrize("kind,cap,threads", [("gwfq", 20, 262144), ("glfq", 20, 262144)])
def test_balanced_chunk_then_drain_conserves_payloads(gcq, kind, cap, threads):
    """One balanced chunk at the timed size through the end-to-end entry point,
    then a drain: every value dequeued in the chunk plus every value left behind
    is one of the chunk's payloads, and the counts add up."""
    chunk = 8
    rng = np.random.default_rng(21)
    pay = rng.integers(1, 2**32, size=threads * chunk, dtype=np.uint64).astype(np.uint32)
    with gcq.Queue(kind, cap, threads) as q:
        c = q.tb_chunk_host(0, threads, chunk, pay)
        assert c["enq_success"] == threads * chunk and c["enq_fail"] == 0
        left = q.drain_host(threads=4096, cap=1 << 21)
        assert len(left) == c["enq_success"] - c["deq_success"]
        vals, cnt = np.unique(pay, return_counts=True)
        lv, lc = np.unique(left, return_counts=True)
        pos = np.searchsorted(vals, lv)
        assert np.all(pos < len(vals)) and np.array_equal(vals[pos], lv)
        assert np.all(lc <= cnt[pos])
        assert q.error_word() == 0
