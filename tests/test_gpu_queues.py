"""GPU parity tests: the CUDA queues, called through the C ABI of libgcq.so, checked
by the CPU oracle.  Dequeue values are nondeterministic, so parity means: every
history is linearizable under the reference's FIFO model, every FIFO drain is
exactly-once and per-producer ordered, and throughput counters balance."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

KINDS = ["gwfq", "glfq", "wfq", "sfq"]


def _lin(oracle_lib, recs):
    v = oracle_lib.check(recs, timeout_s=60.0)
    assert v == "Linearizable (FIFO)", (v, oracle_lib.patterns(recs))


@pytest.mark.parametrize("kind", KINDS)
def test_history_small_config(gcq, oracle_lib, kind):
    # the small history configuration: 64 threads, block 64, 16 alternating ops, capacity 2^15
    with gcq.Queue(kind, 15, 64) as q:
        for rep in range(3):
            recs = q.history(threads=64, ops=16, block=64)
            assert len(recs) == 64 * 16 * 2
            _lin(oracle_lib, recs)
        assert q.error_word() & ~gcq.ERR_POOL == 0


@pytest.mark.parametrize("kind", KINDS)
def test_history_u32_values(gcq, oracle_lib, kind):
    with gcq.Queue(kind, 15, 64) as q:
        recs = q.history(threads=64, ops=16, block=64, value_mode=1)
        _lin(oracle_lib, recs)


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("threads,block", [(256, 256), (1024, 256)])
def test_history_larger(gcq, oracle_lib, kind, threads, block):
    with gcq.Queue(kind, 15, threads) as q:
        recs = q.history(threads=threads, ops=8, block=block)
        _lin(oracle_lib, recs)


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("pct", [25, 50, 75])
def test_history_split(gcq, oracle_lib, kind, pct):
    # split mode at a size the exact search decides (it is exponential in the number
    # of concurrent producers in the worst case, like the reference's checker)
    with gcq.Queue(kind, 15, 32) as q:
        for rep in range(3):
            recs = q.history(threads=32, ops=16, block=32, mode=1, producer_percent=pct)
            _lin(oracle_lib, recs)


@pytest.mark.parametrize("kind", KINDS)
def test_history_split_large_patterns(gcq, oracle_lib, kind):
    # 1024 threads: the O(n log n) pattern scan (sound; complete when no dequeue
    # reports empty) must find no violation
    with gcq.Queue(kind, 15, 1024) as q:
        recs = q.history(threads=1024, ops=16, block=256, mode=1, producer_percent=50)
        rep = oracle_lib.patterns(recs)
        assert not rep["violations"], rep


@pytest.mark.parametrize("kind", ["gwfq", "glfq"])
def test_history_small_ring_wraps(gcq, oracle_lib, kind):
    # capacity 2^6 with 64 threads: many ring cycles and full/empty boundaries
    with gcq.Queue(kind, 6, 64) as q:
        for rep in range(3):
            recs = q.history(threads=64, ops=64, block=64)
            _lin(oracle_lib, recs)
            recs = q.history(threads=16, ops=32, block=32, mode=1, producer_percent=50)
            _lin(oracle_lib, recs)


def test_gwfq_slow_path_and_helping(gcq, oracle_lib):
    """Patience 2 sends almost every G-WFQ operation to the wait-free slow path
    (cooperative fetch-and-add, phase-2 records, Enq=0 two-step insertion) and a
    help delay of 1 makes every operation help a peer."""
    with gcq.Queue("gwfq", 8, 128, enq_patience=2, deq_patience=2, help_delay=1) as q:
        for rep in range(3):
            recs = q.history(threads=128, ops=32, block=128)
            _lin(oracle_lib, recs)
            recs = q.history(threads=32, ops=16, block=32, mode=1, producer_percent=50)
            _lin(oracle_lib, recs)
        assert q.error_word() == 0
    # every token exactly once through slow-path enqueues and dequeues at 256
    # threads (phase-2 helpers check the record they help, gwf_ring.hpp:548-590)
    with gcq.Queue("gwfq", 15, 256, enq_patience=2, deq_patience=2, help_delay=1) as q:
        r = q.fifo_check(threads=256, ops_per_thread=32)
        assert r["verified"] == 1, r
        assert q.error_word() == 0


def test_ymc_slow_path_and_helping(gcq, oracle_lib):
    """Patience 0 sends every YMC operation that misses its first cell to the slow
    path (enqueue requests bound to cells by dequeuers, dequeue requests announced
    and claimed by helpers): histories check linearizable and a produce-then-drain
    FIFO check takes every token exactly once."""
    with gcq.Queue("wfq", 0, 1024, ymc_patience=0) as q:
        for rep in range(3):
            recs = q.history(threads=128, ops=32, block=128)
            _lin(oracle_lib, recs)
            recs = q.history(threads=32, ops=16, block=32, mode=1, producer_percent=50)
            _lin(oracle_lib, recs)
        r = q.fifo_check(threads=256, ops_per_thread=32)
        assert r["verified"] == 1, r
        assert q.error_word() & ~gcq.ERR_POOL == 0


def test_gwfq_remap_layout(gcq, oracle_lib):
    with gcq.Queue("gwfq", 10, 256, remap=1) as q:
        recs = q.history(threads=256, ops=16, block=256)
        _lin(oracle_lib, recs)


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("threads", [1024, 8192])
def test_fifo_drain(gcq, kind, threads):
    with gcq.Queue(kind, 15, threads) as q:
        r = q.fifo_check(threads=threads, ops_per_thread=32)
        assert r["verified"] == 1, r
        assert r["in_count"] == r["out_count"] == threads * r["ops_per_thread"]


def test_fifo_drain_skipped_when_over_capacity(gcq):
    # 2^15 capacity, 65536 threads: cap/threads = 0 -> skipped, as the reference does
    with gcq.Queue("glfq", 15, 65536) as q:
        assert q.fifo_check(threads=65536, ops_per_thread=32)["verified"] == -1


@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("mode", [0, 1])
def test_throughput_counters(gcq, kind, mode):
    threads = 4096
    with gcq.Queue(kind, 15, threads) as q:
        r = q.tb_run(mode=mode, threads=threads, chunk_ops=64, warmup_ms=20, run_ms=100, graph_chunks=4)
        assert r["launches"] >= 4 and r["gpu_ms"] > 0
        ops = r["launches"] * threads * 64
        if mode == 0:
            assert r["enq_success"] + r["enq_fail"] == ops
            assert r["deq_success"] + r["deq_empty"] == ops
        if kind != "wfq":
            assert r["succ_mops"] > 0
        # a balanced run leaves at most `threads` values queued per launch boundary
        assert r["deq_success"] <= r["enq_success"] + (1 << 15)
        assert q.error_word() & ~gcq.ERR_POOL == 0


def test_chunk_host_matches_device_counts(gcq):
    threads, chunk = 8192, 32
    rng = np.random.default_rng(5)
    pay = rng.integers(0, 2**32, size=threads * chunk, dtype=np.uint64).astype(np.uint32)
    with gcq.Queue("gwfq", 15, threads) as q:
        c = q.tb_chunk_host(0, threads, chunk, pay)
        assert c["enq_success"] + c["enq_fail"] == threads * chunk
        assert c["deq_success"] + c["deq_empty"] == threads * chunk
        assert c["enq_success"] == threads * chunk     # capacity 2^15 >= threads: never full
        assert c["deq_success"] >= c["enq_success"] - threads


def test_tb_chunk_host_pinned_in_place(gcq):
    """Pinned payloads are read by the kernel in place over the host link; the
    counts equal those of the staged (pageable) path for the same payloads."""
    torch = pytest.importorskip("torch")
    threads, chunk = 8192, 16
    rng = np.random.default_rng(6)
    vals = rng.integers(0, 2**32, size=threads * chunk, dtype=np.uint64).astype(np.uint32)
    pinned = torch.empty(threads * chunk, dtype=torch.int32).pin_memory()
    pin = pinned.numpy().view(np.uint32)
    pin[:] = vals
    for mode in (0, 1):
        with gcq.Queue("gwfq", 15, threads) as q:
            a = q.tb_chunk_host(mode, threads, chunk, pin)
        with gcq.Queue("gwfq", 15, threads) as q:
            b = q.tb_chunk_host(mode, threads, chunk, vals.copy())
        assert a["enq_success"] + a["enq_fail"] == b["enq_success"] + b["enq_fail"]
        if mode == 0:
            assert a["enq_success"] == b["enq_success"] == threads * chunk
            assert a["deq_success"] + a["deq_empty"] == threads * chunk


def test_envelope_rejections(gcq):
    # G-WFQ requires max_threads <= capacity (gwf_queue.hpp:320)
    with pytest.raises(gcq.GcqError) as e:
        gcq.Queue("gwfq", 10, 2048)
    assert e.value.status == gcq.EUNSUPPORTED
    # SFQ: MAX_ID >= 2 (max_threads + 1) (sfqueue_hip.hpp:45-47); L = 2^20 allows 4095
    with pytest.raises(gcq.GcqError):
        gcq.Queue("sfq", 20, 8192)
    gcq.Queue("sfq", 20, 4095).close()
    # the SCQ rings hold Threshold = 3N - 1 in an int: N <= 2^29
    for kind in ("gwfq", "glfq"):
        with pytest.raises(gcq.GcqError) as e:
            gcq.Queue(kind, 30, 64)
        assert e.value.status == gcq.EINVAL
