"""gcq_tb_chunk_host_noalloc, the chunk entry point that allocates no device memory.

Some callers cannot allocate while they run (stream-ordered or pool-managed memory,
real-time paths that must not take allocator locks, embedders that own all device
memory); this variant stages through a fixed array inside libgcq.so instead.  Its
results must equal those of gcq_tb_chunk_host, on two calls in a row (the second
call sees the array the first one left behind).  This file is collected last so
that a failure here does not stop the other tests from running.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _call(gcq, q, pay, threads, chunk):
    c = gcq.TbCounters()
    rc = gcq.lib().gcq_tb_chunk_host_noalloc(q.handle, 0, 50, threads, 256, chunk, pay.ctypes.data,
                                             C.byref(c), None)
    assert rc == gcq.OK, gcq.lib().gcq_strerror(rc)
    return (c.enq_success, c.enq_fail, c.deq_success, c.deq_empty)


def test_noalloc_matches_chunk_host_twice(gcq):
    threads, chunk = 8192, 64
    rng = np.random.default_rng(11)
    pay = rng.integers(0, 2**32, size=threads * chunk, dtype=np.uint64).astype(np.uint32)
    with gcq.Queue("gwfq", 15, threads) as q:
        ref = q.tb_chunk_host(0, threads, chunk, pay)
        want = (ref["enq_success"], ref["enq_fail"], ref["deq_success"], ref["deq_empty"])
        # balanced mode with capacity >= threads: every enqueue and every dequeue
        # succeeds in a linearizable queue, so the counts are exact
        assert want == (threads * chunk, 0, threads * chunk, 0)
        first = _call(gcq, q, pay, threads, chunk)
        second = _call(gcq, q, pay, threads, chunk)
        assert first == want
        assert second == want
        assert q.error_word() == 0


def test_noalloc_payloads_reach_the_queue_twice(gcq):
    """The payloads themselves, not only the counts: with every thread a producer
    (split mode, 100 %), a call enqueues all its payloads, and a drain returns
    exactly that multiset -- from gcq_tb_chunk_host and from the no-allocation entry
    point alike, on two calls in a row with different payloads (the second call
    stages over what the first one left in the shared array)."""
    threads, chunk = 4096, 16
    rng = np.random.default_rng(13)
    for rep in range(2):
        pay = rng.integers(0, 2**32, size=threads * chunk, dtype=np.uint64).astype(np.uint32)
        want = np.sort(pay.astype(np.uint64))
        with gcq.Queue("gwfq", 16, threads) as q:
            c = q.tb_chunk_host(1, threads, chunk, pay, producer_percent=100)
            assert c["enq_success"] == threads * chunk
            ref = np.sort(q.drain_host(threads=1024, cap=1 << 17))
        with gcq.Queue("gwfq", 16, threads) as q:
            c = q.tb_chunk_host_noalloc(1, threads, chunk, pay, producer_percent=100)
            assert c["enq_success"] == threads * chunk
            got = np.sort(q.drain_host(threads=1024, cap=1 << 17))
            assert q.error_word() == 0
        assert np.array_equal(ref, want)
        assert np.array_equal(got, want)


def test_noalloc_rejects_oversize(gcq):
    threads, chunk = 65536, 128   # 8 Mi payloads > 4 Mi maximum
    pay = np.zeros(threads * chunk, dtype=np.uint32)
    with gcq.Queue("gwfq", 17, threads) as q:
        c = gcq.TbCounters()
        rc = gcq.lib().gcq_tb_chunk_host_noalloc(q.handle, 0, 50, threads, 256, chunk, pay.ctypes.data,
                                                 C.byref(c), None)
        assert rc == gcq.ECAPACITY
