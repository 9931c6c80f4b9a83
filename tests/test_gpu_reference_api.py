"""The reference-named device API, used the way a program written against the
reference's headers uses it.

tests/refapi/ref_api_history.cu includes only include/gcq/*.cuh and touches each
queue only through the reference's names: wf_mpmc_t<gwf_32k, 32768> with
wf_mpmc_init and Enqueue_Ptr/Dequeue_Ptr (gwf_queue.hpp:313-345, gwf_ring.hpp:
229-298, 1362-1380); fq_mpmc_t with fq_init and fq_enqueue_ptr/fq_dequeue_ptr
(glf_queue.hpp:126-138, 418-440, 566-582); wf_queue_host_init with
wf_enqueue/wf_dequeue on wf_handle* (wfqueue_hip_opt.hpp:161-178, 527-555, 594-764);
sfq_queue_host_init with sfq_enqueue/sfq_dequeue (sfqueue_hip.hpp:53-102,
sfqueue_hip.cpp:130-180, 356-399).  It records the history harness's shape
(correctness/history.cpp:188-227): 64 threads, 16 alternating enqueue/dequeue
pairs each, and the oracle must find every history linearizable.
"""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "refapi", "ref_api_history.cu")
OUT = os.path.join(ROOT, "tests", "refapi", "_build")
LIB = os.path.join(OUT, "libref_api.so")
KINDS = {"gwfq": 0, "glfq": 1, "wfq": 2, "sfq": 3}


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    pytest.skip("nvcc not found")


def _build():
    os.makedirs(OUT, exist_ok=True)
    hdrs = [os.path.join(ROOT, "include", "gcq", f) for f in os.listdir(os.path.join(ROOT, "include", "gcq"))]
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) > os.path.getmtime(p) for p in hdrs + [SRC]):
        return LIB
    cmd = [_nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
           "-shared", "-I" + os.path.join(ROOT, "include"), SRC, "-o", LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return LIB


def test_reference_api_compiles_against_headers_alone():
    """Cross-compiles for sm_103a here (no GPU needed): the reference's names and
    signatures exist in include/gcq/*.cuh."""
    lib = _build()
    assert os.path.getsize(lib) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("kind", sorted(KINDS))
def test_reference_api_history_linearizable(oracle_lib, kind):
    L = C.CDLL(_build())
    L.ref_api_history.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p]
    L.ref_api_history.restype = C.c_int
    threads, ops = 64, 16
    for rep in range(3):
        recs = np.zeros(threads * 2 * ops, dtype=oracle_lib.HIST_DTYPE)
        rc = L.ref_api_history(KINDS[kind], threads, ops, recs.ctypes.data)
        assert rc == 0, "CUDA error %d" % rc
        enq = recs[recs["op"] == 0]
        deq = recs[recs["op"] == 1]
        assert len(enq) == len(deq) == threads * ops
        assert np.all(enq["ret"] == 1)                     # capacity far above 64 x 16
        got = deq["ret"][deq["ret"] != 0]
        assert len(np.unique(got)) == len(got)             # no value twice
        assert set(got.tolist()) <= set(enq["arg"].tolist())
        order = np.lexsort((recs["op"], recs["proc"], recs["end"], recs["call"]))
        v = oracle_lib.check(recs[order], timeout_s=60.0)
        assert v == "Linearizable (FIFO)", (v, oracle_lib.patterns(recs[order]))


@pytest.mark.gpu
@pytest.mark.parametrize("kind", sorted(KINDS))
def test_reference_api_publishes_producer_writes(kind):
    """A queue of record ids between producer and consumer blocks: each producer
    fills a 32-byte record with plain stores and enqueues its id; each consumer
    dequeues ids and reads the records with plain loads.  The reference's enqueues
    publish the producer's earlier writes (gwf_ring.hpp:1362-1369 fences before the
    index enqueue), so no record may read incomplete, and every id arrives once."""
    L = C.CDLL(_build())
    L.ref_api_publish.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]
    L.ref_api_publish.restype = C.c_int
    for rep in range(3):
        out = np.zeros(5, dtype=np.uint64)
        rc = L.ref_api_publish(KINDS[kind], 8, 256, 8, out.ctypes.data)
        assert rc == 0, "CUDA error %d" % rc
        received, incomplete, gave_up, twice, total = (int(x) for x in out)
        assert gave_up == 0, out
        assert received == total == 4 * 256 * 8, out
        assert incomplete == 0 and twice == 0, out
