"""ctypes bindings to oracle/_build/liboracle.so (test infrastructure only).

Covers the FIFO linearizability checker (lincheck.cpp), the std::atomic CPU
restatements of the four queues (cpu_queues.cpp), the serial BFS
(bfs_serial.cpp) and the serial renders (rt_cpu.cpp: the reference's scenes, the
stream-compaction comparator's shading, and the benchmark scenes).
"""
from __future__ import annotations

import ctypes as C
import itertools
import json
import os

import numpy as np

from . import build as _build

KINDS = {"gwfq": 0, "glfq": 1, "wfq": 2, "sfq": 3}
VERDICT = {0: "Linearizable (FIFO)", 1: "Not linearizable (FIFO)", 2: "Unknown (timeout)"}

# Same layout as gcq_log_entry in include/gcq.h and gcq_hist_rec in lincheck.cpp.
HIST_DTYPE = np.dtype([("proc", "<u8"), ("op", "<u4"), ("_pad", "<u4"), ("arg", "<u8"),
                       ("ret", "<u8"), ("call", "<i8"), ("end", "<i8")])


class TbStats(C.Structure):
    _fields_ = [("enq_success", C.c_uint64), ("enq_fail", C.c_uint64),
                ("deq_success", C.c_uint64), ("deq_empty", C.c_uint64),
                ("elapsed_ms", C.c_double), ("threads", C.c_uint32), ("_pad", C.c_uint32)]


class PatternReport(C.Structure):
    _fields_ = [("fresh", C.c_uint64), ("repeat", C.c_uint64),
                ("order", C.c_uint64), ("empty", C.c_uint64)]


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        # GCQ_ORACLE_LIBRARY selects another build of the same sources (the
        # ThreadSanitizer copy of the race tests)
        path = os.environ.get("GCQ_ORACLE_LIBRARY") or os.path.join(_build.OUT, "liboracle.so")
        if not os.path.exists(path):
            path = _build.build()
        L = C.CDLL(path)
        P = C.c_void_p
        L.gcq_lincheck_records.argtypes = [P, C.c_size_t, C.c_double]
        L.gcq_lincheck_records.restype = C.c_int
        L.gcq_lincheck_search.argtypes = [P, C.c_size_t, C.c_double]
        L.gcq_lincheck_search.restype = C.c_int
        L.gcq_lincheck_patterns.argtypes = [P, C.c_size_t, C.POINTER(PatternReport)]
        L.gcq_lincheck_patterns.restype = C.c_int
        L.gcq_lincheck_parse_jsonl.argtypes = [C.c_char_p, P, C.c_size_t, C.POINTER(C.c_size_t)]
        L.gcq_lincheck_parse_jsonl.restype = C.c_int
        L.oracle_history.argtypes = [C.c_int, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, C.c_int,
                                     C.c_int, P, C.c_uint64]
        L.oracle_history.restype = C.c_int64
        L.oracle_tb_run.argtypes = [C.c_int, C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_double,
                                    C.c_double, C.POINTER(TbStats)]
        L.oracle_tb_run.restype = C.c_int
        L.oracle_fifo_check.argtypes = [C.c_int, C.c_uint32, C.c_uint32, C.c_uint32, P]
        L.oracle_fifo_check.restype = C.c_int
        for name, args, res in _EXTRA:
            if hasattr(L, name):
                f = getattr(L, name)
                f.argtypes = args
                f.restype = res
        _LIB = L
    return _LIB


_EXTRA = [
    ("oracle_bfs", [C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p], C.c_int32),
    ("oracle_rt_render", [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p], C.c_int64),
    ("oracle_rt_compact_render", [C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p], C.c_int64),
    ("oracle_rt_bounce_render", [C.c_int, C.c_int, C.c_int, C.c_int, C.c_uint64, C.c_int, C.c_void_p],
     C.c_int64),
    ("oracle_levels_checksum", [C.c_int32, C.c_void_p], C.c_uint64),
    ("oracle_gwf_slow_passed_slot", [C.c_int, C.c_void_p], C.c_int),
    ("oracle_gwf_finalize_loser", [C.c_int, C.c_void_p], C.c_int),
    ("oracle_gwf_stalled_helping", [C.c_uint32, C.c_uint32, C.c_uint32, C.c_void_p], C.c_int),
    ("oracle_gwf_slow_stress", [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_int],
     C.c_int),
    ("oracle_ymc_slow_stress", [C.c_uint32, C.c_uint32, C.c_int, C.c_uint32], C.c_int),
    ("oracle_gwf_split_stress", [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                 C.c_uint32, C.c_int], C.c_int),
    ("oracle_gwf_device_model_stress", [C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                        C.c_int, C.c_int, C.c_int, C.c_uint32], C.c_int),
    ("oracle_port_mpmc_stress", [C.c_int, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32, C.c_uint32,
                                 C.c_uint32], C.c_int),
    ("oracle_glf_device_model_stress", [C.c_uint32, C.c_uint32, C.c_uint32, C.c_int, C.c_int, C.c_uint32, C.c_uint32],
     C.c_int),
]


# ------------------------------------------------------------------ BFS
def bfs(offsets: np.ndarray, indices: np.ndarray, src: int):
    """Serial BFS depths (-1 unreached) and the eccentricity of src."""
    off = np.ascontiguousarray(offsets, dtype=np.int32)
    idx = np.ascontiguousarray(indices, dtype=np.int32)
    lv = np.empty(len(off) - 1, dtype=np.int32)
    ecc = lib().oracle_bfs(len(off) - 1, off.ctypes.data, idx.ctypes.data, int(src), lv.ctypes.data)
    if ecc < 0:
        raise ValueError("bad source vertex %d" % src)
    return lv, ecc


def levels_checksum(levels: np.ndarray) -> int:
    """Checksum of a level array as the served traversals report it."""
    lv = np.ascontiguousarray(levels, dtype=np.int32)
    return int(lib().oracle_levels_checksum(len(lv), lv.ctypes.data))


def bfs_summary(offsets: np.ndarray, indices: np.ndarray, src: int):
    """(checksum, reached, eccentricity) of one traversal, as a served request answers."""
    lv, ecc = bfs(offsets, indices, src)
    return levels_checksum(lv), int(np.count_nonzero(lv >= 0)), int(ecc)


# ------------------------------------------------------------------ histories
def records_from_dicts(recs) -> np.ndarray:
    a = np.zeros(len(recs), dtype=HIST_DTYPE)
    for i, r in enumerate(recs):
        a[i] = (r["proc"], r["op"], 0, r.get("arg", 0), r["ret"], r["call"], r["end"])
    return a


def load_jsonl(path) -> np.ndarray:
    with open(path) as f:
        return records_from_dicts([json.loads(l) for l in f if l.strip()])


def check(records: np.ndarray, timeout_s: float = 10.0) -> str:
    """Exact search (Wing-Gong with Lowe's memoisation); returns the verdict string."""
    a = np.ascontiguousarray(records, dtype=HIST_DTYPE)
    rc = lib().gcq_lincheck_records(a.ctypes.data, len(a), timeout_s)
    if rc < 0:
        raise ValueError("malformed history")
    return VERDICT[rc]


def search(records: np.ndarray, timeout_s: float = 10.0) -> str:
    """The exact search alone, without the pattern pre-check."""
    a = np.ascontiguousarray(records, dtype=HIST_DTYPE)
    rc = lib().gcq_lincheck_search(a.ctypes.data, len(a), timeout_s)
    if rc < 0:
        raise ValueError("malformed history")
    return VERDICT[rc]


def patterns(records: np.ndarray) -> dict:
    """O(n log n) violation-pattern scan for distinct-value histories."""
    a = np.ascontiguousarray(records, dtype=HIST_DTYPE)
    rep = PatternReport()
    rc = lib().gcq_lincheck_patterns(a.ctypes.data, len(a), C.byref(rep))
    if rc == -2:
        raise ValueError("values are not distinct")
    return {"fresh": rep.fresh, "repeat": rep.repeat, "order": rep.order, "empty": rep.empty,
            "violations": rc == 1}


def brute_force(records) -> bool:
    """Exhaustive linearizability check for tiny histories (at most ~8 operations).

    Tries every total order consistent with real time and replays it against the
    FIFO model of correctness/lincheck/main.go:93-121.  Independent of the C++
    search, used to cross-check it on random small histories.
    """
    ops = [dict(proc=int(r["proc"]), op=int(r["op"]), arg=int(r["arg"]), ret=int(r["ret"]),
                call=int(r["call"]), end=int(r["end"])) for r in records]
    n = len(ops)
    for perm in itertools.permutations(range(n)):
        pos = {k: i for i, k in enumerate(perm)}
        # real-time: a.end < b.call  =>  a before b
        if any(ops[a]["end"] < ops[b]["call"] and pos[a] > pos[b] for a in range(n) for b in range(n)):
            continue
        q = []
        ok = True
        for k in perm:
            o = ops[k]
            if o["op"] == 2:
                pass
            elif o["op"] == 0:
                if o["ret"] != 0:
                    q.append(o["arg"])
            elif not q:
                ok = o["ret"] == 0
            elif o["ret"] == 0 or o["ret"] != q[0]:
                ok = False
            else:
                q.pop(0)
            if not ok:
                break
        if ok:
            return True
    return False


# ------------------------------------------------------------------ CPU queues
def cpu_history(kind: str, threads: int, ops: int, mode: int = 0, producer_percent: int = 50,
                order: int = 15, value_mode: int = 0) -> np.ndarray:
    cap = threads * ops * 2
    out = np.zeros(cap, dtype=HIST_DTYPE)
    n = lib().oracle_history(KINDS[kind], order, threads, ops, mode, producer_percent, value_mode,
                             out.ctypes.data, cap)
    if n < 0:
        raise RuntimeError("oracle_history failed: %d" % n)
    return out[:n]


def cpu_throughput(kind: str, threads: int, mode: int = 0, producer_percent: int = 50,
                   order: int = 15, warmup_ms: float = 50.0, run_ms: float = 200.0) -> dict:
    st = TbStats()
    rc = lib().oracle_tb_run(KINDS[kind], order, threads, mode, producer_percent, warmup_ms,
                             run_ms, C.byref(st))
    if rc != 0:
        raise RuntimeError("oracle_tb_run failed: %d" % rc)
    d = {f: getattr(st, f) for f, _ in TbStats._fields_ if not f.startswith("_")}
    d["succ_mops"] = (st.enq_success + st.deq_success) / (st.elapsed_ms * 1e3)
    return d


def cpu_fifo_check(kind: str, threads: int, ops_per_thread: int, order: int = 15) -> dict:
    c = np.zeros(5, dtype=np.uint64)
    rc = lib().oracle_fifo_check(KINDS[kind], order, threads, ops_per_thread, c.ctypes.data)
    keys = ["in", "out", "dup", "order", "missing"]
    d = {k: int(v) for k, v in zip(keys, c)}
    d["verified"] = rc == 0
    return d
