"""gcq_gb300: gCQ's GPU concurrent FIFO queues (G-WFQ, G-LFQ, WFQ-YMC, SFQ) on GB300.

The product is the CUDA code in include/gcq/*.cuh and gcq_gb300/csrc/*.cu, built
for sm_103a into gcq_gb300/_build/libgcq.so with the C ABI of include/gcq.h.  This
module is a thin ctypes binding to that library for Python callers, the tests and
bench.py.  There is no CPU fallback: if libgcq.so is missing, or no CUDA device is
present, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# GCQ_LIBRARY_PATH selects another build of the same library (e.g. a tuning variant)
LIB_PATH = os.environ.get("GCQ_LIBRARY_PATH") or os.path.join(HERE, "_build", "libgcq.so")

KINDS = {"gwfq": 0, "glfq": 1, "wfq": 2, "sfq": 3}
KIND_NAMES = {v: k for k, v in KINDS.items()}

# gcq_status
OK, EINVAL, ENOMEM, ECUDA, ETIMEDOUT, EDEVICE, EUNSUPPORTED, ECAPACITY = 0, -1, -2, -3, -4, -5, -6, -7
ERR_SPIN, ERR_TIMEOUT, ERR_TID, ERR_POOL, ERR_CAPACITY = 0x1, 0x2, 0x4, 0x8, 0x10

# gcq_log_entry (include/gcq.h)
LOG_DTYPE = np.dtype([("proc", "<u8"), ("op", "<u4"), ("_pad", "<u4"), ("arg", "<u8"),
                      ("ret", "<u8"), ("call", "<i8"), ("end", "<i8")])


class Knobs(C.Structure):
    _fields_ = [("help_delay", C.c_uint32), ("enq_patience", C.c_uint32), ("deq_patience", C.c_uint32),
                ("remap", C.c_uint32), ("ymc_patience", C.c_uint32), ("ymc_ops_per_thread", C.c_uint32),
                ("wait_timeout_ns", C.c_uint64), ("deq_wait", C.c_uint32), ("_pad", C.c_uint32)]


class TbCounters(C.Structure):
    _fields_ = [("enq_success", C.c_uint64), ("enq_fail", C.c_uint64),
                ("deq_success", C.c_uint64), ("deq_empty", C.c_uint64)]


class TbResult(C.Structure):
    _fields_ = [("counters", TbCounters), ("gpu_ms", C.c_double), ("launches", C.c_uint64)]


class FifoResult(C.Structure):
    _fields_ = [("in_count", C.c_uint64), ("out_count", C.c_uint64), ("err_oob", C.c_uint32),
                ("err_dup", C.c_uint32), ("err_order", C.c_uint32), ("err_missing", C.c_uint32),
                ("err_gt1", C.c_uint32), ("ops_per_thread", C.c_uint32), ("verified", C.c_int),
                ("_pad", C.c_int)]


class Roofline(C.Structure):
    _fields_ = [("r1_single", C.c_double), ("r1_warp", C.c_double), ("rs_lines", C.c_double),
                ("rs_contig", C.c_double), ("rc_lines", C.c_double), ("rc128_lines", C.c_double),
                ("hbm_gbs", C.c_double), ("sms", C.c_int), ("_pad", C.c_int), ("fp32_gops", C.c_double)]


class BfsResult(C.Structure):
    _fields_ = [("total_ms", C.c_double), ("kernel_ms", C.c_double), ("init_ms", C.c_double),
                ("edges_scanned", C.c_uint64), ("reached", C.c_uint32), ("levels", C.c_int32),
                ("max_frontier", C.c_uint32), ("drops", C.c_uint32)]


class RtResult(C.Structure):
    _fields_ = [("gen_ms", C.c_double), ("trace_ms", C.c_double), ("total_ms", C.c_double),
                ("primary_rays", C.c_uint64), ("total_rays", C.c_uint64), ("leftover", C.c_uint64)]


class ServeCfg(C.Structure):
    _fields_ = [("budget_bytes", C.c_uint64), ("timeout_ns", C.c_uint64), ("max_slots", C.c_uint32),
                ("threads", C.c_uint32), ("work_log2", C.c_uint32), ("_pad", C.c_uint32),
                ("run_limit_ns", C.c_uint64), ("work_knobs", Knobs),
                ("rt_scenes", C.c_uint32), ("rt_width", C.c_uint32), ("rt_height", C.c_uint32),
                ("rt_tile_px", C.c_uint32), ("rt_max_bounces", C.c_uint32), ("rt_slots", C.c_uint32),
                ("rt_seed", C.c_uint64)]


class ServeStats(C.Structure):
    _fields_ = [("kernel_ms", C.c_double), ("items", C.c_uint64), ("stale", C.c_uint64),
                ("edges", C.c_uint64), ("sweeps", C.c_uint64), ("completed", C.c_uint32),
                ("error_word", C.c_uint32), ("released", C.c_uint32), ("inflight", C.c_uint32),
                ("reserved", C.c_uint64), ("work_tail", C.c_uint64 * 2), ("work_head", C.c_uint64 * 2),
                ("work_threshold", C.c_int32 * 2), ("rays", C.c_uint64)]


# gcq_serve_req / gcq_serve_res (include/gcq.h)
SERVE_REQ_DTYPE = np.dtype([("graph", "<i4"), ("src", "<i4"), ("arrival_ns", "<u8")])
SERVE_RES_DTYPE = np.dtype([("admit_ns", "<u8"), ("done_ns", "<u8"), ("finish_ns", "<u8"),
                            ("checksum", "<u8"), ("reached", "<u4"), ("max_level", "<i4")])


class TunePoint(C.Structure):
    _fields_ = [("block", C.c_uint32), ("chunk_ops", C.c_uint32), ("deq_wait", C.c_uint32), ("remap", C.c_uint32),
                ("succ_mops", C.c_double), ("status", C.c_int32), ("_pad", C.c_int32)]


class GcqError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        msg = "%s: %s" % (what, _lib().gcq_strerror(status).decode()) if _LIB else str(status)
        if status == ECUDA and _LIB:
            msg += " (%s)" % _lib().gcq_last_cuda_error().decode()
        super().__init__(msg)


# Exported symbols with (argtypes, restype); the CPU tests check that each one is
# present in libgcq.so and declared in include/gcq.h.
P, U32, U64, I32, SZ = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int, C.c_size_t
SIGNATURES = {
    "gcq_default_knobs": ([C.POINTER(Knobs)], None),
    "gcq_create": ([I32, U32, U32, C.POINTER(Knobs), C.POINTER(P)], I32),
    "gcq_destroy": ([P], I32),
    "gcq_reset": ([P, P], I32),
    "gcq_device_ptr": ([P, C.POINTER(P)], I32),
    "gcq_error_word": ([P, C.POINTER(U32), I32], I32),
    "gcq_device_bytes": ([P], U64),
    "gcq_info": ([P, C.POINTER(I32), C.POINTER(U32), C.POINTER(U32)], I32),
    "gcq_device_info": ([C.c_char_p, I32, C.POINTER(I32)], I32),
    "gcq_strerror": ([I32], C.c_char_p),
    "gcq_last_cuda_error": ([], C.c_char_p),
    "gcq_run_history": ([P, U32, U32, U32, I32, I32, I32, P, SZ, C.POINTER(SZ), P], I32),
    "gcq_tb_launch": ([P, I32, I32, U32, U32, U32, U64, P, P], I32),
    "gcq_tb_chunk_host": ([P, I32, I32, U32, U32, U32, P, C.POINTER(TbCounters), P], I32),
    "gcq_tb_run": ([P, I32, I32, U32, U32, U32, C.c_double, C.c_double, U32, C.POINTER(TbResult)], I32),
    "gcq_tb_run_bounded": ([P, I32, I32, U32, U32, U32, C.c_double, C.c_double, U32, C.POINTER(TbResult)], I32),
    "gcq_fifo_check": ([P, U32, U32, U32, C.POINTER(FifoResult)], I32),
    "gcq_fifo_check_split": ([P, U32, U32, I32, U32, C.POINTER(FifoResult)], I32),
    "gcq_drain_host": ([P, U32, U32, P, SZ, C.POINTER(SZ)], I32),
    "gcq_roofline_measure": ([C.POINTER(Roofline), I32], I32),
    "gcq_stats": ([P, C.POINTER(C.c_uint64), I32], I32),
    "gcq_tb_chunk_host_noalloc": ([P, I32, I32, U32, U32, U32, P, C.POINTER(TbCounters), P], I32),
    "gcq_graph_grid": ([U32, U32, C.c_double, C.c_double, U64, C.POINTER(P), C.POINTER(P),
                        C.POINTER(C.c_int32), C.POINTER(C.c_int64)], I32),
    "gcq_free": ([P], None),
    "gcq_graph_rmat": ([U32, U32, C.c_double, C.c_double, C.c_double, U64, C.POINTER(P), C.POINTER(P),
                        C.POINTER(C.c_int32), C.POINTER(C.c_int64)], I32),
    "gcq_graph_load_mtx": ([C.c_char_p, C.POINTER(P), C.POINTER(P), C.POINTER(C.c_int32), C.POINTER(C.c_int64)], I32),
    "gcq_graph_load_snap": ([C.c_char_p, C.POINTER(P), C.POINTER(P), C.POINTER(C.c_int32), C.POINTER(C.c_int64)], I32),
    "gcq_bfs_create": ([I32, P, P, C.c_int32, C.c_int64, U32, U32, C.POINTER(Knobs), C.POINTER(P)], I32),
    "gcq_bfs_destroy": ([P], I32),
    "gcq_bfs_run": ([P, C.c_int32, U32, I32, P, C.POINTER(BfsResult)], I32),
    "gcq_rt_render": ([I32, I32, I32, I32, I32, I32, I32, I32, U32, P, C.POINTER(RtResult)], I32),
    "gcq_rt_compact_render": ([I32, I32, I32, I32, P, C.POINTER(RtResult)], I32),
    "gcq_rt_bounce_render": ([I32, I32, I32, I32, I32, I32, I32, U32, U64, P, C.POINTER(RtResult)], I32),
    "gcq_rt_ctx_create": ([I32, I32, I32, I32, I32, I32, I32, U32, U64, I32, C.POINTER(P)], I32),
    "gcq_rt_ctx_render": ([P, P, I32, P, C.POINTER(RtResult)], I32),
    "gcq_rt_ctx_destroy": ([P], I32),
    "gcq_serve_image": ([P, I32, P], I32),
    "gcq_tb_autotune": ([I32, U32, U32, I32, I32, C.c_double, U32, C.POINTER(TunePoint), C.POINTER(TunePoint), SZ,
                         C.POINTER(SZ)], I32),
    "gcq_serve_default_cfg": ([C.POINTER(ServeCfg)], None),
    "gcq_serve_create": ([I32, P, P, P, P, C.POINTER(ServeCfg), C.POINTER(P)], I32),
    "gcq_serve_destroy": ([P], I32),
    "gcq_serve_info": ([P, I32, C.POINTER(U32), C.POINTER(U32), C.POINTER(U64)], I32),
    "gcq_serve_run": ([P, P, U32, P, C.POINTER(ServeStats)], I32),
}

_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("libgcq.so is not built (%s); run __graft_entry__.build() or "
                               "python -m gcq_gb300.build" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (args, res) in SIGNATURES.items():
            f = getattr(L, name, None)
            if f is None:
                continue
            f.argtypes = args
            f.restype = res
        _LIB = L
    return _LIB


def lib():
    """The loaded libgcq.so (ctypes.CDLL)."""
    return _lib()


def _check(rc, what):
    if rc != OK:
        raise GcqError(rc, what)


def default_knobs() -> Knobs:
    k = Knobs()
    _lib().gcq_default_knobs(C.byref(k))
    return k


class Queue:
    """One device queue owned by libgcq.so (gcq_create / gcq_destroy)."""

    def __init__(self, kind: str, capacity_log2: int, max_threads: int, knobs: Knobs | None = None,
                 **overrides):
        if kind not in KINDS:
            raise ValueError("kind must be one of %s" % sorted(KINDS))
        k = knobs or default_knobs()
        for name, v in overrides.items():
            setattr(k, name, v)
        h = P()
        _check(_lib().gcq_create(KINDS[kind], capacity_log2, max_threads, C.byref(k), C.byref(h)),
               "gcq_create(%s, 2^%d, %d)" % (kind, capacity_log2, max_threads))
        self._h = h
        self.kind = kind
        self.capacity_log2 = capacity_log2
        self.max_threads = max_threads

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            _lib().gcq_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset(self, stream: int = 0):
        _check(_lib().gcq_reset(self._h, P(stream)), "gcq_reset")

    def device_ptr(self) -> int:
        d = P()
        _check(_lib().gcq_device_ptr(self._h, C.byref(d)), "gcq_device_ptr")
        return d.value

    def device_bytes(self) -> int:
        return int(_lib().gcq_device_bytes(self._h))

    def error_word(self, clear: bool = False) -> int:
        e = U32()
        _check(_lib().gcq_error_word(self._h, C.byref(e), int(clear)), "gcq_error_word")
        return e.value

    STAT_NAMES = ["try_enq", "try_deq", "deq_retry", "enq_slow", "deq_slow", "finalize",
                  "finalize_scan", "deq_waited"]

    def stats(self, clear: bool = False) -> dict:
        """G-WFQ operation counters per ring (non-zero only in GCQ_STATS builds)."""
        a = (C.c_uint64 * 16)()
        _check(_lib().gcq_stats(self._h, a, int(clear)), "gcq_stats")
        return {ring: dict(zip(self.STAT_NAMES, list(a)[i * 8:(i + 1) * 8])) for i, ring in enumerate(["aq", "fq"])}

    # --- history harness -------------------------------------------------------
    def history(self, threads: int, ops: int, block: int = 256, mode: int = 0, producer_percent: int = 50,
                value_mode: int = 0, stream: int = 0) -> np.ndarray:
        cap = threads * ops * 2
        out = np.zeros(cap, dtype=LOG_DTYPE)
        n = SZ()
        _check(_lib().gcq_run_history(self._h, threads, block, ops, mode, producer_percent, value_mode,
                                      out.ctypes.data, cap, C.byref(n), P(stream)), "gcq_run_history")
        return out[: n.value].copy()

    # --- throughput harness ----------------------------------------------------
    def tb_launch(self, mode: int, threads: int, chunk_ops: int, dev_counters: int, block: int = 256,
                  producer_percent: int = 50, seed: int = 0, stream: int = 0):
        _check(_lib().gcq_tb_launch(self._h, mode, producer_percent, threads, block, chunk_ops, seed,
                                    P(dev_counters), P(stream)), "gcq_tb_launch")

    def tb_chunk_host(self, mode: int, threads: int, chunk_ops: int, payloads: np.ndarray, block: int = 256,
                      producer_percent: int = 50, stream: int = 0) -> dict:
        assert payloads.dtype == np.uint32 and payloads.size == threads * chunk_ops
        c = TbCounters()
        _check(_lib().gcq_tb_chunk_host(self._h, mode, producer_percent, threads, block, chunk_ops,
                                        payloads.ctypes.data, C.byref(c), P(stream)), "gcq_tb_chunk_host")
        return {f: getattr(c, f) for f, _ in TbCounters._fields_}

    def tb_chunk_host_noalloc(self, mode: int, threads: int, chunk_ops: int, payloads: np.ndarray,
                              block: int = 256, producer_percent: int = 50, stream: int = 0) -> dict:
        """gcq_tb_chunk_host without device allocation (fixed staging in libgcq.so)."""
        assert payloads.dtype == np.uint32 and payloads.size == threads * chunk_ops
        c = TbCounters()
        _check(_lib().gcq_tb_chunk_host_noalloc(self._h, mode, producer_percent, threads, block, chunk_ops,
                                                payloads.ctypes.data, C.byref(c), P(stream)),
               "gcq_tb_chunk_host_noalloc")
        return {f: getattr(c, f) for f, _ in TbCounters._fields_}

    def tb_run(self, mode: int, threads: int, chunk_ops: int = 128, block: int = 256, producer_percent: int = 50,
               warmup_ms: float = 200.0, run_ms: float = 1000.0, graph_chunks: int = 16) -> dict:
        r = TbResult()
        _check(_lib().gcq_tb_run(self._h, mode, producer_percent, threads, block, chunk_ops, warmup_ms, run_ms,
                                 graph_chunks, C.byref(r)), "gcq_tb_run")
        return self._tb_dict(r)

    def tb_run_bounded(self, mode: int, threads: int, chunk_ops: int = 128, block: int = 256,
                       producer_percent: int = 50, warmup_ms: float = 200.0, run_ms: float = 1000.0,
                       reset_every: int = 0) -> dict:
        """gcq_tb_run with a device deadline on every chunk (gcq_tb_run_bounded)."""
        r = TbResult()
        _check(_lib().gcq_tb_run_bounded(self._h, mode, producer_percent, threads, block, chunk_ops, warmup_ms,
                                         run_ms, reset_every, C.byref(r)), "gcq_tb_run_bounded")
        return self._tb_dict(r)

    @staticmethod
    def _tb_dict(r) -> dict:
        c = r.counters
        sec = r.gpu_ms / 1e3
        d = {f: getattr(c, f) for f, _ in TbCounters._fields_}
        d.update(gpu_ms=r.gpu_ms, launches=r.launches,
                 succ_mops=(c.enq_success + c.deq_success) / sec / 1e6 if sec > 0 else 0.0,
                 enq_mops=c.enq_success / sec / 1e6 if sec > 0 else 0.0,
                 deq_mops=c.deq_success / sec / 1e6 if sec > 0 else 0.0,
                 empty_mops=c.deq_empty / sec / 1e6 if sec > 0 else 0.0,
                 fail_mops=c.enq_fail / sec / 1e6 if sec > 0 else 0.0)
        return d

    # --- FIFO check --------------------------------------------------------------
    def fifo_check(self, threads: int, ops_per_thread: int = 32, block: int = 256) -> dict:
        r = FifoResult()
        _check(_lib().gcq_fifo_check(self._h, threads, block, ops_per_thread, C.byref(r)), "gcq_fifo_check")
        return {f: getattr(r, f) for f, _ in FifoResult._fields_ if not f.startswith("_")}

    def fifo_check_split(self, threads: int, producer_percent: int = 50, ops_per_producer: int = 32,
                         block: int = 256) -> dict:
        """Producers and consumers in one launch (gcq_fifo_check_split)."""
        r = FifoResult()
        _check(_lib().gcq_fifo_check_split(self._h, threads, block, producer_percent, ops_per_producer,
                                           C.byref(r)), "gcq_fifo_check_split")
        return {f: getattr(r, f) for f, _ in FifoResult._fields_ if not f.startswith("_")}

    def drain_host(self, threads: int = 1024, cap: int = 1 << 20, block: int = 256) -> np.ndarray:
        """Dequeue everything the queue holds into a host array (gcq_drain_host)."""
        out = np.zeros(cap, dtype=np.uint64)
        n = SZ()
        _check(_lib().gcq_drain_host(self._h, threads, block, out.ctypes.data, cap, C.byref(n)), "gcq_drain_host")
        return out[: n.value].copy()


def autotune(kind: str, capacity_log2: int, threads: int, mode: int = 0, producer_percent: int = 50,
             ms_per_point: float = 60.0, passes: int = 2) -> dict:
    """Autotune block, chunk length and queue knobs of one throughput configuration
    (gcq_tb_autotune); returns {"best": {...}, "table": [...]}."""
    best = TunePoint()
    table = (TunePoint * 256)()
    n = SZ()
    _check(_lib().gcq_tb_autotune(KINDS[kind], capacity_log2, threads, mode, producer_percent, ms_per_point, passes,
                                  C.byref(best), table, 256, C.byref(n)), "gcq_tb_autotune")
    row = lambda p: {f: getattr(p, f) for f, _ in TunePoint._fields_ if not f.startswith("_")}
    return {"best": row(best), "table": [row(table[i]) for i in range(min(n.value, 256))]}


def graph_grid(rows: int, cols: int, keep_p: float = 0.6, diag_p: float = 0.01, seed: int = 1):
    """Seeded grid graph as CSR (offsets, indices) int32 numpy arrays (gcq_graph_grid)."""
    po, pi = P(), P()
    V, E = C.c_int32(), C.c_int64()
    _check(_lib().gcq_graph_grid(rows, cols, keep_p, diag_p, seed, C.byref(po), C.byref(pi),
                                 C.byref(V), C.byref(E)), "gcq_graph_grid")
    off = np.ctypeslib.as_array(C.cast(po, C.POINTER(C.c_int32)), shape=(V.value + 1,)).copy()
    idx = np.ctypeslib.as_array(C.cast(pi, C.POINTER(C.c_int32)), shape=(max(E.value, 1),))[: E.value].copy()
    _lib().gcq_free(po)
    _lib().gcq_free(pi)
    return off, idx


def graph_rmat(scale: int, edge_factor: int = 16, a: float = 0.57, b: float = 0.19, c: float = 0.19,
               seed: int = 1):
    """Seeded R-MAT graph as CSR int32 numpy arrays (gcq_graph_rmat)."""
    po, pi = P(), P()
    V, E = C.c_int32(), C.c_int64()
    _check(_lib().gcq_graph_rmat(scale, edge_factor, a, b, c, seed, C.byref(po), C.byref(pi),
                                 C.byref(V), C.byref(E)), "gcq_graph_rmat")
    off = np.ctypeslib.as_array(C.cast(po, C.POINTER(C.c_int32)), shape=(V.value + 1,)).copy()
    idx = np.ctypeslib.as_array(C.cast(pi, C.POINTER(C.c_int32)), shape=(max(E.value, 1),))[: E.value].copy()
    _lib().gcq_free(po)
    _lib().gcq_free(pi)
    return off, idx


def graph_load(path: str):
    """CSR int32 arrays of a MatrixMarket (.mtx) file or a SNAP edge list (any other
    name), as the BFS harness reads them (gcq_graph_load_mtx / gcq_graph_load_snap)."""
    po, pi = P(), P()
    V, E = C.c_int32(), C.c_int64()
    fn = _lib().gcq_graph_load_mtx if path.endswith(".mtx") else _lib().gcq_graph_load_snap
    _check(fn(path.encode(), C.byref(po), C.byref(pi), C.byref(V), C.byref(E)), "graph_load(%s)" % path)
    off = np.ctypeslib.as_array(C.cast(po, C.POINTER(C.c_int32)), shape=(V.value + 1,)).copy()
    idx = np.ctypeslib.as_array(C.cast(pi, C.POINTER(C.c_int32)), shape=(max(E.value, 1),))[: E.value].copy()
    _lib().gcq_free(po)
    _lib().gcq_free(pi)
    return off, idx


class Bfs:
    """A CSR graph on the device with two frontier queues (gcq_bfs_create)."""

    def __init__(self, kind: str, offsets: np.ndarray, indices: np.ndarray, threads: int = 8192,
                 capacity_log2: int = 0, knobs: Knobs | None = None, **overrides):
        self.off = np.ascontiguousarray(offsets, dtype=np.int32)
        self.idx = np.ascontiguousarray(indices, dtype=np.int32)
        self.V = len(self.off) - 1
        k = knobs or default_knobs()
        for name, v in overrides.items():
            setattr(k, name, v)
        h = P()
        _check(_lib().gcq_bfs_create(KINDS[kind], self.off.ctypes.data, self.idx.ctypes.data, self.V,
                                     len(self.idx), threads, capacity_log2, C.byref(k), C.byref(h)),
               "gcq_bfs_create")
        self._h = h
        self.threads = threads

    def run(self, src: int = 0, block: int = 256, persistent: bool = False, levels: bool = True):
        lv = np.empty(self.V, dtype=np.int32) if levels else None
        r = BfsResult()
        _check(_lib().gcq_bfs_run(self._h, src, block, int(persistent), lv.ctypes.data if levels else None,
                                  C.byref(r)), "gcq_bfs_run")
        return {f: getattr(r, f) for f, _ in BfsResult._fields_}, lv

    def close(self):
        if self._h:
            _lib().gcq_bfs_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Persistent BFS and ray-tile server over resident CSR graphs and scenes
    (gcq_serve_create / gcq_serve_run).

    graphs: a list of (offsets, indices) int32 CSR pairs.  rt_scenes > 0 also serves
    tiles of the benchmark scenes 0 .. rt_scenes-1 as targets len(graphs) + scene.
    run() takes a structured array of SERVE_REQ_DTYPE sorted by arrival_ns and
    returns (SERVE_RES_DTYPE array, stats dict)."""

    def __init__(self, graphs, budget_bytes: int | None = None, max_slots: int = 0, threads: int = 0,
                 work_log2: int = 0, timeout_s: float = 0.0, run_limit_s: float = 0.0, rt_scenes: int = 0,
                 rt_size=(1024, 1024), rt_tile_px: int = 32, rt_max_bounces: int = 4, rt_slots: int = 0,
                 rt_seed: int = 1, **work_knobs):
        self.graphs = [(np.ascontiguousarray(o, dtype=np.int32), np.ascontiguousarray(i, dtype=np.int32))
                       for o, i in graphs]
        n = len(self.graphs)
        offs = (C.c_void_p * max(n, 1))(*[o.ctypes.data for o, _ in self.graphs])
        idxs = (C.c_void_p * max(n, 1))(*[i.ctypes.data for _, i in self.graphs])
        self.V = np.array([len(o) - 1 for o, _ in self.graphs], dtype=np.int32)
        E = np.array([len(i) for _, i in self.graphs], dtype=np.int64)
        cfg = ServeCfg()
        _lib().gcq_serve_default_cfg(C.byref(cfg))
        if budget_bytes is not None:
            cfg.budget_bytes = int(budget_bytes)
        if max_slots:
            cfg.max_slots = max_slots
        if threads:
            cfg.threads = threads
        if work_log2:
            cfg.work_log2 = work_log2
        if timeout_s:
            cfg.timeout_ns = int(timeout_s * 1e9)
        if run_limit_s:
            cfg.run_limit_ns = int(run_limit_s * 1e9)
        for name, v in work_knobs.items():   # knobs of the worklist queue
            setattr(cfg.work_knobs, name, v)
        cfg.rt_scenes = rt_scenes
        cfg.rt_width, cfg.rt_height = rt_size
        cfg.rt_tile_px, cfg.rt_max_bounces, cfg.rt_seed = rt_tile_px, rt_max_bounces, rt_seed
        if rt_slots:
            cfg.rt_slots = rt_slots
        self.rt_size = tuple(rt_size)
        self.rt_tiles = ((rt_size[0] + rt_tile_px - 1) // rt_tile_px) * ((rt_size[1] + rt_tile_px - 1) // rt_tile_px)
        h = P()
        _check(_lib().gcq_serve_create(n, C.cast(offs, P), C.cast(idxs, P), self.V.ctypes.data, E.ctypes.data,
                                       C.byref(cfg), C.byref(h)), "gcq_serve_create")
        self._h = h

    def info(self, graph: int = -1) -> dict:
        slots, threads, lb = U32(), U32(), U64()
        _check(_lib().gcq_serve_info(self._h, graph, C.byref(slots), C.byref(threads), C.byref(lb)),
               "gcq_serve_info")
        return {"slots": slots.value, "threads": threads.value, "level_bytes": lb.value}

    def run(self, reqs: np.ndarray):
        reqs = np.ascontiguousarray(reqs, dtype=SERVE_REQ_DTYPE)
        res = np.zeros(len(reqs), dtype=SERVE_RES_DTYPE)
        st = ServeStats()
        rc = _lib().gcq_serve_run(self._h, reqs.ctypes.data, len(reqs), res.ctypes.data, C.byref(st))
        self.last_stats = {f: (list(getattr(st, f)) if f.startswith("work_") else getattr(st, f))
                           for f, _ in ServeStats._fields_}
        self.last_results = res
        _check(rc, "gcq_serve_run")
        return res, self.last_stats

    def image(self, scene: int) -> np.ndarray:
        """The served scene's image (height x width x 3 float32)."""
        img = np.zeros((self.rt_size[1], self.rt_size[0], 3), dtype=np.float32)
        _check(_lib().gcq_serve_image(self._h, scene, img.ctypes.data), "gcq_serve_image")
        return img

    def close(self):
        if self._h:
            _lib().gcq_serve_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def serve_autotune(graphs, sample_reqs: np.ndarray, candidates=None, **server_kw):
    """Pick the served engine's persistent-thread count and worklist size by timing
    a sample of requests on each candidate (the reference has no server; its BFS
    harness takes the thread count from the command line).  Returns (best keyword
    arguments for Server, [(candidate, requests per second or None)])."""
    if candidates is None:
        candidates = [dict(threads=t, work_log2=w) for t in (32768, 65536, 0) for w in (28, 29)]
    table = []
    for cand in candidates:
        kw = dict(server_kw)
        kw.update(cand)
        try:
            with Server(graphs, **kw) as srv:
                srv.run(sample_reqs)
                _, st = srv.run(sample_reqs)
            table.append((cand, len(sample_reqs) / (st["kernel_ms"] * 1e-3)))
        except GcqError:
            table.append((cand, None))
    ok = [t for t in table if t[1]]
    if not ok:
        raise GcqError(EINVAL, "serve_autotune: no candidate ran")
    return max(ok, key=lambda t: t[1])[0], table


def serve_requests(n: int, ngraphs: int, V, rate_per_s: float = 0.0, seed: int = 1, weights=None):
    """A seeded request schedule: graph drawn by `weights` (uniform by default), a
    uniform source vertex, Poisson arrivals at `rate_per_s` (0: all at time 0)."""
    rng = np.random.default_rng(seed)
    r = np.zeros(n, dtype=SERVE_REQ_DTYPE)
    p = None if weights is None else np.asarray(weights, dtype=np.float64) / np.sum(weights)
    r["graph"] = rng.choice(ngraphs, size=n, p=p)
    r["src"] = (rng.random(n) * np.asarray(V)[r["graph"]]).astype(np.int64)
    if rate_per_s > 0:
        r["arrival_ns"] = np.cumsum(rng.exponential(1e9 / rate_per_s, size=n)).astype(np.uint64)
    return r


def tile_checksum(img: np.ndarray, tile: int, tile_px: int = 32) -> int:
    """The checksum a served tile reports (gcq_serve_res.checksum), from an image."""
    h, w = img.shape[:2]
    tx = (w + tile_px - 1) // tile_px
    x0, y0 = (tile % tx) * tile_px, (tile // tx) * tile_px
    ys, xs = np.mgrid[y0:min(y0 + tile_px, h), x0:min(x0 + tile_px, w)]
    g = (ys * w + xs).reshape(-1).astype(np.uint64)
    bits = img[y0:y0 + tile_px, x0:x0 + tile_px].reshape(-1, 3).view(np.uint32).astype(np.uint64)
    key = ((3 * g[:, None] + np.arange(3, dtype=np.uint64)[None, :]) << np.uint64(32)) | bits
    with np.errstate(over="ignore"):
        return int(splitmix64(key.reshape(-1)).sum(dtype=np.uint64))


def splitmix64(x: np.ndarray) -> np.ndarray:
    """splitmix64 finaliser over a uint64 array (as the library's checksums use it)."""
    x = np.asarray(x, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = x + np.uint64(0x9E3779B97F4A7C15)
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return x ^ (x >> np.uint64(31))


def rt_render(kind: str = "gwfq", scene: int = 0, width: int = 1280, height: int = 720, tiles_x: int = 8,
              tiles_y: int = 8, threads_per_tile: int = 1024, max_bounces: int = 4, queue_log2: int = 15):
    """Render one frame with the persistent per-tile ray tracer; returns (result, image HxWx3)."""
    img = np.zeros((height, width, 3), dtype=np.float32)
    r = RtResult()
    _check(_lib().gcq_rt_render(KINDS[kind], scene, width, height, tiles_x, tiles_y, threads_per_tile,
                                max_bounces, queue_log2, img.ctypes.data, C.byref(r)), "gcq_rt_render")
    return {f: getattr(r, f) for f, _ in RtResult._fields_}, img


def rt_bounce_render(kind: str = "gwfq", scene: int = 0, width: int = 1024, height: int = 1024, tile_px: int = 32,
                     threads_per_tile: int = 1024, max_bounces: int = 4, queue_log2: int = 15, seed: int = 1):
    """Render a benchmark scene (gcq_rt_bounce_render); returns (result, image HxWx3)."""
    img = np.zeros((height, width, 3), dtype=np.float32)
    r = RtResult()
    _check(_lib().gcq_rt_bounce_render(KINDS[kind], scene, width, height, tile_px, threads_per_tile, max_bounces,
                                       queue_log2, seed, img.ctypes.data, C.byref(r)), "gcq_rt_bounce_render")
    return {f: getattr(r, f) for f, _ in RtResult._fields_}, img


class RtTiles:
    """A benchmark-scene render context (gcq_rt_ctx_*): renders lists of tiles."""

    def __init__(self, kind: str = "gwfq", scene: int = 0, width: int = 1024, height: int = 1024, tile_px: int = 32,
                 threads_per_tile: int = 1024, max_bounces: int = 4, queue_log2: int = 15, seed: int = 1,
                 max_tiles: int = 0):
        self.width, self.height = width, height
        self._h = P()
        _check(_lib().gcq_rt_ctx_create(KINDS[kind], scene, width, height, tile_px, threads_per_tile, max_bounces,
                                        queue_log2, seed, max_tiles, C.byref(self._h)), "gcq_rt_ctx_create")

    def render(self, tiles=None, image: bool = False):
        """Render the tiles (sequence of tile indices, None: all); returns (result, image or None)."""
        img = np.zeros((self.height, self.width, 3), dtype=np.float32) if image else None
        r = RtResult()
        if tiles is None:
            lst, n, ptr = None, 0, None
        else:
            lst = np.ascontiguousarray(tiles, dtype=np.int32)
            n, ptr = len(lst), lst.ctypes.data
        _check(_lib().gcq_rt_ctx_render(self._h, ptr, n, img.ctypes.data if image else None, C.byref(r)),
               "gcq_rt_ctx_render")
        return {f: getattr(r, f) for f, _ in RtResult._fields_}, img

    def close(self):
        if self._h:
            _lib().gcq_rt_ctx_destroy(self._h)
            self._h = P()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rt_compact_render(scene: int = 0, width: int = 1280, height: int = 720, max_bounces: int = 4):
    """Render one frame with the stream-compaction baseline; returns (result, image HxWx3)."""
    img = np.zeros((height, width, 3), dtype=np.float32)
    r = RtResult()
    _check(_lib().gcq_rt_compact_render(scene, width, height, max_bounces, img.ctypes.data, C.byref(r)),
           "gcq_rt_compact_render")
    return {f: getattr(r, f) for f, _ in RtResult._fields_}, img


def roofline(reps: int = 3) -> dict:
    """Measure the atomic roofline of the current GPU (gcq_roofline_measure)."""
    r = Roofline()
    _check(_lib().gcq_roofline_measure(C.byref(r), reps), "gcq_roofline_measure")
    return {f: getattr(r, f) for f, _ in Roofline._fields_ if not f.startswith("_")}


def history_to_jsonl(recs: np.ndarray, path: str, reference_format: bool = False):
    """Write records as the reference's JSONL (correctness/history.cpp:271-280).

    reference_format=True writes a failed-without-effect dequeue (op 2) as the
    reference does, op 1 with ret 0.
    """
    with open(path, "w") as f:
        for r in recs:
            op = int(r["op"])
            if reference_format and op == 2:
                op = 1
            f.write('{"proc":%d,"op":%d,"arg":%d,"ret":%d,"call":%d,"end":%d}\n'
                    % (r["proc"], op, r["arg"], r["ret"], r["call"], r["end"]))
