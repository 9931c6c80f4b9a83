"""Queue throughput benchmark (the reference's throughput harness, balanced mode).

Workload: G-WFQ, balanced mode (every thread enqueues then dequeues,
throughout_bench.cpp:810-840), capacity 2^20, 262144 threads in blocks of 256,
128 operations per thread per chunk, uint32 payloads from a seed.  A step is one
chunk launch over all threads.  Metric: successful queue operations per second
(enq_success + deq_success, throughout_bench.cpp:894), in Mops/s.

  value    device time of K chunk launches (CUDA events on the launching stream),
           L2 flushed between steps by writing a 256 MiB buffer
  e2e      the same chunks through the C-ABI entry point gcq_tb_chunk_host with the
           payloads in pinned host memory: their transfer to the device (the kernel
           reads pinned payloads in place over the host link), the kernel, and the
           counters read back to the host are inside the timed region
  roofline the chunk kernel against the measured L2 atomic throughput of this GPU
           (gcq_roofline_measure, run in the same process)
  cpu_baseline the oracle's std::atomic G-WFQ on all host cores (a reported
           baseline, not the target)

--workload served-bfs measures the served BFS engine instead (gcq_serve_run): a
stream of traversal requests over resident graphs -- R-MAT scales 16..22 (edge
factor 16, a,b,c = 0.57,0.19,0.19) and the two seeded grids (4096^2 and 212^2,
keep 0.6, diagonals 0.01) -- admitted into a 150 GiB level-array budget and served
by one persistent kernel, mixed with ray-tile requests (--serve-tiles, default
2048: every 32x32 tile of both 1024x1024 benchmark scenes) served by the same
kernel.  A step is one run of the whole request set.  Metric: traversals per
second (tiles per second beside it); latency p50/p99 from arrival to response for
each kind.  It also times one launch per request -- a persistent gcq_bfs_run per
traversal, a single-tile gcq_rt_ctx_render per tile -- on a sample of the same
requests, and the oracle's serial BFS and render on the host.

--workload rt renders the two benchmark scenes with the ray-bounce queues: 1024x1024
pixels, 1 sample per pixel, at most 4 bounces, 32x32-pixel tiles with 1024 threads
and a 2^15 G-WFQ ring each, 32-byte rays.  A step is one frame of each scene
(gcq_rt_ctx_render over all tiles); metric: rays traced per second (MRays/s).  The
roofline is the unfused fp32 rate measured in the same run (the renderer is built
without multiply-add contraction); the CPU baseline is the oracle's serial render.

--workload bfs runs the BFS configuration: graphs A and B from vertex 0, the
reference's level-synchronous traversal and the asynchronous one, 512 and 8192
queue threads, 3 warm-up and 10 timed traversals each; depths are checked against
the oracle's serial BFS.  Metric: graph A traversals per second (asynchronous, 8192
threads).

--impl reference runs the reference algorithm on the host cores instead: the
reference is HIP for AMD GPUs and cannot run here, so its arm is the oracle's CPU
restatement of the same G-WFQ (oracle/cpu_queues.cpp), on every host core; with
--workload rt it is the oracle's serial render on every host core, with --workload
bfs the oracle's serial BFS of graph A, with --workload served-bfs the mix's
requests one at a time on one core (sampled per graph and scene).

Multi-GPU (torchrun, --gpus N): replicas only -- a queue is one linearizable object
with global counters, so each rank runs its own queue; value = all ranks' operations
over the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

KIND = "gwfq"
CAPACITY_LOG2 = 20
THREADS = 262144
BLOCK = 256
CHUNK_OPS = 128
# algorithmic L2 atomics per successful operation: each user operation is two ring
# operations (indirection through fq/aq), each one entry RMW (CAS or OR) plus a
# 1/32 share of a warp-aggregated ticket fetch-and-add
ATOMICS_PER_OP = 2.0 + 2.0 / 32.0
METRIC = "queue succ Mops/s (G-WFQ balanced)"


def whole_job(ms, count, device=None):
    """Across the ranks of an initialised process group: the slowest rank's time and
    the sum of all ranks' work (the whole-job value is sum / max).  With one rank,
    or no process group, the inputs come back unchanged."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(ms), float(count)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    c = torch.tensor([float(count)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return t.item(), c.item()


def _env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def profile_values(name):
    """`key: value` lines of a committed ncu summary under profiles/ (the counters
    an ncu capture of the kernel gave; bench.py cannot run ncu itself).  {} when
    the file is absent."""
    out = {}
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return out
    for line in open(path):
        line = line.strip().lstrip("-* ")
        if line.startswith("`") and "`:" in line:
            k, v = line[1:].split("`:", 1)
            try:
                out[k.strip()] = float(v.strip().split()[0].replace(",", ""))
            except ValueError:
                pass
    return out


TB_PROFILE = "gwfq_tb_chunk_262144t_traffic.md"


def cpu_baseline(seconds=3.0, order=CAPACITY_LOG2):
    """The oracle's G-WFQ (std::atomic, the reference algorithm) on all host cores."""
    from oracle import lib as olib
    cores = os.cpu_count() or 1
    r = olib.cpu_throughput("gwfq", cores, mode=0, order=order, warmup_ms=200, run_ms=seconds * 1000)
    return {"value": round(r["succ_mops"], 3), "unit": "Mops/s", "cores": cores, "kind": "port",
            "sample": "balanced G-WFQ (oracle/cpu_queues.cpp), %d host threads, capacity 2^%d, %.1f s timed"
                      % (cores, order, seconds)}


def per_queue(g):
    """Every queue of the sweep, balanced and split 50 %, at its largest thread count
    within its envelope (gcq_tb_run, CUDA-graph chunks of 128 ops, 300 ms).  YMC never
    reclaims its cell pool (wfqueue_hip_opt.hpp:208-237), so a run of many chunks
    exhausts it and then counts only failures; its rows come from chunks with the
    pool reset before each one, outside the timed launches (gcq_tb_run_bounded), as
    in the sweep and as the BFS resets it per level."""
    out = {}
    for kind, cap, threads in [("gwfq", 20, 262144), ("glfq", 20, 262144), ("sfq", 16, 32768), ("wfq", 0, 65536)]:
        row = {"threads": threads, "capacity_log2": cap}
        for mode, name in [(0, "balanced"), (1, "split50")]:
            t = threads if mode == 0 else min(threads, 65536)
            with g.Queue(kind, cap, t) as q:
                if kind == "wfq":
                    r = q.tb_run_bounded(mode, t, chunk_ops=128, producer_percent=50, warmup_ms=100, run_ms=300,
                                         reset_every=1)
                else:
                    r = q.tb_run(mode=mode, producer_percent=50, threads=t, chunk_ops=128, warmup_ms=100,
                                 run_ms=300, graph_chunks=8)
            row[name + "_mops"] = round(r["succ_mops"], 1)
            if mode == 1:
                row["split_threads"] = t
        if kind == "wfq":
            row["pool"] = "reset before every chunk, outside the timed launches"
        out[kind] = row
    return out


def _reference_line(args, metric, value, unit, config, sample, cores, dtype, steps, extra=None):
    line = {"impl": "reference", "metric": metric, "value": round(value, 3), "unit": unit,
            "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic", "config": config,
            "cpu_baseline": {"value": round(value, 3), "unit": unit, "cores": cores, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 3), "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    line.update(extra or {})
    print(json.dumps(line), flush=True)
    return 0


def run_reference_rt(args, olib, cores):
    """The serial render of the benchmark scenes on every host core (the reference's
    RT harness has no CPU path; its algorithm for these scenes is the oracle's)."""
    import numpy as np
    steps = max(1, min(args.steps, 3))
    img = np.zeros((RT_SIZE, RT_SIZE, 3), np.float32)
    olib.lib().oracle_rt_bounce_render(1, 256, 256, RT_BOUNCES, RT_SEED, cores, img.ctypes.data)   # warm-up
    rays, t0 = 0, time.perf_counter()
    for _ in range(steps):
        for sc in (0, 1):
            rays += olib.lib().oracle_rt_bounce_render(sc, RT_SIZE, RT_SIZE, RT_BOUNCES, RT_SEED, cores,
                                                       img.ctypes.data)
    sec = time.perf_counter() - t0
    return _reference_line(args, RT_METRIC, rays / sec / 1e6, "MRays/s",
                           {"workload": "serial render (oracle/rt_cpu.cpp) of both benchmark scenes, %dx%d, "
                                        "1 spp, %d bounces, rows split over %d host threads" % (RT_SIZE, RT_SIZE,
                                                                                             RT_BOUNCES, cores)},
                           "%d frame(s) of each scene, %d threads" % (steps, cores), cores, "f32", steps,
                           {"ms_per_step": round(sec * 1e3 / steps, 3)})


def run_reference_bfs(args, olib, cores):
    """The serial BFS of graph A from vertex 0 (one core)."""
    import gcq_gb300 as g   # host-side graph generator only
    off, idx = g.graph_grid(4096, 4096, 0.6, 0.01, 2)
    steps = max(1, min(args.steps, 3))
    olib.bfs(off, idx, 0)
    t0 = time.perf_counter()
    for _ in range(steps):
        olib.bfs(off, idx, 0)
    sec = (time.perf_counter() - t0) / steps
    return _reference_line(args, BFS_METRIC, 1.0 / sec, "traversals/s",
                           {"workload": "serial BFS (oracle/bfs_serial.cpp) of graph A from vertex 0"},
                           "%d traversal(s) of graph A, 1 thread" % steps, 1, "int32", steps,
                           {"ms_per_step": round(sec * 1e3, 3)})


def run_reference_served(args, olib, cores):
    """The served mix's requests run one at a time on the host: the oracle's serial
    BFS from one source per graph and a 256x256 serial render per scene scaled to a
    tile, summed over the same request mix as the GPU arm."""
    import numpy as np
    import gcq_gb300 as g   # host-side graph generators only
    scales = [int(x) for x in args.serve_scales.split(",") if x]
    graphs, names = _serve_graphs(g, scales)
    ng = len(graphs)
    V = [len(o) - 1 for o, _ in graphs]
    bfs = g.serve_requests(args.serve_requests, ng, V, rate_per_s=0, seed=7)
    per_graph = {}
    for gi, (o, i) in enumerate(graphs):
        srcs = bfs["src"][bfs["graph"] == gi][:1]
        if len(srcs):
            t0 = time.perf_counter()
            olib.bfs(o, i, int(srcs[0]))
            per_graph[gi] = time.perf_counter() - t0
    per_tile = {}
    for sc in (0, 1):
        tmp = np.zeros((256, 256, 3), np.float32)
        t0 = time.perf_counter()
        olib.lib().oracle_rt_bounce_render(sc, 256, 256, RT_BOUNCES, RT_SEED, 1, tmp.ctypes.data)
        per_tile[sc] = (time.perf_counter() - t0) * (RT_TILE * RT_TILE) / (256 * 256)
    n_tiles = args.serve_tiles
    total = sum(per_graph[int(gg)] for gg in bfs["graph"]) + sum(per_tile[k % 2] for k in range(n_tiles))
    rate = (args.serve_requests + n_tiles) / total
    return _reference_line(args, SERVE_METRIC, args.serve_requests / total, "traversals/s",
                           {"workload": "the served mix (%s + %d tiles) one request at a time on one host core"
                                        % ("+".join(names), n_tiles)},
                           "oracle serial BFS, one request per graph, and a 256x256 serial render per scene "
                           "scaled to a tile, summed over the mix", 1, "int32", 1,
                           {"requests_per_s": round(rate, 3)})


def run_reference(args):
    rank, world, _ = _env_rank()
    if rank != 0:
        return 0
    from oracle import build as obuild, lib as olib
    obuild.build()
    if args.workload == "rt":
        return run_reference_rt(args, olib, os.cpu_count() or 1)
    if args.workload == "bfs":
        return run_reference_bfs(args, olib, os.cpu_count() or 1)
    if args.workload == "served-bfs":
        return run_reference_served(args, olib, os.cpu_count() or 1)
    cores = os.cpu_count() or 1
    step_ms = 400.0
    for _ in range(args.warmup):
        olib.cpu_throughput("gwfq", cores, mode=0, order=CAPACITY_LOG2, warmup_ms=50, run_ms=step_ms)
    ops = 0
    ms = 0.0
    for _ in range(args.steps):
        r = olib.cpu_throughput("gwfq", cores, mode=0, order=CAPACITY_LOG2, warmup_ms=50, run_ms=step_ms)
        ops += r["enq_success"] + r["deq_success"]
        ms += r["elapsed_ms"]
    value = ops / (ms * 1e3)
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mops/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(ms / args.steps, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": {"workload": "gwfq balanced, capacity 2^20, %d host threads (reference algorithm on "
                                   "the host cores; the HIP reference has no NVIDIA/CPU build)" % cores,
                       "threads": cores, "capacity_log2": CAPACITY_LOG2},
            "cpu_baseline": {"value": round(value, 3), "unit": "Mops/s", "cores": cores, "kind": "port",
                             "sample": "%d steps of %.0f ms, balanced G-WFQ, %d host threads"
                                       % (args.steps, step_ms, cores)},
            "e2e": {"value": round(value, 3), "unit": "Mops/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def run_gpu(args):
    import numpy as np
    import torch
    import gcq_gb300 as g

    rank, world, local = _env_rank()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    sptr = stream.cuda_stream

    threads, chunk = args.threads, args.chunk_ops
    q = g.Queue(KIND, args.capacity_log2, threads)
    ctr = torch.zeros(4, dtype=torch.int64, device=dev)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    peaks = g.roofline(reps=3) if rank == 0 else None

    def step(seed):
        q.tb_launch(0, threads, chunk, ctr.data_ptr(), block=BLOCK, seed=seed, stream=sptr)

    for w in range(args.warmup):
        step(1000 + w)
        flush.zero_()
    torch.cuda.synchronize()
    ctr.zero_()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    for i in range(args.steps):
        ev[i][0].record(stream)
        step(i)
        ev[i][1].record(stream)
        flush.zero_()          # outside the event pair: evicts L2 between steps
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clocks = sampler.stop()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    dev_ms = sum(step_ms)
    c = ctr.cpu().tolist()
    succ = c[0] + c[2]
    err = q.error_word()
    if err & ~g.ERR_POOL:
        raise RuntimeError("queue error word 0x%x during the bench" % err)
    # whole-job: every rank's operations over the slowest rank's time
    dev_ms_all, succ_all = whole_job(dev_ms, succ, device=dev)
    value = succ_all / (dev_ms_all * 1e3)

    # ---- end to end through the C ABI with host buffers -----------------------
    rng = np.random.default_rng(12345)
    pin = torch.empty(threads * chunk, dtype=torch.int32).pin_memory()
    pay = pin.numpy().view(np.uint32)
    pay[:] = rng.integers(0, 2**32, size=threads * chunk, dtype=np.uint64).astype(np.uint32)
    for w in range(max(1, args.warmup)):
        q.tb_chunk_host(0, threads, chunk, pay, block=BLOCK, stream=sptr)
    torch.cuda.synchronize()
    e2e_ops, e2e_s = 0, 0.0
    for i in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        cc = q.tb_chunk_host(0, threads, chunk, pay, block=BLOCK, stream=sptr)   # raises on a device error
        e2e_s += time.perf_counter() - t0
        e2e_ops += cc["enq_success"] + cc["deq_success"]
        # balanced, capacity >= threads: every enqueue and every dequeue succeeds
        if not (cc["enq_success"] == cc["deq_success"] == threads * chunk):
            raise RuntimeError("end-to-end chunk %d counted %s, not %d operations each" % (i, cc, threads * chunk))
    err = q.error_word()
    if err & ~g.ERR_POOL:
        raise RuntimeError("queue error word 0x%x after the end-to-end chunks" % err)
    e2e_s, e2e_ops = whole_job(e2e_s, e2e_ops, device=dev)
    e2e = e2e_ops / (e2e_s * 1e6)

    # ---- the timed queue's values: produce-then-drain FIFO check at the same size
    # (the reference's FIFO mode; ops per thread capped to capacity / threads)
    fifo = q.fifo_check(threads=threads, ops_per_thread=32, block=BLOCK)
    if fifo["verified"] != 1:
        raise RuntimeError("FIFO check of the bench queue failed: %s" % fifo)

    if rank == 0:
        per_launch_ms = dev_ms / args.steps
        atom_rate = succ / args.steps * ATOMICS_PER_OP / (per_launch_ms * 1e-3)
        peak_rs = max(peaks["rs_lines"], peaks["rs_contig"])
        roof = {
            "bound": "l2_atomic",
            "achieved": round(atom_rate / 1e9, 3),
            "peak": round(peak_rs / 1e9, 3),
            "unit": "Gatomic/s",
            "frac": round(atom_rate / peak_rs, 4),
            "traffic": None,
            "kernel": "k_tb_chunk<GCQ_GWFQ>",
            "traffic_source": None,
            "peak_source": "measured in this run by gcq_roofline_measure: max of spread 64-bit "
                           "fetch-add on distinct lines (%.1f G/s) and warp-contiguous words (%.1f G/s)"
                           % (peaks["rs_lines"] / 1e9, peaks["rs_contig"] / 1e9),
            # 4 ticket counters (fq.Head, aq.Tail, aq.Head, fq.Tail), each at most the
            # measured single-word ticket rate; a successful operation takes 2 tickets
            "ticket_ceiling_mops": round(4 * peaks["r1_warp"] / 2 / 1e6, 1),
            "single_address_gatomic_s": round(peaks["r1_single"] / 1e9, 3),
            "hbm_measured_gbs": round(peaks["hbm_gbs"], 1),
        }
        mp = os.path.join(ROOT, "MEASURED_PEAKS.json")
        if os.path.exists(mp):
            roof["hbm_peak_gbs_of_measured"] = json.load(open(mp)).get("hbm_gbs")
        # per-launch counters of one ncu capture of this kernel at this size
        pv = profile_values(TB_PROFILE)
        if "dram_bytes_per_launch" in pv:
            roof["traffic"] = int(pv["dram_bytes_per_launch"])
            roof["traffic_source"] = "profiles/%s (dram__bytes_read.sum + dram__bytes_write.sum, one launch)" % TB_PROFILE
        if "l2_atomic_requests_per_launch" in pv:
            roof["l2_atomic_requests_per_launch"] = int(pv["l2_atomic_requests_per_launch"])
            roof["l2_atomic_requests_per_op"] = round(pv["l2_atomic_requests_per_launch"] / (succ / args.steps), 3)
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "Mops/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dev_ms_all / args.steps, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic (uint32 payloads from a seed)",
            "config": {"workload": "gwfq balanced, capacity 2^%d, %d threads, block %d, %d ops/thread/chunk"
                                   % (args.capacity_log2, threads, BLOCK, chunk),
                       "queue": KIND, "mode": "balanced", "capacity_log2": args.capacity_log2,
                       "threads": threads, "block": BLOCK, "chunk_ops": chunk,
                       "l2": "flushed between steps (256 MiB write)",
                       "parallelism": "replicas" if world > 1 else "1 gpu"},
            "e2e": {"value": round(e2e, 3), "unit": "Mops/s",
                    "h2d_bytes_per_step": threads * chunk * 4, "d2h_bytes_per_step": 32},
            "gpu_launches": args.steps,
            "clocks": clocks,
            "roofline": roof,
            "step_ms": {"min": round(min(step_ms), 4), "median": round(statistics.median(step_ms), 4),
                        "max": round(max(step_ms), 4)},
            "counters": {"enq_success": c[0], "enq_fail": c[1], "deq_success": c[2], "deq_empty": c[3]},
            "fifo_verified": fifo["verified"],
            "fifo": {"threads": threads, "capacity_log2": args.capacity_log2,
                     "ops_per_thread": fifo["ops_per_thread"], "in": fifo["in_count"], "out": fifo["out_count"],
                     "check": "produce-then-drain of the timed queue: exactly once, per-producer order"},
        }
        if not args.no_per_queue:
            line["queues"] = per_queue(g)
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(seconds=args.cpu_seconds)
        if not args.tb_only:
            line.update(other_workloads(args, local))
        print(json.dumps(line), flush=True)
    q.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


SWEEP_METRIC = "queue succ Mops/s sweep (4 queues x capacity 2^15/2^20 x balanced/split 50/split 25 x 2^10..2^18 threads)"
SWEEP_MODES = (("balanced", 0, 50), ("split50", 1, 50), ("split25", 1, 25))
FIFO_NAMES = {1: "YES", 0: "NO", -1: "skipped"}


def sweep_points(kinds, caps, threads_list):
    """(kind, capacity_log2, mode name, mode, producer percent, threads) of the sweep.
    YMC has no capacity (its cell pool grows with the thread count), so it is swept
    once, with capacity_log2 None."""
    for kind in kinds:
        for cap in ((None,) if kind == "wfq" else caps):
            for name, mode, pct in SWEEP_MODES:
                for t in threads_list:
                    yield kind, cap, name, mode, pct, t


def run_sweep(args):
    """The throughput sweep: every queue x capacity x mode x thread count, each point
    a bounded fixed-duration run (gcq_tb_run_bounded: 128-op chunks, warm-up, timed
    window, every chunk stopped at a device deadline) followed by the reference's
    FIFO check at 32 ops per producer (capped to capacity / threads; "skipped" when
    that is 0, as throughout_bench.cpp:633-635 reports it)."""
    import gcq_gb300 as g
    rank, world, local = _env_rank()
    if rank != 0:
        return 0   # replicas only: the sweep runs on one GPU
    kinds = args.sweep_queues.split(",")
    threads_list = [1 << k for k in range(args.sweep_min_log2, args.sweep_max_log2 + 1)]
    rows, t0 = [], time.perf_counter()
    sampler = ClockSampler(local)
    sampler.start()
    for kind, cap, name, mode, pct, t in sweep_points(kinds, (15, 20), threads_list):
        row = {"queue": kind, "capacity_log2": cap, "mode": name, "threads": t}
        try:
            q = g.Queue(kind, cap or 0, t)
        except g.GcqError as e:
            row["status"] = "n/a: %s" % e
            rows.append(row)
            continue
        try:
            r = q.tb_run_bounded(mode, t, chunk_ops=128, producer_percent=pct, warmup_ms=args.sweep_warmup_ms,
                                 run_ms=args.sweep_run_ms, reset_every=1 if kind == "wfq" else 0)
            row.update(status="ok", succ_mops=round(r["succ_mops"], 2), enq_mops=round(r["enq_mops"], 2),
                       deq_mops=round(r["deq_mops"], 2), launches=r["launches"], gpu_ms=round(r["gpu_ms"], 1))
            f = q.fifo_check(threads=t, ops_per_thread=32)
            row["fifo"] = FIFO_NAMES[f["verified"]]
            row["fifo_ops"] = f["ops_per_thread"]
        except g.GcqError as e:
            row["status"] = ("n/a: %s" % e) if e.status == g.EUNSUPPORTED else ("error: %s" % e)
        finally:
            q.close()
        rows.append(row)
        print(json.dumps(row), file=sys.stderr, flush=True)
    clocks = sampler.stop()
    bad = [r for r in rows if r.get("fifo") == "NO" or r["status"].startswith("error")]
    if args.sweep_md:
        with open(args.sweep_md, "w") as f:
            f.write(sweep_markdown(rows, args))
    head = [r for r in rows if (r["queue"], r["capacity_log2"], r["mode"], r["threads"]) ==
            ("gwfq", 20, "balanced", threads_list[-1]) and r["status"] == "ok"]
    line = {
        "metric": SWEEP_METRIC, "value": head[0]["succ_mops"] if head else None, "unit": "Mops/s",
        "n_gpus": 1, "steps": len(rows), "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "synthetic (uint32 payloads from a seed)",
        "config": {"workload": "throughput sweep: %s x capacity 2^15, 2^20 (YMC: pool) x balanced, split 50 %%, "
                               "split 25 %% x 2^%d..2^%d threads, block 256, 128 ops per chunk, %.0f ms warm-up, "
                               "%.0f ms timed; FIFO check at 32 ops per producer"
                               % ("/".join(kinds), args.sweep_min_log2, args.sweep_max_log2,
                                  args.sweep_warmup_ms, args.sweep_run_ms),
                   "value": "G-WFQ balanced, capacity 2^20, 2^%d threads" % args.sweep_max_log2},
        "points": len(rows), "measured": sum(1 for r in rows if r["status"] == "ok"),
        "not_applicable": sum(1 for r in rows if r["status"].startswith("n/a")),
        "failures": len(bad), "wall_s": round(time.perf_counter() - t0, 1), "clocks": clocks,
        "gpu_launches": sum(r.get("launches", 0) for r in rows),
        "table": rows,
    }
    print(json.dumps(line), flush=True)
    return 1 if bad else 0


def sweep_markdown(rows, args):
    out = ["| queue | capacity | mode | " + " | ".join("2^%d" % k for k in range(args.sweep_min_log2,
                                                                           args.sweep_max_log2 + 1)) + " |",
           "|---|---|---|" + "---:|" * (args.sweep_max_log2 - args.sweep_min_log2 + 1)]
    keyed = {}
    for r in rows:
        keyed.setdefault((r["queue"], r["capacity_log2"], r["mode"]), {})[r["threads"]] = r
    for (kind, cap, mode), pts in keyed.items():
        cells = []
        for k in range(args.sweep_min_log2, args.sweep_max_log2 + 1):
            r = pts.get(1 << k)
            if r is None:
                cells.append("")
            elif r["status"] != "ok":
                cells.append("n/a" if r["status"].startswith("n/a") else "error")
            else:
                cells.append("%.1f%s" % (r["succ_mops"], "" if r.get("fifo") == "YES" else
                                         (" (fifo skipped)" if r.get("fifo") == "skipped" else " (FIFO NO)")))
        out.append("| %s | %s | %s | %s |" % (kind, "pool" if cap is None else "2^%d" % cap, mode, " | ".join(cells)))
    return "\n".join(out) + "\n"


def other_workloads(args, local):
    """The metric's second half beside the queue throughput: graph A BFS
    traversals/s (asynchronous, 8192 threads; 3 warm-up and 10 timed traversals,
    depths checked against the serial BFS) and the served mix (traversals/s with
    p50/p99, one launch per request on the same mix; 3 warm-up and 3 timed runs, the
    server's configuration fixed at the autotuner's choice).  Each keeps its own
    timing, parity check and CPU baseline."""
    import copy
    keep = ("value", "unit", "ms_per_step", "steps", "warmup", "config", "e2e", "roofline", "parity",
            "cpu_baseline", "clocks", "gpu_launches")
    a = copy.copy(args)
    a.steps, a.warmup = 10, 3
    bfs = bfs_line(a, local, full=False)
    out = {"bfs": {k: bfs[k] for k in keep if k in bfs}}
    out["bfs"]["metric"] = bfs["metric"]
    a = copy.copy(args)
    a.steps, a.warmup = 3, 3
    a.serve_autotune = False
    a.serve_sample = 2
    srv = served_line(a, local)
    sv = {k: srv[k] for k in keep + ("latency_ms", "tiles_per_s", "tiles_per_s_while_served", "poisson",
                                      "one_launch_per_request", "work") if k in srv}
    sv["metric"] = srv["metric"]
    sv["parity"] = "every sampled traversal's checksum, reached count and eccentricity equal the serial BFS; " \
                   "every tile's checksum equals the serial render's"
    ol = srv["one_launch_per_request"]
    sv["served_vs_one_launch_per_request"] = ol["speedup"]
    # traversals/s served against one launch per traversal of plain G-WFQ (the
    # reference's level-synchronous traversal; and this build's asynchronous one)
    if ol.get("traversals_per_s"):
        sv["served_vs_one_launch_traversals"] = round(srv["value"] / ol["traversals_per_s"], 2)
    if ol.get("traversals_per_s_async_launch"):
        sv["served_vs_async_launch_traversals"] = round(srv["value"] / ol["traversals_per_s_async_launch"], 2)
    out["served"] = sv
    return out


SERVE_METRIC = "served BFS traversals/s (RMAT 16..22 + grids A, B, mixed with ray tiles)"
RT_METRIC = "RT MRays/s (ray-bounce queue, 1024x1024, 1 spp, 4 bounces, scenes 0 and 1)"
RT_SIZE, RT_TILE, RT_TPT, RT_BOUNCES, RT_QLOG2, RT_SEED = 1024, 32, 1024, 4, 15, 1


def rt_flops_per_ray(spheres, quads):
    """Algorithmic fp32 operations of one ray: 20 per sphere test, 12 per quad test,
    60 for the shading."""
    return 20 * spheres + 12 * quads + 60


RT_SCENE_PRIMS = {0: (512, 1), 1: (0, 17)}   # spheres, quads of each benchmark scene


def run_rt(args):
    """The benchmark scenes: one frame of each per step."""
    import numpy as np
    import torch
    import gcq_gb300 as g
    from oracle import build as obuild, lib as olib

    rank, world, local = _env_rank()
    if rank != 0:
        return 0   # replicas only: the render runs on one GPU
    torch.cuda.set_device(local)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    peaks = g.roofline(reps=2)
    kind = args.rt_queue
    ctxs = [g.RtTiles(kind, scene=sc, width=RT_SIZE, height=RT_SIZE, tile_px=RT_TILE, threads_per_tile=RT_TPT,
                      max_bounces=RT_BOUNCES, queue_log2=RT_QLOG2, seed=RT_SEED) for sc in (0, 1)]
    for _ in range(args.warmup):
        for c in ctxs:
            c.render()
        flush.zero_()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    rays = [0, 0]
    trace_ms = [0.0, 0.0]
    dev_ms = 0.0
    for _ in range(args.steps):
        for sc, c in enumerate(ctxs):
            r, _ = c.render()
            rays[sc] += r["total_rays"]
            trace_ms[sc] += r["trace_ms"]
            dev_ms += r["total_ms"]
            flush.zero_()          # between frames, outside the timed kernels
    torch.cuda.synchronize()
    clocks = sampler.stop()
    value = sum(rays) / (dev_ms * 1e3)
    # end to end: the tile list in, the whole image out, wall clock
    all_tiles = np.arange((RT_SIZE // RT_TILE) ** 2, dtype=np.int32)
    e2e_s, e2e_rays, images = 0.0, 0, [None, None]
    for _ in range(args.steps):
        for sc, c in enumerate(ctxs):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r, images[sc] = c.render(all_tiles, image=True)
            e2e_s += time.perf_counter() - t0
            e2e_rays += r["total_rays"]
    for c in ctxs:
        c.close()
    # parity of the last frames against the serial render (all host threads)
    obuild.build()
    cores = os.cpu_count() or 1
    want_rays = []
    for sc in (0, 1):
        want = np.zeros((RT_SIZE, RT_SIZE, 3), np.float32)
        want_rays.append(olib.lib().oracle_rt_bounce_render(sc, RT_SIZE, RT_SIZE, RT_BOUNCES, RT_SEED, cores,
                                                            want.ctypes.data))
        d = float(np.abs(images[sc] - want).max())
        if d > 1e-4 or rays[sc] != want_rays[sc] * args.steps:
            raise RuntimeError("scene %d differs from the serial render: max |diff| %g" % (sc, d))
    # CPU baseline: the serial render, one core, on a 256x256 frame of each scene
    t0 = time.perf_counter()
    cpu_rays = 0
    for sc in (0, 1):
        tmp = np.zeros((256, 256, 3), np.float32)
        cpu_rays += olib.lib().oracle_rt_bounce_render(sc, 256, 256, RT_BOUNCES, RT_SEED, 1, tmp.ctypes.data)
    cpu_s = time.perf_counter() - t0
    # roofline of the dominant kernel (scene 0's k_btrace)
    flops0 = rays[0] * rt_flops_per_ray(*RT_SCENE_PRIMS[0])
    achieved = flops0 / (trace_ms[0] * 1e-3) / 1e12
    peak = peaks["fp32_gops"] / 1e3
    line = {
        "metric": RT_METRIC, "value": round(value, 2), "unit": "MRays/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(dev_ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic scenes from a seed (512 random spheres; box room)",
        "config": {"workload": "ray-bounce queues (%s), %dx%d, 1 spp, %d bounces, %dx%d-pixel tiles, %d threads "
                               "and a 2^%d ring per tile, 32-byte rays; step = one frame of scene 0 and of scene 1"
                               % (kind, RT_SIZE, RT_SIZE, RT_BOUNCES, RT_TILE, RT_TILE, RT_TPT, RT_QLOG2),
                   "queue": kind, "rays_per_frame": {"scene0": want_rays[0], "scene1": want_rays[1]},
                   "l2": "flushed between frames (256 MiB write)"},
        "per_scene_ms": {"scene0": round(trace_ms[0] / args.steps, 3), "scene1": round(trace_ms[1] / args.steps, 3)},
        "e2e": {"value": round(e2e_rays / (e2e_s * 1e6), 2), "unit": "MRays/s", "h2d_bytes_per_step": 2 * 4 * len(all_tiles),
                "d2h_bytes_per_step": 2 * RT_SIZE * RT_SIZE * 12},
        "gpu_launches": 4 * args.steps,
        "clocks": clocks,
        "roofline": {"bound": "fp32", "achieved": round(achieved, 3), "peak": round(peak, 3), "unit": "TFLOP/s",
                     "frac": round(achieved / peak, 4), "traffic": None, "kernel": "k_btrace<GCQ_GWFQ> (scene 0)",
                     "flops_per_ray": rt_flops_per_ray(*RT_SCENE_PRIMS[0]),
                     "peak_source": "unfused fp32 multiply+add rate measured in this run (gcq_roofline_measure)"},
        "parity": "images within 1e-4 of the serial render (max |diff| 0 expected), ray counts equal",
        "cpu_baseline": {"value": round(cpu_rays / cpu_s / 1e6, 3), "unit": "MRays/s", "cores": 1, "kind": "port",
                         "sample": "oracle serial render (oracle/rt_cpu.cpp), 256x256 frame of each scene, 1 thread"},
    }
    print(json.dumps(line), flush=True)
    return 0


def _serve_graphs(g, scales):
    graphs, names = [], []
    for sc in scales:
        graphs.append(g.graph_rmat(sc, 16, 0.57, 0.19, 0.19, seed=100 + sc))
        names.append("rmat%d" % sc)
    graphs.append(g.graph_grid(4096, 4096, 0.6, 0.01, 2))
    names.append("gridA_4096")
    graphs.append(g.graph_grid(212, 212, 0.6, 0.01, 2))
    names.append("gridB_212")
    return graphs, names


BFS_METRIC = "BFS traversals/s (graph A: 4096^2 grid, keep 0.6, diagonals 0.01; G-WFQ frontier)"


def run_bfs(args):
    rank, world, local = _env_rank()
    if rank != 0:
        return 0   # replicas only
    print(json.dumps(bfs_line(args, local)), flush=True)
    return 0


def bfs_line(args, local, full=True):
    """BFS with the queue as frontier worklist: graphs A and B from vertex 0, level-
    synchronous (the reference's launch per level) and asynchronous (one persistent
    launch), 512 and 8192 queue threads in blocks of 256, 3 warm-up and 10 timed
    traversals.  full=False times only the headline configuration (graph A,
    asynchronous, 8192 threads)."""
    import numpy as np
    import gcq_gb300 as g
    from oracle import build as obuild, lib as olib

    peaks = g.roofline(reps=2)
    graphs = {"A": g.graph_grid(4096, 4096, 0.6, 0.01, 2), "B": g.graph_grid(212, 212, 0.6, 0.01, 2)}
    if not full:
        graphs = {"A": graphs["A"]}
    warm, iters = max(3, args.warmup), max(args.steps, 10)
    table, depths = {}, {}
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    for name, (off, idx) in graphs.items():
        for mode, persistent in ((("level_sync", 0), ("async", 2)) if full else (("async", 2),)):
            for threads in ((512, 8192) if full else (8192,)):
                with g.Bfs("gwfq", off, idx, threads=threads) as b:
                    for _ in range(warm):
                        b.run(0, persistent=persistent, levels=False)
                    ks, ts = [], []
                    for _ in range(iters):
                        r, lv = b.run(0, persistent=persistent, levels=True)
                        ks.append(r["kernel_ms"])
                        ts.append(r["total_ms"])
                    depths[(name, mode, threads)] = lv
                table[(name, mode, threads)] = {
                    "kernel_ms_median": round(float(np.median(ks)), 3), "total_ms_median": round(float(np.median(ts)), 3),
                    "edges_scanned": int(r["edges_scanned"]), "reached": int(r["reached"]),
                    "gteps": round(r["edges_scanned"] / (float(np.median(ks)) * 1e-3) / 1e9, 3)}
    clocks = sampler.stop()
    obuild.build()
    cpu_s = {}
    for name, (off, idx) in graphs.items():
        t = time.perf_counter()
        want, _ = olib.bfs(off, idx, 0)
        cpu_s[name] = time.perf_counter() - t
        for key, lv in depths.items():
            if key[0] == name and not np.array_equal(lv, want):
                raise RuntimeError("BFS depths differ from the serial BFS: %s" % (key,))
    best = table[("A", "async", 8192)]
    V, E = len(graphs["A"][0]) - 1, len(graphs["A"][1])
    alg_bytes = 4 * (V + 1) + 8 * E + 4 * V + 40 * best["reached"]
    achieved = alg_bytes / (best["kernel_ms_median"] * 1e-3) / 1e9
    line = {
        "metric": BFS_METRIC, "value": round(1e3 / best["kernel_ms_median"], 3), "unit": "traversals/s", "n_gpus": 1,
        "steps": iters, "warmup": warm, "ms_per_step": best["kernel_ms_median"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic seeded grids (graph A 4096x4096, graph B 212x212; keep 0.6, diagonals 0.01, seed 2)",
        "config": {"workload": "BFS from vertex 0 of graph A, G-WFQ frontier, 8192 threads, block 256, asynchronous "
                               "(one persistent launch); %d timed traversals, median" % iters,
                   "graphs": {n: {"V": len(o) - 1, "E": len(i)} for n, (o, i) in graphs.items()},
                   "l2": "inputs larger than L2 (graph A: %.0f MB of CSR)" % ((4 * (V + 1) + 4 * E) / 1e6)},
        "table": {"%s/%s/%d" % k: v for k, v in table.items()},
        "e2e": {"value": round(1e3 / best["total_ms_median"], 3), "unit": "traversals/s",
                "h2d_bytes_per_step": 4, "d2h_bytes_per_step": 4 * V},
        "gpu_launches": iters,
        "clocks": clocks,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": round(peaks["hbm_gbs"], 1), "unit": "GB/s",
                     "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": None, "kernel": "k_bfs_async",
                     "bytes_per_traversal": alg_bytes,
                     "peak_source": "device copy bandwidth measured in this run (gcq_roofline_measure); the "
                                    "traversal is bound by its 8258 dependent levels, not by bytes"},
        "parity": "every timed configuration's depths equal the serial BFS bit for bit",
        "cpu_baseline": {"value": round(1.0 / cpu_s["A"], 3), "unit": "traversals/s", "cores": 1, "kind": "port",
                         "sample": "oracle serial BFS (oracle/bfs_serial.cpp) of graph A from vertex 0, once"},
    }
    return line


def run_served(args):
    rank, world, local = _env_rank()
    if rank != 0:
        return 0   # replicas only; the served bench runs on one GPU
    print(json.dumps(served_line(args, local)), flush=True)
    return 0


def served_line(args, local):
    """Served BFS and ray tiles: one persistent kernel per step over the whole
    request set."""
    import numpy as np
    import gcq_gb300 as g
    from oracle import build as obuild, lib as olib

    scales = [int(x) for x in args.serve_scales.split(",") if x]
    t0 = time.perf_counter()
    graphs, names = _serve_graphs(g, scales)
    gen_s = time.perf_counter() - t0
    ng = len(graphs)
    V = [len(o) - 1 for o, _ in graphs]
    E = [len(i) for _, i in graphs]
    n_bfs, n_tiles = args.serve_requests, args.serve_tiles
    tiles_per_frame = (RT_SIZE // RT_TILE) ** 2
    bfs = g.serve_requests(n_bfs, ng, V, rate_per_s=0, seed=7)
    tiles = np.zeros(n_tiles, dtype=g.SERVE_REQ_DTYPE)
    tiles["graph"] = ng + (np.arange(n_tiles) % 2)                  # both scenes
    tiles["src"] = (np.arange(n_tiles) // 2) % tiles_per_frame
    rng = np.random.default_rng(8)
    reqs = np.concatenate([bfs, tiles])[rng.permutation(n_bfs + n_tiles)]
    if args.serve_rate > 0:
        reqs["arrival_ns"] = np.cumsum(rng.exponential(1e9 / args.serve_rate, size=len(reqs))).astype(np.uint64)
    is_tile = reqs["graph"] >= ng
    peaks = g.roofline(reps=2)
    common = dict(budget_bytes=150 << 30, run_limit_s=60.0, rt_scenes=2 if n_tiles else 0,
                  rt_size=(RT_SIZE, RT_SIZE), rt_tile_px=RT_TILE, rt_max_bounces=RT_BOUNCES, rt_seed=RT_SEED)
    if args.serve_patience == "reference":
        # the worklist's G-WFQ at the reference's patience (gwf_queue.hpp:300-306): an
        # operation that keeps failing on the fast path takes the wait-free slow path
        common.update(enq_patience=128, deq_patience=256)
    tuned, tune_table = dict(threads=args.serve_threads, work_log2=args.serve_work_log2), None
    if args.serve_autotune:
        sample = reqs[: min(len(reqs), 384)].copy()
        sample["arrival_ns"] = 0
        tuned, tune_table = g.serve_autotune(graphs, sample, **common)
    srv = g.Server(graphs, **common, **tuned)
    info = srv.info()
    for _ in range(args.warmup):
        srv.run(reqs)
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    kern_ms, wall_s, lat, items, stale, edges, rays = 0.0, 0.0, [], 0, 0, 0, 0
    for _ in range(args.steps):
        t = time.perf_counter()
        res, st = srv.run(reqs)          # host requests in, host results out
        wall_s += time.perf_counter() - t
        kern_ms += st["kernel_ms"]
        lat.append((res["finish_ns"] - reqs["arrival_ns"]) / 1e6)
        items += st["items"]; stale += st["stale"]; edges += st["edges"]; rays += st["rays"]
    clocks = sampler.stop()
    # an open-loop Poisson stream of the same requests at 70 % of the closed-batch
    # rate, for latency under a load the server keeps up with
    poisson = None
    if args.serve_poisson:
        rate = 0.7 * len(reqs) * args.steps / (kern_ms * 1e-3)
        preqs = reqs.copy()
        prng = np.random.default_rng(9)
        preqs["arrival_ns"] = np.cumsum(prng.exponential(1e9 / rate, size=len(preqs))).astype(np.uint64)
        pres, pst = srv.run(preqs)
        plat = (pres["finish_ns"] - preqs["arrival_ns"]) / 1e6
        span = float(pres["finish_ns"].max()) * 1e-9
        poisson = {"offered_requests_per_s": round(rate, 1), "served_requests_per_s": round(len(preqs) / span, 1),
                   "p50_ms": round(float(np.percentile(plat[~is_tile], 50)), 3),
                   "p99_ms": round(float(np.percentile(plat[~is_tile], 99)), 3),
                   "tiles_p50_ms": round(float(np.percentile(plat[is_tile], 50)), 3) if n_tiles else None,
                   "tiles_p99_ms": round(float(np.percentile(plat[is_tile], 99)), 3) if n_tiles else None}
    # parity of the last step against the oracle: a sample of traversals, every tile
    obuild.build()
    bfs_idx = np.nonzero(~is_tile)[0]
    for i in bfs_idx[:: max(1, len(bfs_idx) // 16)]:
        gi, src = int(reqs[i]["graph"]), int(reqs[i]["src"])
        want = olib.bfs_summary(graphs[gi][0], graphs[gi][1], src)
        got = (int(res[i]["checksum"]), int(res[i]["reached"]), int(res[i]["max_level"]))
        if got != want:
            raise RuntimeError("served traversal %d differs from the oracle: %s vs %s" % (i, got, want))
    cores = os.cpu_count() or 1
    if n_tiles:
        for sc in (0, 1):
            want = np.zeros((RT_SIZE, RT_SIZE, 3), np.float32)
            olib.lib().oracle_rt_bounce_render(sc, RT_SIZE, RT_SIZE, RT_BOUNCES, RT_SEED, cores, want.ctypes.data)
            sums = {}
            for i in np.nonzero(reqs["graph"] == ng + sc)[0]:
                tl = int(reqs[i]["src"])
                if tl not in sums:
                    sums[tl] = g.tile_checksum(want, tl, RT_TILE)
                if int(res[i]["checksum"]) != sums[tl]:
                    raise RuntimeError("served tile %d of scene %d differs from the serial render" % (tl, sc))
    srv.close()
    kern_s = kern_ms * 1e-3
    # tile throughput over the span in which tiles were in the system (first tile
    # arrival to last tile response), the kernel's other time being traversals
    tiles_rate = None
    if n_tiles:
        t_first = float(reqs["arrival_ns"][is_tile].min())
        t_last = float(res["finish_ns"][is_tile].max())
        tiles_rate = n_tiles / max(1e-9, (t_last - t_first) * 1e-9)
    lat = np.concatenate(lat)
    lat_tile = lat.reshape(args.steps, -1)[:, is_tile].reshape(-1)
    lat_bfs = lat.reshape(args.steps, -1)[:, ~is_tile].reshape(-1)
    value = n_bfs * args.steps / kern_s
    # one launch per request, timed on a sample of each target's requests
    # (the reference's traversal shape: one cooperative level-synchronous launch; and
    # beside it this build's asynchronous single launch, the fastest one-launch form)
    per_graph_ms, per_graph_async_ms = {}, {}
    for gi, (o, i) in enumerate(graphs):
        srcs = bfs["src"][bfs["graph"] == gi][: args.serve_sample]
        if len(srcs) == 0:
            continue
        with g.Bfs("gwfq", o, i, threads=8192) as b:
            for mode, dst in ((1, per_graph_ms), (2, per_graph_async_ms)):
                b.run(int(srcs[0]), persistent=mode, levels=False)
                ts = [b.run(int(sv), persistent=mode, levels=False)[0]["total_ms"] for sv in srcs]
                dst[gi] = float(np.mean(ts))
    per_scene_ms = {}
    if n_tiles:
        for sc in (0, 1):
            with g.RtTiles("gwfq", scene=sc, width=RT_SIZE, height=RT_SIZE, tile_px=RT_TILE,
                           threads_per_tile=RT_TPT, max_bounces=RT_BOUNCES, queue_log2=RT_QLOG2, seed=RT_SEED,
                           max_tiles=1) as c:
                c.render([0])
                ts = []
                for tl in range(0, tiles_per_frame, tiles_per_frame // 32):
                    t = time.perf_counter()
                    c.render([tl])
                    ts.append((time.perf_counter() - t) * 1e3)
            per_scene_ms[sc] = float(np.mean(ts))
    single_bfs_ms = sum(per_graph_ms[int(gg)] for gg in bfs["graph"])
    single_async_ms = sum(per_graph_async_ms[int(gg)] for gg in bfs["graph"])
    single_tile_ms = sum(per_scene_ms[int(gg) - ng] for gg in tiles["graph"])
    single_rate = (n_bfs + n_tiles) / ((single_bfs_ms + single_tile_ms) * 1e-3)
    served_rate = (n_bfs + n_tiles) * args.steps / kern_s
    # serial BFS on the host (one core), one request per graph; serial tiles from a
    # 256x256 frame of each scene
    cpu_ms = {}
    for gi, (o, i) in enumerate(graphs):
        srcs = bfs["src"][bfs["graph"] == gi][:1]
        if len(srcs):
            t = time.perf_counter()
            olib.bfs(o, i, int(srcs[0]))
            cpu_ms[gi] = (time.perf_counter() - t) * 1e3
    cpu_tile_ms = {}
    for sc in (0, 1):
        tmp = np.zeros((256, 256, 3), np.float32)
        t = time.perf_counter()
        olib.lib().oracle_rt_bounce_render(sc, 256, 256, RT_BOUNCES, RT_SEED, 1, tmp.ctypes.data)
        cpu_tile_ms[sc] = (time.perf_counter() - t) * 1e3 * (RT_TILE * RT_TILE) / (256 * 256)
    cpu_total = sum(cpu_ms.get(int(gg), 0.0) for gg in bfs["graph"]) + \
        sum(cpu_tile_ms[int(gg) - ng] for gg in tiles["graph"])
    # HBM roofline of the traversals: per traversal, offsets 4(V+1) + adjacency 4E +
    # level probes 4E + level writes 4V + the sweep's read and reset 8V
    alg_bytes = sum(4 * (V[gi] + 1) + 8 * E[gi] + 12 * V[gi] for gi in bfs["graph"].astype(int)) * args.steps
    achieved = alg_bytes / kern_s / 1e9
    pct = lambda a, q: round(float(np.percentile(a, q)), 3) if len(a) else None
    line = {
        "metric": SERVE_METRIC, "value": round(value, 2), "unit": "traversals/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(kern_ms / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic graphs from seeds (R-MAT and grids) and the seeded benchmark scenes; %d traversal and "
                "%d tile requests, %s arrivals" % (n_bfs, n_tiles, "Poisson %.0f/s" % args.serve_rate
                                                   if args.serve_rate else "closed-batch"),
        "config": {"workload": "served BFS + ray tiles: %s + scenes 0,1 (1024x1024, 32x32 tiles, 4 bounces); "
                               "%d requests; 150 GiB budget (%d slots, %.1f GB of level arrays); %d persistent "
                               "threads; worklist 2^%s; worklist patience %s" % (
                                   "+".join(names), len(reqs), info["slots"], info["level_bytes"] / 1e9,
                                   info["threads"], tuned.get("work_log2") or "auto",
                                   "128/256 (the reference's: wait-free slow path reachable)"
                                   if args.serve_patience == "reference" else "2^16 (fast path only)"),
                   "graphs": {nm: {"V": v, "E": e} for nm, v, e in zip(names, V, E)},
                   "l2": "inputs larger than L2 (graphs %.1f GB)" % (sum(4 * (v + 1) + 4 * e for v, e in zip(V, E)) / 1e9)},
        "tiles_per_s": round(n_tiles * args.steps / kern_s, 1),
        "tiles_per_s_while_served": round(tiles_rate, 1) if tiles_rate else None,
        "latency_ms": {"p50": pct(lat_bfs, 50), "p99": pct(lat_bfs, 99),
                       "tiles_p50": pct(lat_tile, 50), "tiles_p99": pct(lat_tile, 99)},
        "poisson": poisson,
        "autotune": {"chosen": tuned, "candidates": [{"config": c, "requests_per_s": None if r is None else round(r, 1)}
                                                    for c, r in tune_table]} if tune_table else None,
        "e2e": {"value": round(n_bfs * args.steps / wall_s, 2), "unit": "traversals/s",
                "h2d_bytes_per_step": len(reqs) * 16, "d2h_bytes_per_step": len(reqs) * 40},
        "one_launch_per_request": {
            "value": round(single_rate, 2), "unit": "requests/s", "served_requests_per_s": round(served_rate, 2),
            "speedup": round(served_rate / single_rate, 2),
            "traversals_per_s": round(n_bfs / (single_bfs_ms * 1e-3), 2) if n_bfs else None,
            "traversals_per_s_async_launch": round(n_bfs / (single_async_ms * 1e-3), 2) if n_bfs else None,
            "speedup_vs_async_launch": round(value / (n_bfs / (single_async_ms * 1e-3)), 2) if n_bfs else None,
            "tiles_per_s": round(n_tiles / (single_tile_ms * 1e-3), 1) if n_tiles else None,
            "sample": "%d gcq_bfs_run launches per graph and mode (G-WFQ, 8192 threads; cooperative "
                      "level-synchronous, and asynchronous) and 32 single-tile "
                      "gcq_rt_ctx_render calls per scene (wall clock), averaged and summed over the request mix"
                      % args.serve_sample},
        "work": {"items": items, "stale_items": stale, "edges_scanned": edges, "rays": rays},
        "gpu_launches": args.steps,
        "clocks": clocks,
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": round(peaks["hbm_gbs"], 1),
                     "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": None,
                     "kernel": "k_serve",
                     "peak_source": "device copy bandwidth measured in this run (gcq_roofline_measure); achieved "
                                    "counts the traversals' bytes only, over the whole mixed kernel time"},
        "cpu_baseline": {"value": round(len(reqs) / (cpu_total * 1e-3), 2), "unit": "requests/s", "cores": 1,
                         "kind": "port", "sample": "oracle serial BFS, one request per graph, and a 256x256 serial "
                                                   "render per scene scaled to a tile, summed over the mix"},
        "graph_gen_s": round(gen_s, 1),
    }
    return line


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gcq", "reference"], default="gcq")
    ap.add_argument("--threads", type=int, default=THREADS)
    ap.add_argument("--chunk-ops", type=int, default=CHUNK_OPS)
    ap.add_argument("--capacity-log2", type=int, default=CAPACITY_LOG2)
    ap.add_argument("--cpu-seconds", type=float, default=3.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-per-queue", action="store_true", help="skip the table of all four queues")
    ap.add_argument("--tb-only", action="store_true",
                    help="the queue throughput line alone, without the BFS and served results beside it")
    ap.add_argument("--workload", choices=["tb", "served-bfs", "rt", "bfs", "sweep"], default="tb")
    ap.add_argument("--sweep-queues", default="gwfq,glfq,wfq,sfq")
    ap.add_argument("--sweep-min-log2", type=int, default=10)
    ap.add_argument("--sweep-max-log2", type=int, default=18)
    ap.add_argument("--sweep-warmup-ms", type=float, default=200.0)
    ap.add_argument("--sweep-run-ms", type=float, default=1000.0)
    ap.add_argument("--sweep-md", default="", help="also write the sweep as a markdown table to this file")
    ap.add_argument("--rt-queue", choices=["gwfq", "glfq", "wfq", "sfq"], default="gwfq")
    ap.add_argument("--serve-tiles", type=int, default=2048, help="ray-tile requests mixed into the served stream")
    ap.add_argument("--serve-requests", type=int, default=1024)
    ap.add_argument("--serve-rate", type=float, default=0.0, help="Poisson arrivals per second (0: closed batch)")
    ap.add_argument("--serve-scales", default="16,17,18,19,20,21,22")
    ap.add_argument("--serve-sample", type=int, default=3)
    ap.add_argument("--serve-threads", type=int, default=65536, help="persistent server threads (0: all resident)")
    ap.add_argument("--serve-work-log2", type=int, default=29,
                    help="worklist capacity log2 (0: the library default, 2^25 raised to 4x the largest graph)")
    ap.add_argument("--no-serve-autotune", dest="serve_autotune", action="store_false",
                    help="use --serve-threads / --serve-work-log2 instead of timing candidates on a sample")
    ap.add_argument("--serve-patience", choices=["reference", "fast"], default="fast",
                    help="worklist patience: the reference's 128/256 (wait-free slow path reachable) or "
                         "2^16 (the library default, fast path only)")
    ap.add_argument("--no-serve-poisson", dest="serve_poisson", action="store_false",
                    help="skip the open-loop Poisson run at 70 %% of the closed-batch rate")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "served-bfs":
        return run_served(args)
    if args.workload == "rt":
        return run_rt(args)
    if args.workload == "bfs":
        return run_bfs(args)
    if args.workload == "sweep":
        return run_sweep(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
