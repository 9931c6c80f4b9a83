/* gcq.h: C ABI of libgcq.so, the GB300 (sm_103a) build of gCQ's GPU FIFO queues.
 *
 * The reference has no host API for its queues: each harness allocates a queue
 * with hipMalloc, initialises it with a <<<1,1>>> kernel and calls the per-thread
 * device API from its own kernels (throughout_bench.cpp:415-453, history.cpp:151-177,
 * bfs_bench.cpp:723-737, rt_final.cpp:794-833).  This header is the boundary a host
 * program (or a cgo/ctypes binding) uses instead: the library owns the device memory
 * of a queue, callers hold an opaque handle, and the harness kernels of the four
 * reference harnesses are exposed as calls.  Device code that wants the per-thread
 * API links against the headers in include/gcq/ and gets the device-side queue from
 * gcq_device_ptr().
 *
 * Conventions: every call returns GCQ_OK (0) or a negative gcq_status; no call
 * exits the process (the reference's HIP_CHECK exits, throughout_bench.cpp:79-86).
 * `stream` is a cudaStream_t passed as void* (NULL = the legacy default stream).
 * A handle may be used by one host thread at a time.
 */
#ifndef GCQ_H
#define GCQ_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Queue algorithms; names as in the reference Makefile's QUEUE knob (Makefile:67-81). */
typedef enum { GCQ_GWFQ = 0, GCQ_GLFQ = 1, GCQ_WFQ = 2, GCQ_SFQ = 3 } gcq_kind;

typedef enum {
    GCQ_OK = 0,
    GCQ_EINVAL = -1,        /* bad argument (capacity, thread count, mode) */
    GCQ_ENOMEM = -2,        /* device or host allocation failed */
    GCQ_ECUDA = -3,         /* a CUDA runtime call failed (see gcq_last_cuda_error) */
    GCQ_ETIMEDOUT = -4,     /* a bounded device wait gave up (queue error word) */
    GCQ_EDEVICE = -5,       /* the queue's device error word is set */
    GCQ_EUNSUPPORTED = -6,  /* configuration outside the algorithm's envelope */
    GCQ_ECAPACITY = -7      /* a harness input does not fit the queue */
} gcq_status;

/* Bits of the device error word (gcq_error_word). */
#define GCQ_ERR_SPIN 0x1u      /* a retry loop hit its bound */
#define GCQ_ERR_TIMEOUT 0x2u   /* a blocking wait passed its deadline */
#define GCQ_ERR_TID 0x4u       /* a thread index >= max_threads */
#define GCQ_ERR_POOL 0x8u      /* YMC cell pool exhausted (operations failed, as in the reference) */
#define GCQ_ERR_CAPACITY 0x10u /* harness overflow (e.g. BFS frontier larger than the queue) */

/* Compile-time knobs of the reference, here per queue at run time. */
typedef struct gcq_knobs {
    uint32_t help_delay;          /* G-WFQ WF_HELP_DELAY, gwf_queue.hpp:296-298 (64) */
    uint32_t enq_patience;        /* G-WFQ WF_ENQ_PATIENCE, gwf_queue.hpp:300-302 (128) */
    uint32_t deq_patience;        /* G-WFQ WF_DEQ_PATIENCE, gwf_queue.hpp:304-306 (256) */
    uint32_t remap;               /* slot permutation: 0 identity (the default for both rings here, as the
                                     reference's G-WFQ, gwf_ring.hpp:43-50), 1 spread tickets over 128-B
                                     lines (the reference's G-LFQ default, glf_queue.hpp:116-120) */
    uint32_t ymc_patience;        /* WF_PATIENCE, wfqueue_hip_opt.hpp:29-31 (16) */
    uint32_t ymc_ops_per_thread;  /* WF_PREALLOC_OPS_PER_THREAD, wfqueue_hip_opt.hpp:33-35 (512) */
    uint64_t wait_timeout_ns;     /* deadline of one blocking wait (SFQ), default 2 s */
    uint32_t deq_wait;            /* G-WFQ/G-LFQ: re-reads (with back-off) of a not-yet-filled
                                     slot before a dequeuer marks it; default 8 (0 = mark at
                                     once, as the reference does) */
    uint32_t _pad;
} gcq_knobs;

typedef struct gcq_queue gcq_queue;

/* Fill `k` with the reference defaults (remap follows the kind in gcq_create). */
void gcq_default_knobs(gcq_knobs* k);

/* Create a queue of 2^capacity_log2 elements usable by thread indices
 * [0, max_threads).  Replaces the hipMalloc + queue_init_kernel<<<1,1>>> pair of
 * throughout_bench.cpp:420-442 and the host initialisers wf_queue_host_init
 * (wfqueue_hip_opt.hpp:594-644) and sfq_queue_host_init (sfqueue_hip.cpp:356-390).
 * Envelope checks of the reference, made at run time:
 *   G-WFQ: max_threads <= 2^capacity_log2 (gwf_queue.hpp:320) and the cycle-bit
 *          inequality of gwf_queue.hpp:321-323;
 *   SFQ:   MAX_ID >= 2 * (max_threads + 1) (sfqueue_hip.hpp:45-47);
 *   G-WFQ, G-LFQ: capacity_log2 <= 29 (their Threshold, 3N - 1, is an int).
 * For YMC capacity_log2 is ignored; the pool holds
 * max_threads * (3 * ymc_ops_per_thread + 128) cells plus 8 segments. */
int gcq_create(int kind, uint32_t capacity_log2, uint32_t max_threads, const gcq_knobs* knobs,
               gcq_queue** out);
/* Free the queue's device memory (throughout_bench.cpp:444-453). */
int gcq_destroy(gcq_queue* q);
/* Re-initialise on `stream` with a grid-stride kernel (the reference re-runs its
 * serial init, bfs_bench.cpp:531-552). */
int gcq_reset(gcq_queue* q, void* stream);
/* Device address of the queue object for kernels using the headers in include/gcq/:
 * gcq::gwf::mpmc*, gcq::glf::mpmc*, gcq::ymc::queue* or gcq::sfq::queue*.  As in the
 * reference, a successful enqueue publishes the calling thread's earlier writes to
 * the thread that dequeues the value (release on the enqueue, acquire on the
 * dequeue, at gpu scope). */
int gcq_device_ptr(gcq_queue* q, void** dev);
/* Read (and optionally clear) the device error word; synchronises the device. */
int gcq_error_word(gcq_queue* q, uint32_t* err, int clear);
/* Bytes of device memory held by the queue. */
uint64_t gcq_device_bytes(const gcq_queue* q);
/* G-WFQ operation counters per ring (aq then fq, 8 each: fast-path enqueue
 * attempts, dequeue attempts, dequeue retries, slow enqueues, slow dequeues,
 * finalize calls, finalize record scans, dequeues served by waiting).  Counted only
 * when libgcq.so is built with GCQ_STATS=1 (the reference's GWF_PROFILE counters,
 * gwf_ring.hpp:23-36); otherwise all zero.  out must hold 16 values. */
int gcq_stats(gcq_queue* q, uint64_t* out, int clear);
/* Kind, capacity_log2 and max_threads the queue was created with. */
int gcq_info(const gcq_queue* q, int* kind, uint32_t* capacity_log2, uint32_t* max_threads);
/* Name and SM count of the current CUDA device, for harness output lines (the
 * reference reads hipGetDeviceProperties, throughout_bench.cpp:1058-1062). */
int gcq_device_info(char* name, int name_cap, int* sms);
const char* gcq_strerror(int status);
/* Text of the last failing CUDA call in this process ("" if none). */
const char* gcq_last_cuda_error(void);

/* ---------------------------------------------------------------- history ----
 * One record per completed operation, the fields of WFLogEntry
 * (correctness/wf_linlog.hpp:7-14) and of the JSONL line
 * (correctness/history.cpp:271-280): op 0 enqueue (ret 1 ok / 0 failed),
 * op 1 dequeue (ret value or 0 for empty), op 2 dequeue that failed without
 * effect (SFQ's BUSY; the reference writes it as op 1 ret 0). */
typedef struct gcq_log_entry {
    uint64_t proc;
    uint32_t op;
    uint32_t _pad;
    uint64_t arg;
    uint64_t ret;
    int64_t call;   /* logical clock at call */
    int64_t end;    /* logical clock at return */
} gcq_log_entry;

/* History kernel of correctness/history.cpp:188-227 on `threads` threads (block
 * `block`), `ops` operations each: mode 0 alternating enqueue/dequeue, mode 1 the
 * first producer_percent % of threads enqueue and the rest dequeue.  Values:
 * value_mode 0 = (tid << 32) | (seq + 1) (history.cpp:184), 1 = 32-bit
 * (tid << 16) | (seq + 1); SFQ always uses the 15+16-bit encoding of
 * history.cpp:121-140 and its non-blocking operations.  Every event is bracketed
 * by a device-wide logical clock (wf_linlog.hpp:25-45).  Records with end != 0
 * are sorted by (call, end, proc, op) as history.cpp:257-267 does and copied to
 * host_out (capacity `cap`); *n_out receives the count.  The queue is reset first. */
int gcq_run_history(gcq_queue* q, uint32_t threads, uint32_t block, uint32_t ops, int mode,
                    int producer_percent, int value_mode, gcq_log_entry* host_out, size_t cap,
                    size_t* n_out, void* stream);

/* ------------------------------------------------------------- throughput ----
 * Counters of throughout_bench.cpp:775-785. */
typedef struct gcq_tb_counters {
    uint64_t enq_success, enq_fail, deq_success, deq_empty;
} gcq_tb_counters;

/* One chunk launch of balanced_chunk_kernel (mode 0, throughout_bench.cpp:810-840)
 * or split_chunk_kernel (mode 1, :842-882): each of `threads` threads does
 * chunk_ops iterations; payloads are uint32 splitmix64(seed, tid, i) values.
 * Counters accumulate into dev_counters (device memory, gcq_tb_counters layout).
 * SFQ uses blocking operations in mode 0 and non-blocking ones in mode 1, as the
 * reference does; blocking SFQ needs every thread resident, so mode 0 with more
 * threads than the device can hold at once returns GCQ_EUNSUPPORTED. */
int gcq_tb_launch(gcq_queue* q, int mode, int producer_percent, uint32_t threads, uint32_t block,
                  uint32_t chunk_ops, uint64_t seed, void* dev_counters, void* stream);

/* End-to-end chunk through host memory: moves threads*chunk_ops uint32 payloads
 * (payload i of thread t at host_payloads[i * threads + t]) to the GPU, runs one
 * chunk with them, and copies the counters of that chunk back to host_counters.
 * Pinned payloads (cudaHostAlloc / cudaHostRegister) are read by the kernel in
 * place over the host link while it runs; pageable ones are copied first.  The
 * call synchronises `stream`, then reads the queue's error word: GCQ_ETIMEDOUT or
 * GCQ_EDEVICE when a bounded wait or retry loop gave up during the chunk (the
 * counters then hold what completed), as gcq_tb_run does. */
int gcq_tb_chunk_host(gcq_queue* q, int mode, int producer_percent, uint32_t threads, uint32_t block,
                      uint32_t chunk_ops, const uint32_t* host_payloads, gcq_tb_counters* host_counters,
                      void* stream);

/* Capacity of gcq_tb_chunk_host_noalloc: payloads per call (16 MiB of uint32). */
#define GCQ_NOALLOC_MAX_PAYLOADS (4u * 1024u * 1024u)

/* No counterpart in the reference.  gcq_tb_chunk_host without any device
 * allocation, for callers that cannot call cudaMalloc while they run: code inside a
 * stream-ordered or pool-managed memory regime, real-time callers that may not take
 * the allocator's locks or synchronisation, and embedders that own all device
 * memory.  The payload staging and the counters live in a fixed 16 MiB + 256 B
 * array compiled into libgcq.so (GCQ_NOALLOC_MAX_PAYLOADS payloads; larger
 * threads * chunk_ops returns GCQ_ECAPACITY).  Every GPU that loads the library
 * holds that array until the process exits.  The first call in each CUDA context
 * (per device, and again after cudaDeviceReset) looks up the array's device
 * address with cudaGetSymbolAddress and caches it by the context's id; make that
 * first call before any stream capture.  Like gcq_tb_chunk_host, every call
 * synchronises `stream` before it returns.  All calls share the one array: the
 * counters are cleared at the start of every call, and calls whose work overlaps
 * on the GPU (on different streams, or from different host threads) race on it.
 * Arguments, results and error returns are those of gcq_tb_chunk_host. */
int gcq_tb_chunk_host_noalloc(gcq_queue* q, int mode, int producer_percent, uint32_t threads,
                              uint32_t block, uint32_t chunk_ops, const uint32_t* host_payloads,
                              gcq_tb_counters* host_counters, void* stream);

typedef struct gcq_tb_result {
    gcq_tb_counters counters;
    double gpu_ms;       /* CUDA-event time of the timed window */
    uint64_t launches;   /* chunk launches in the timed window */
} gcq_tb_result;

/* Fixed-duration run of run_balanced_timed / run_split_timed
 * (throughout_bench.cpp:959-1051): warm up for warmup_ms, zero the counters, then
 * replay a CUDA graph of `graph_chunks` chunk launches until run_ms of host time
 * has passed.  The reference launches and synchronises every chunk from the host. */
int gcq_tb_run(gcq_queue* q, int mode, int producer_percent, uint32_t threads, uint32_t block,
               uint32_t chunk_ops, double warmup_ms, double run_ms, uint32_t graph_chunks,
               gcq_tb_result* out);

/* Fixed-duration run for sweeps: gcq_tb_run with every chunk kernel bounded by a
 * device deadline (%globaltimer), stamped at the start of the warm-up and of the
 * timed window, so a configuration whose chunk would run for seconds (SFQ's
 * non-blocking split mode, many consumers polling an almost empty queue) ends with
 * its window and reports the operations it completed.  Chunks are launched one at
 * a time; gpu_ms sums their CUDA-event times.  reset_every > 0 re-initialises the
 * queue (gcq_reset, outside the timed events) before every reset_every-th chunk:
 * YMC consumes its cell pool without reclamation (wfqueue_hip_opt.hpp:208-237), so
 * a reset gives each chunk a fresh pool.  0 never resets.  The reference's loop
 * (run_balanced_timed / run_split_timed, throughout_bench.cpp:959-1051) has no
 * bound on a chunk. */
int gcq_tb_run_bounded(gcq_queue* q, int mode, int producer_percent, uint32_t threads, uint32_t block,
                       uint32_t chunk_ops, double warmup_ms, double run_ms, uint32_t reset_every,
                       gcq_tb_result* out);

/* ------------------------------------------------------------- FIFO check ----
 * Produce-then-drain check of throughout_bench.cpp:456-767 (MODE_FIFO).  Every
 * thread enqueues ops_per_thread tokens (tid << 32 | seq + 1; SFQ 15+16 bits),
 * then all threads drain.  Exactly-once as in the reference (in/out counts,
 * duplicates, missing, out-of-range).  err_order counts token pairs of one
 * producer, seq a < seq b, where the dequeue of b returned before the dequeue of a
 * was called (logical clock); the reference's atomicMax order check (:585-588)
 * starts from 0xFFFFFFFF (:691) and never fires.  ops_per_thread is capped to
 * capacity / threads for bounded queues (:627-653); 0 after the cap = skipped. */
/* Autotuner (no counterpart in the reference, which fixes these at compile time):
 * coordinate descent over block {128..1024}, chunk_ops {32..256} and, for G-WFQ and
 * G-LFQ, the deq_wait back-off {0, 2, 8, 32} and the slot permutation {0, 1}, each
 * candidate a fresh queue of 2^capacity_log2 and a gcq_tb_run of ms_per_point;
 * `passes` rounds over the knobs.  *best receives the fastest point; table (cap
 * entries, may be NULL) every point measured, *n_out their number.  Blocks that do
 * not divide `threads` are skipped (status -1). */
typedef struct gcq_tune_point {
    uint32_t block, chunk_ops, deq_wait, remap;
    double succ_mops;      /* successful operations per microsecond (Mops/s) */
    int32_t status;        /* 0 measured, -1 skipped or failed */
    int32_t _pad;
} gcq_tune_point;

int gcq_tb_autotune(int kind, uint32_t capacity_log2, uint32_t threads, int mode, int producer_percent,
                    double ms_per_point, uint32_t passes, gcq_tune_point* best, gcq_tune_point* table, size_t cap,
                    size_t* n_out);

typedef struct gcq_fifo_result {
    uint64_t in_count, out_count;
    uint32_t err_oob, err_dup, err_order, err_missing, err_gt1;
    uint32_t ops_per_thread;   /* after the capacity cap */
    int verified;              /* 1 = YES, 0 = NO, -1 = skipped */
    int _pad;
} gcq_fifo_result;

int gcq_fifo_check(gcq_queue* q, uint32_t threads, uint32_t block, uint32_t ops_per_thread,
                   gcq_fifo_result* out);

/* The same exactly-once and per-producer order check with producers and consumers
 * running at once, in the roles of split_chunk_kernel (throughout_bench.cpp:842-882:
 * thread t produces when t * 100 / threads < producer_percent).  Each producer
 * enqueues ops_per_producer tokens, retrying while the queue is full; the others
 * dequeue until every token is taken.  No counterpart in the reference, whose FIFO
 * mode produces everything before it drains.  Producers and consumers wait for one
 * another, so every thread must be resident at once: more threads than the device
 * holds returns GCQ_EUNSUPPORTED (as does SFQ above 32768 threads, its token's
 * producer field).  producer_percent in 1..99.  The queue is reset first. */
int gcq_fifo_check_split(gcq_queue* q, uint32_t threads, uint32_t block, int producer_percent,
                         uint32_t ops_per_producer, gcq_fifo_result* out);

/* Dequeue everything the queue holds into host_out (at most cap values) with
 * `threads` threads of the per-thread API, stopping when each thread's dequeue
 * reports empty; *n_out receives the count.  Meant for a quiescent queue (no
 * operation in flight): then an empty dequeue means empty.  Values are returned as
 * the queue holds them (YMC: payload + 1; SFQ: the 32-bit item).  GCQ_ECAPACITY
 * when more than cap values come out (the first cap are kept).  No counterpart in
 * the reference; the tests use it to check a queue's contents. */
int gcq_drain_host(gcq_queue* q, uint32_t threads, uint32_t block, uint64_t* host_out, size_t cap,
                   size_t* n_out);

/* ------------------------------------------------------------------ BFS ----
 * Level-synchronous BFS with a queue as the frontier (concurrent_bfs/bfs_bench.cpp). */
typedef struct gcq_bfs_ctx gcq_bfs_ctx;

typedef struct gcq_bfs_result {
    double total_ms;          /* host time of the whole traversal, init included */
    double kernel_ms;         /* CUDA-event time of the level kernels */
    double init_ms;           /* reset of levels and queues + source enqueue */
    uint64_t edges_scanned;
    uint32_t reached;         /* vertices with a level, the source included */
    int32_t levels;           /* BFS levels processed (the last one finds nothing) */
    uint32_t max_frontier;
    uint32_t drops;           /* enqueues refused because the frontier outgrew the queue */
} gcq_bfs_result;

/* Seeded grid graph: vertex r*cols+c; each right/down edge kept with probability
 * keep_p; from each vertex, with probability diag_p, one diagonal shortcut to the
 * next row.  Undirected CSR (neighbours ascending), arrays from malloc (free them
 * with gcq_free).  With keep_p = 1 and diag_p = 0 it is build_grid of
 * bfs_bench.cpp:245-256. */
int gcq_graph_grid(uint32_t rows, uint32_t cols, double keep_p, double diag_p, uint64_t seed,
                   int32_t** offsets, int32_t** indices, int32_t* V, int64_t* E);
void gcq_free(void* p);

/* Seeded R-MAT graph with 2^scale vertices and edge_factor * 2^scale generated
 * edges (quadrant probabilities a, b, c, 1-a-b-c), self loops and duplicates
 * removed, undirected CSR.  Arrays as for gcq_graph_grid.  No counterpart in the
 * reference, which reads graph files (bfs_bench.cpp:202-243). */
int gcq_graph_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                   int32_t** offsets, int32_t** indices, int32_t* V, int64_t* E);

/* Graph files as the BFS harness reads them (load_mtx / load_snap / csr_from_edges,
 * bfs_bench.cpp:186-243): a MatrixMarket coordinate file (1-based, V = max(rows,
 * cols), entries outside the size dropped) or a SNAP edge list ('#'/'%' comments,
 * ids shifted down when the smallest is 1, V = largest id + 1).  Self loops are
 * dropped, every edge is stored in both directions, duplicates are removed and each
 * adjacency list is sorted.  Arrays as for gcq_graph_grid.  GCQ_EINVAL for a
 * missing or malformed file. */
int gcq_graph_load_mtx(const char* path, int32_t** offsets, int32_t** indices, int32_t* V, int64_t* E);
int gcq_graph_load_snap(const char* path, int32_t** offsets, int32_t** indices, int32_t* V, int64_t* E);

/* Upload the CSR and create the two frontier queues of `kind` for `threads`
 * worker threads (a multiple of 32) with capacity 2^capacity_log2 (0 = the
 * smallest power of two >= V, at least 2^15, within the queue's envelope).
 * Replaces bfs_bench.cpp:702-737. */
int gcq_bfs_create(int kind, const int32_t* offsets, const int32_t* indices, int32_t V, int64_t E,
                   uint32_t threads, uint32_t capacity_log2, const gcq_knobs* knobs, gcq_bfs_ctx** out);
int gcq_bfs_destroy(gcq_bfs_ctx* c);

/* One traversal from src (run_bfs, bfs_bench.cpp:509-633).  persistent = 0 launches
 * bfs_expand_kernel + bfs_hub_kernel per level and reads the next frontier size on
 * the host, as the reference does; persistent = 1 runs every level in one
 * cooperative launch with grid barriers; persistent = 2 (G-WFQ, G-LFQ) runs an
 * asynchronous label-correcting traversal in one launch with one queue and no
 * level barrier (same depths; max_frontier is reported as 0).  host_levels (V entries, may be NULL)
 * receives the depths, -1 for unreached vertices.  A frontier larger than the queue
 * returns GCQ_ECAPACITY (the reference drops the vertices silently). */
int gcq_bfs_run(gcq_bfs_ctx* c, int32_t src, uint32_t block, int persistent, int32_t* host_levels,
                gcq_bfs_result* out);

/* ------------------------------------------------------------ ray tracer ----
 * Persistent per-tile ray tracer (concurrent_rt/rt_final.cpp). */
typedef struct gcq_rt_result {
    double gen_ms;          /* k_generate */
    double trace_ms;        /* k_trace: every bounce in one launch */
    double total_ms;
    uint64_t primary_rays;
    uint64_t total_rays;    /* rays traced, bounces included */
    uint64_t leftover;      /* rays still alive after the trace (must be 0) */
} gcq_rt_result;

/* Render one frame of the reference scene `scene` (0 spheres, 1 Cornell-style box;
 * rt_final.cpp:650-684, cameras :849-859) at width x height in tiles_x x tiles_y
 * tiles, threads_per_tile workers and one queue of 2^queue_log2 per tile, up to
 * max_bounces reflections.  kind: any of the four queues (YMC as the reference's
 * USE_WFQ tracer, rt_final.cpp:141-170, with one cell pool per tile; a pool that
 * runs dry returns GCQ_ECAPACITY).  image (may be
 * NULL) receives width*height RGB floats.  Replaces rt_final.cpp:705-1018. */
int gcq_rt_render(int kind, int scene, int width, int height, int tiles_x, int tiles_y, int threads_per_tile,
                  int max_bounces, uint32_t queue_log2, float* image, gcq_rt_result* out);

/* The ray-tracing workload of the benchmark configuration (no reference
 * counterpart): scene 0 = 512 seeded spheres (diffuse / metal / glass) over a ground
 * quad under a sky, scene 1 = a box room with two boxes and a ceiling light; one
 * sample per pixel, 32-byte rays in per-tile ray-bounce queues (tile_px x tile_px
 * pixels, threads_per_tile workers, 2^queue_log2 entries per tile), paths of at most
 * max_bounces scattering events from `seed`.  kind: any of the four queues.
 * Sampling uses integer PCG and rejection, so the image is reproducible bit for bit
 * on the CPU. */
int gcq_rt_bounce_render(int kind, int scene, int width, int height, int tile_px, int threads_per_tile,
                         int max_bounces, uint32_t queue_log2, uint64_t seed, float* image, gcq_rt_result* out);

/* The same renderer as a context that renders lists of tiles, for callers that
 * render a tile at a time (one launch per tile request).  Rings, ray storage for
 * up to max_tiles tiles (<= 0: every tile) and the device image are allocated
 * once; gcq_rt_ctx_render renders the listed row-major tile indices (tiles NULL:
 * all, which needs max_tiles <= 0) into the image and copies the whole image to
 * `image` when it is not NULL.  A tile's pixels are the same whichever list
 * renders it. */
typedef struct gcq_rt_ctx gcq_rt_ctx;
int gcq_rt_ctx_create(int kind, int scene, int width, int height, int tile_px, int threads_per_tile,
                      int max_bounces, uint32_t queue_log2, uint64_t seed, int max_tiles, gcq_rt_ctx** out);
int gcq_rt_ctx_render(gcq_rt_ctx* ctx, const int32_t* tiles, int ntiles, float* image, gcq_rt_result* out);
int gcq_rt_ctx_destroy(gcq_rt_ctx* ctx);

/* The stream-compaction baseline (concurrent_rt/baselines/rt_compaction.cpp): the
 * same scenes (plus its scene 2, the mirror tunnel, which gcq_rt_render also
 * accepts), double-buffered ray lists packed in order after every pass, its own
 * shading (each bounce weighted 0.5 and added; depth 0 written).  image (may be
 * NULL) receives width*height RGB floats.  A non-queue comparator for the
 * persistent per-tile tracer. */
int gcq_rt_compact_render(int scene, int width, int height, int max_bounces, float* image, gcq_rt_result* out);

/* ------------------------------------------------------------- roofline ----
 * The atomic roofline of this GPU, measured by a microbenchmark in the same
 * process (the reference reports raw Mops/s only).  Rates are operations per
 * second (r1_warp: tickets per second); hbm_gbs is copy read+write GB/s. */
typedef struct gcq_roofline {
    double r1_single;    /* one 64-bit word, atomicAdd from every thread */
    double r1_warp;      /* one word, warp-aggregated tickets */
    double rs_lines;     /* spread fetch-add, one 128-B line per thread */
    double rs_contig;    /* spread fetch-add, a warp on 32 consecutive words */
    double rc_lines;     /* spread 64-bit CAS, one line per thread */
    double rc128_lines;  /* spread 128-bit CAS (atom.cas.b128) */
    double hbm_gbs;      /* device copy bandwidth */
    int sms;
    int _pad;
    double fp32_gops;    /* unfused fp32 multiplies + adds per second (1e9), all SMs */
} gcq_roofline;

/* Run the microbenchmark (best of `reps`); synchronises the device. */
int gcq_roofline_measure(gcq_roofline* out, int reps);

/* --------------------------------------------------------- served BFS ----
 * A persistent server of BFS traversal requests over several resident graphs,
 * built on G-WFQ queues (Enqueue_Ptr/Dequeue_Ptr, gwf_ring.hpp:1362-1380) and the
 * persistent worker loop of the ray tracer (rt_final.cpp:574-641).  The reference
 * runs one traversal per process (bfs_bench.cpp:327-496); it has no server.
 *
 * Requests arrive on the device clock (arrival_ns after the start of the run).  A
 * request is admitted when a level-array slot of its graph is free (slots are
 * carved out of budget_bytes, an even share per graph) and its graph's vertex count
 * fits the worklist reservation.  Each traversal computes exact hop distances and
 * returns, instead of the level array, its checksum
 *     sum over v < V of splitmix64(v << 32 | level(v))   (mod 2^64)
 * with level 0xFFFFFFFF for unreached vertices, its reached count and its
 * eccentricity (max_level). */
typedef struct gcq_server gcq_server;

typedef struct gcq_serve_cfg {
    uint64_t budget_bytes;  /* HBM for level arrays; default 150 GiB */
    uint64_t timeout_ns;    /* bound of every device wait; default 10 s */
    uint32_t max_slots;     /* level-array slots per graph, at most; default 1024 */
    uint32_t threads;       /* persistent threads; 0 = every resident thread */
    uint32_t work_log2;     /* worklist capacity (<= 29); default 25, raised to 4 x the
                               largest graph.  Each large traversal reserves V entries, so
                               a larger worklist admits more of them at once */
    uint32_t _pad;
    uint64_t run_limit_ns;  /* a run gives up (GCQ_ETIMEDOUT) this long after the last
                               arrival; default 60 s */
    gcq_knobs work_knobs;   /* knobs of the worklist queue; default gcq_default_knobs */
    /* Ray tiles (gcq_rt_bounce_render's scenes): rt_scenes > 0 serves tile requests of
     * scenes 0 .. rt_scenes-1 as targets ngraphs + scene.  Default 0 (none); the
     * other fields default to the benchmark image (1024 x 1024, 32-pixel tiles,
     * 4 bounces, seed 1) and 1024 tile slots per scene. */
    uint32_t rt_scenes;
    uint32_t rt_width, rt_height, rt_tile_px, rt_max_bounces, rt_slots;
    uint64_t rt_seed;
} gcq_serve_cfg;

typedef struct gcq_serve_req {
    int32_t graph;          /* target: a graph given to gcq_serve_create, or
                               ngraphs + scene for a ray tile */
    int32_t src;            /* source vertex, or the tile's row-major index */
    uint64_t arrival_ns;    /* release time (<= 60 s); requests are sorted by it */
} gcq_serve_req;

typedef struct gcq_serve_res {
    uint64_t admit_ns;      /* slot granted */
    uint64_t done_ns;       /* last vertex settled / last path of the tile ended */
    uint64_t finish_ns;     /* checksum folded, slot returned (response time) */
    uint64_t checksum;      /* traversal: see gcq_serve_run; tile: sum over its pixels g
                               and channels c of splitmix64((3g + c) << 32 | float bits) */
    uint32_t reached;       /* vertices reached; tile: rays traced */
    int32_t max_level;      /* eccentricity of the source; tile: longest path in rays */
} gcq_serve_res;

typedef struct gcq_serve_stats {
    double kernel_ms;       /* CUDA-event time of the persistent kernel */
    uint64_t items;         /* vertex items dequeued */
    uint64_t stale;         /* of those, superseded by a shorter path */
    uint64_t edges;         /* adjacency entries scanned */
    uint64_t sweeps;        /* checksum/reset sweeps of level arrays */
    uint32_t completed;
    uint32_t error_word;
    uint32_t released;      /* requests moved into submission queues */
    uint32_t inflight;      /* slots still holding a traversal at the end (0 after success) */
    uint64_t reserved;      /* worklist reservation left at the end (0 after success) */
    uint64_t work_tail[2];  /* ticket counters of the worklist's rings at the end: */
    uint64_t work_head[2];  /*   [0] the item ring, [1] the free-index ring */
    int32_t work_threshold[2];
    uint64_t rays;          /* ray items traced (tile requests) */
} gcq_serve_stats;

void gcq_serve_default_cfg(gcq_serve_cfg* cfg);
/* Upload the CSR graphs (host arrays as made by gcq_graph_grid/gcq_graph_rmat) and
 * allocate slots and queues.  GCQ_EINVAL for a malformed CSR (offsets not starting
 * at 0, decreasing or not ending at E; a neighbour outside [0, V)); GCQ_ECAPACITY
 * if one level array of a graph does not fit its share of the budget. */
int gcq_serve_create(int ngraphs, const int32_t* const* offsets, const int32_t* const* indices,
                     const int32_t* V, const int64_t* E, const gcq_serve_cfg* cfg, gcq_server** out);
int gcq_serve_destroy(gcq_server* s);
/* Slots of `graph` (-1: all graphs), persistent threads, bytes of level arrays. */
int gcq_serve_info(const gcq_server* s, int graph, uint32_t* slots, uint32_t* threads, uint64_t* level_bytes);
/* Serve nreq requests (<= 2^20, sorted by arrival_ns) in one persistent launch;
 * res[i] answers reqs[i].  Synchronises the device. */
int gcq_serve_run(gcq_server* s, const gcq_serve_req* reqs, uint32_t nreq, gcq_serve_res* res,
                  gcq_serve_stats* stats);
/* Copy the image of a served scene (rt_width * rt_height RGB floats): every pixel
 * of a tile served so far equals gcq_rt_bounce_render's. */
int gcq_serve_image(const gcq_server* s, int scene, float* image);

#ifdef __cplusplus
}
#endif

#endif /* GCQ_H */
