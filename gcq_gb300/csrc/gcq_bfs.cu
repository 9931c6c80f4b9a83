// BFS with a queue as the frontier worklist (concurrent_bfs/bfs_bench.cpp), for all
// four queues: the reference's level-synchronous form (one expand + hub launch per
// level, host sync per level, bfs_bench.cpp:509-633) and a persistent form (one
// cooperative launch for the whole traversal, levels separated by a bounded grid
// barrier).  Also the seeded grid-graph generator of the benchmark graphs.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

#include "gcq_internal.cuh"

using gcqi::qops;

struct gcq_bfs_ctx {
    int kind;
    int32_t V;
    int64_t E;
    int32_t* d_off;
    int32_t* d_idx;
    int32_t* d_level;
    int32_t* d_hubs;
    gcq_queue* qa;
    gcq_queue* qb;
    uint32_t threads;
    void* d_misc;          // counters: see struct bfs_misc
    void* h_misc;          // pinned mirror
    cudaStream_t stream;
};

namespace {

// Device counters of one traversal (one 256-B block).
struct bfs_misc {
    unsigned int next_count;     // vertices enqueued for the next level
    unsigned int hub_count;      // hub vertices of the current level
    unsigned long long edges;    // edges scanned (all levels)
    unsigned int levels;         // persistent form: levels completed
    unsigned int drops;          // enqueues that failed (frontier larger than the queue)
    unsigned int bar_count, bar_gen;   // persistent form: grid barrier
    unsigned int reached;        // vertices that got a level
    unsigned int max_frontier;
    unsigned int err;
};

constexpr int INLINE_DEG = 32;     // bfs_bench.cpp:286-288
constexpr int HUB_DEG = 4096;      // bfs_bench.cpp:290-292

__device__ __forceinline__ uint64_t encode_vtx(int v) { return (uint64_t)(uint32_t)v + 1ULL; }   // :138-142
__device__ __forceinline__ int decode_vtx(uint64_t x) { return (int)(x - 1ULL); }

// Queue adapters for BFS (bfs_bench.cpp:35-132): SFQ enqueues blocking and
// dequeues non-blocking with an explicit empty test (head >= tail).
template <int K>
__device__ __forceinline__ bool bfs_enq(void* q, uint64_t v, uint32_t tid) {
    return qops<K>::enq(reinterpret_cast<typename qops<K>::Q*>(q), v, tid, false);
}
template <int K>
__device__ __forceinline__ bool bfs_deq(void* q, uint64_t* out, uint32_t tid) {
    if (K == GCQ_SFQ) {
        auto* s = reinterpret_cast<gcq::sfq::queue*>(q);
        for (int tries = 0; tries < 1 << 16; ++tries) {
            uint32_t item = 0;
            if (gcq::sfq::dequeue_nb(s, &item) == SFQ_SUCCESS) { *out = item; return true; }
            const uint32_t h = gcq::ld_acq(&s->head), t = gcq::ld_acq(&s->tail);
            if ((int32_t)(t - h) <= 0) return false;
            __nanosleep(64);
        }
        return false;
    }
    return qops<K>::deq(reinterpret_cast<typename qops<K>::Q*>(q), out, tid, false) == 1;
}

// Scan the neighbours [beg, end) with stride `step` from offset `first`; claim
// unvisited ones with atomicCAS(level, -1, next) and enqueue them.
template <int K>
__device__ __forceinline__ void scan_edges(int beg, int end, int first, int step, const int* __restrict__ idx,
                                           int* __restrict__ level, int next_level, void* qout, uint32_t tid,
                                           unsigned long long& loc_edges, unsigned int& loc_next, bfs_misc* m) {
    for (int e = beg + first; e < end; e += step) {
        ++loc_edges;
        const int w = idx[e];
        if (atomicCAS(&level[w], -1, next_level) == -1) {
            if (bfs_enq<K>(qout, encode_vtx(w), tid)) ++loc_next;
            else atomicAdd(&m->drops, 1u);
        }
    }
}

__device__ __forceinline__ void block_add(unsigned long long edges, unsigned int next, bfs_misc* m) {
    __shared__ unsigned long long s_e[32];
    __shared__ unsigned int s_n[32];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    for (int o = 16; o > 0; o >>= 1) {
        edges += __shfl_down_sync(0xffffffffu, edges, o);
        next += __shfl_down_sync(0xffffffffu, next, o);
    }
    if (lane == 0) { s_e[warp] = edges; s_n[warp] = next; }
    __syncthreads();
    if (warp == 0) {
        edges = lane < nw ? s_e[lane] : 0ull;
        next = lane < nw ? s_n[lane] : 0u;
        for (int o = 16; o > 0; o >>= 1) {
            edges += __shfl_down_sync(0xffffffffu, edges, o);
            next += __shfl_down_sync(0xffffffffu, next, o);
        }
        if (lane == 0) {
            if (edges) atomicAdd(&m->edges, edges);
            if (next) atomicAdd(&m->next_count, next);
        }
    }
    __syncthreads();
}

// One level's expansion by this thread: bfs_expand_kernel, bfs_bench.cpp:327-431.
// Every lane of the warp stays in the loop until the whole warp found the input
// queue empty (the reference exits on a full-warp ballot, :411-413); all ballots
// and shuffles use the full mask, so the launch keeps every lane (threads are a
// multiple of 32 and all lanes run this function).
template <int K>
__device__ __forceinline__ void expand_level(void* qin, void* qout, const int* __restrict__ off,
                                             const int* __restrict__ idx, int* __restrict__ level, int curr,
                                             int* __restrict__ hubs, bfs_misc* m, uint32_t tid,
                                             unsigned long long& loc_edges, unsigned int& loc_next) {
    const int lane = (int)gcq::lane_id();
    int pending = -1;
    for (uint32_t guard = 0;; ++guard) {
        uint64_t item = 0;
        const bool got = bfs_deq<K>(qin, &item, tid);
        const int u = got ? decode_vtx(item) : -1;
        if (u >= 0) {
            const int beg = off[u], end = off[u + 1], deg = end - beg;
            if (deg <= INLINE_DEG) {
                scan_edges<K>(beg, end, 0, 1, idx, level, curr + 1, qout, tid, loc_edges, loc_next, m);
            } else if (deg >= HUB_DEG) {
                const unsigned int h = atomicAdd(&m->hub_count, 1u);
                hubs[h] = u;
            } else {
                pending = u;
            }
        }
        // warp-cooperative medium-degree vertices (bfs_bench.cpp:392-409)
        for (;;) {
            const unsigned mask = __ballot_sync(0xffffffffu, pending >= 0);
            if (mask == 0) break;
            const int owner = __ffs(mask) - 1;
            const int ou = __shfl_sync(0xffffffffu, pending, owner);
            scan_edges<K>(off[ou], off[ou + 1], lane, 32, idx, level, curr + 1, qout, tid, loc_edges, loc_next, m);
            if (lane == owner) pending = -1;
        }
        if (__ballot_sync(0xffffffffu, u < 0) == 0xffffffffu) break;
        if (guard > (1u << 30)) { gcq::raise_error(&m->err, gcq::ERR_SPIN); break; }
    }
}

// Hub vertices, one block per hub (bfs_hub_kernel, bfs_bench.cpp:434-496).
template <int K>
__device__ __forceinline__ void expand_hubs(void* qout, const int* __restrict__ off, const int* __restrict__ idx,
                                            int* __restrict__ level, int curr, const int* __restrict__ hubs,
                                            unsigned int nhubs, bfs_misc* m, uint32_t tid, unsigned block_id,
                                            unsigned nblocks, unsigned long long& loc_edges, unsigned int& loc_next) {
    for (unsigned int h = block_id; h < nhubs; h += nblocks) {
        const int u = hubs[h];
        scan_edges<K>(off[u], off[u + 1], (int)threadIdx.x, (int)blockDim.x, idx, level, curr + 1, qout, tid,
                      loc_edges, loc_next, m);
    }
}

template <int K>
__global__ void k_bfs_expand(void* qin, void* qout, const int* __restrict__ off, const int* __restrict__ idx,
                             int* __restrict__ level, int curr, int* __restrict__ hubs, bfs_misc* m) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long loc_edges = 0;
    unsigned int loc_next = 0;
    expand_level<K>(qin, qout, off, idx, level, curr, hubs, m, tid, loc_edges, loc_next);
    block_add(loc_edges, loc_next, m);
}

template <int K>
__global__ void k_bfs_hubs(void* qout, const int* __restrict__ off, const int* __restrict__ idx,
                           int* __restrict__ level, int curr, const int* __restrict__ hubs, bfs_misc* m) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long loc_edges = 0;
    unsigned int loc_next = 0;
    const unsigned int nhubs = *(volatile unsigned int*)&m->hub_count;
    expand_hubs<K>(qout, off, idx, level, curr, hubs, nhubs, m, tid, blockIdx.x, gridDim.x, loc_edges, loc_next);
    block_add(loc_edges, loc_next, m);
}

// Source setup: level[src] = 0 and enqueue src (enqueue_source_kernel, :304-322).
template <int K>
__global__ void k_bfs_source(void* q, int* level, int src, bfs_misc* m) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        level[src] = 0;
        if (!bfs_enq<K>(q, encode_vtx(src), 0)) atomicAdd(&m->drops, 1u);
    }
}

// ------------------------------------------------------------- asynchronous form
// One persistent launch, one queue, no level barrier: a label-correcting BFS.  An
// item is (level << 32 | vertex); a vertex of more than ASYNC_HUB_DEG neighbours is
// expanded as chunk items (1 << 63 | chunk << 32 | vertex) of CHUNK_EDGES edges each,
// so many warps share a hub; a chunk relaxes with the vertex's current level.  Relaxing an edge lowers the neighbour's level
// with atomicMin on the unsigned level (unvisited -1 is above every level) and
// queues it when it dropped; an item whose vertex already has a smaller level is
// stale.  The final levels are exact hop distances in any processing order.  A
// pending count (items queued, not yet settled; one update per item, by
// children - 1) ends the traversal at zero.  The reference has no such form: its
// traversal synchronises the grid once per level (bfs_bench.cpp:583-623), which
// bounds it below by levels x barrier latency on high-diameter graphs.
constexpr int ASYNC_HUB_DEG = 2048;
constexpr int CHUNK_EDGES = 1024;
constexpr uint64_t CHUNK_FLAG = 1ull << 63;
// A thread's edges are relaxed GCQ_BFS_RELAX_BATCH at a time: their
// neighbour ids are loaded, then their atomicMins issued back to back, so one
// vertex costs about two dependent round trips instead of one per edge.
#ifndef GCQ_BFS_RELAX_BATCH
#define GCQ_BFS_RELAX_BATCH 4
#endif

struct bfs_async_ctl {
    unsigned long long pending;
    unsigned int done;
    unsigned int err;
    unsigned long long edges;
    unsigned long long items, stale;
    unsigned long long deadline_ns;
    unsigned long long timeout_ns;
};

template <int K> struct async_q;
template <> struct async_q<GCQ_GWFQ> {
    using Q = gcq::gwf::mpmc;
    __device__ static bool peek(Q* q) { return gcq::gwf::maybe_nonempty(&q->aq); }
    __device__ static bool deq(Q* q, uint64_t* v, uint32_t tid) { return gcq::gwf::try_dequeue_ptr(q, v, tid, 2); }
    __device__ static bool enq(Q* q, uint64_t v, uint32_t tid) { return gcq::gwf::enqueue_ptr_lockfree(q, v, tid, 64); }
    __device__ static uint64_t mark(Q* q) { return gcq::ld_rlx(&q->aq.Tail); }
};
template <> struct async_q<GCQ_GLFQ> {
    using Q = gcq::glf::mpmc;
    __device__ static bool peek(Q* q) { return gcq::ld_rlx(&q->aq.Tail) > gcq::ld_rlx(&q->aq.Head); }
    __device__ static bool deq(Q* q, uint64_t* v, uint32_t) { return gcq::glf::dequeue_ptr(q, v); }
    __device__ static bool enq(Q* q, uint64_t v, uint32_t) { return gcq::glf::enqueue_ptr(q, v); }
    __device__ static uint64_t mark(Q* q) { return gcq::ld_rlx(&q->aq.Tail); }
};

template <int K>
__device__ __forceinline__ void async_push(typename async_q<K>::Q* q, uint64_t it, uint32_t tid, bfs_async_ctl* c) {
    if (async_q<K>::enq(q, it, tid)) return;
    const uint64_t t0 = gcq::globaltimer_ns();
    uint32_t ns = 32;
    do {
        if (gcq::globaltimer_ns() - t0 > c->timeout_ns) { gcq::raise_error(&c->err, gcq::ERR_CAPACITY); return; }
        __nanosleep(ns);
        ns = ns < 2048 ? ns * 2 : ns;
    } while (!async_q<K>::enq(q, it, tid));
}

__device__ __forceinline__ void async_settle(bfs_async_ctl* c, uint32_t children) {
    if (children == 1) return;   // the child inherits the item's count
    const uint64_t prev = gcq::fetch_add((gcq::u64a*)&c->pending, (uint64_t)children - 1);
    if (children == 0 && prev == 1) gcq::st_rel((gcq::u32a*)&c->done, 1u);
}

template <int K>
__global__ void __launch_bounds__(256) k_bfs_async(void* qv, const int* __restrict__ off, const int* __restrict__ idx,
                                                   unsigned int* __restrict__ level, bfs_async_ctl* c) {
    using Q = typename async_q<K>::Q;
    Q* q = (Q*)qv;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = (int)(threadIdx.x & 31);
    const unsigned FULL = 0xffffffffu;
    unsigned long long n_edges = 0, n_items = 0, n_stale = 0;
    uint64_t idle_since = 0, idle_mark = 0;
    uint32_t ns = 0;
    for (;;) {
        uint32_t stop = 0;
        if (lane == 0) {
            stop = (gcq::ld_acq((const gcq::u32a*)&c->done) || gcq::ld_rlx((const gcq::u32a*)&c->err)) ? 1u : 0u;
            if (!stop && gcq::globaltimer_ns() > c->deadline_ns) {
                gcq::raise_error(&c->err, gcq::ERR_TIMEOUT);
                stop = 1;
            }
        }
        if (__shfl_sync(FULL, stop, 0)) break;
        uint64_t it = 0;
        const bool got = async_q<K>::peek(q) && async_q<K>::deq(q, &it, tid);
        int big = 0;           // 1: a vertex of 33..ASYNC_HUB_DEG neighbours, 2: a chunk of a hub
        uint32_t v = 0, lvl = 0;
        int rb = 0, re = 0;    // edge range of the warp-wide work
        if (got) {
            ++n_items;
            v = (uint32_t)it;
            if (it & CHUNK_FLAG) {
                const uint32_t k = (uint32_t)(it >> 32) & 0x7FFFFFFFu;
                lvl = gcq::ld_rlx((const gcq::u32a*)&level[v]);
                const int beg = off[v], end = off[v + 1];
                rb = beg + (int)k * CHUNK_EDGES;
                re = min(end, rb + CHUNK_EDGES);
                big = 2;
            } else if (lvl = (uint32_t)(it >> 32), gcq::ld_rlx((const gcq::u32a*)&level[v]) < lvl) {
                ++n_stale;
                async_settle(c, 0);
            } else {
                const int beg = off[v], end = off[v + 1];
                if (end - beg > ASYNC_HUB_DEG) {
                    // split into chunk items; they inherit this item's count
                    const uint32_t chunks = (uint32_t)((end - beg + CHUNK_EDGES - 1) / CHUNK_EDGES);
                    gcq::fetch_add((gcq::u64a*)&c->pending, (uint64_t)chunks - 1);
                    for (uint32_t k = 0; k < chunks; ++k) async_push<K>(q, CHUNK_FLAG | ((uint64_t)k << 32) | v, tid, c);
                } else if (end - beg > 32) {
                    rb = beg;
                    re = end;
                    big = 1;
                } else {
                    n_edges += (unsigned long long)(end - beg);
                    const uint32_t lv = lvl + 1;
                    uint32_t won = 0;
                    for (int e0 = beg; e0 < end; e0 += GCQ_BFS_RELAX_BATCH) {
                        uint32_t w[GCQ_BFS_RELAX_BATCH], old[GCQ_BFS_RELAX_BATCH];
#pragma unroll
                        for (int j = 0; j < GCQ_BFS_RELAX_BATCH; ++j)
                            if (e0 + j < end) w[j] = (uint32_t)idx[e0 + j];
#pragma unroll
                        for (int j = 0; j < GCQ_BFS_RELAX_BATCH; ++j)
                            if (e0 + j < end) old[j] = atomicMin(&level[w[j]], lv);
#pragma unroll
                        for (int j = 0; j < GCQ_BFS_RELAX_BATCH; ++j)
                            if (e0 + j < end && old[j] > lv) won |= 1u << (e0 + j - beg);
                    }
                    const uint32_t kids = (uint32_t)__popc(won);
                    if (kids > 1) gcq::fetch_add((gcq::u64a*)&c->pending, (uint64_t)kids - 1);
                    for (uint32_t mm = won; mm; mm &= mm - 1)
                        async_push<K>(q, ((uint64_t)lv << 32) | (uint32_t)idx[beg + __ffs(mm) - 1], tid, c);
                    if (kids == 0) async_settle(c, 0);
                }
            }
        }
        // vertices of degree > 32 and hub chunks: the whole warp, one at a time
        for (unsigned want = __ballot_sync(FULL, big != 0); want; want = __ballot_sync(FULL, big != 0)) {
            const int owner = __ffs(want) - 1;
            const uint32_t lv = __shfl_sync(FULL, lvl, owner) + 1;
            const int beg = __shfl_sync(FULL, rb, owner), end = __shfl_sync(FULL, re, owner);
            if (lane == owner) n_edges += (unsigned long long)(end - beg);
            for (int base = beg; base < end; base += 32) {
                const int e = base + lane;
                uint32_t w = 0;
                bool won = false;
                if (e < end) {
                    w = (uint32_t)idx[e];
                    won = atomicMin(&level[w], lv) > lv;
                }
                const unsigned wm = __ballot_sync(FULL, won);
                // count the children before any of them can be dequeued
                if (lane == owner && wm) gcq::fetch_add((gcq::u64a*)&c->pending, (uint64_t)__popc(wm));
                __syncwarp();
                if (won) async_push<K>(q, ((uint64_t)lv << 32) | w, tid, c);
            }
            if (lane == owner) {
                async_settle(c, 0);
                big = 0;
            }
        }
        if (got) {
            ns = 0;
            idle_since = 0;
        } else {
            // stall detection: no enqueue anywhere for a whole timeout
            const uint64_t t = gcq::globaltimer_ns();
            const uint64_t mk = async_q<K>::mark(q);
            if (idle_since == 0 || mk != idle_mark) {
                idle_since = t;
                idle_mark = mk;
            } else if (t - idle_since > c->timeout_ns) {
                gcq::raise_error(&c->err, gcq::ERR_TIMEOUT);
            }
            if (ns) __nanosleep(ns);
            ns = ns ? (ns < 1024 ? ns * 2 : ns) : 32;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        n_edges += __shfl_xor_sync(FULL, n_edges, o);
        n_items += __shfl_xor_sync(FULL, n_items, o);
        n_stale += __shfl_xor_sync(FULL, n_stale, o);
    }
    if (lane == 0) {
        atomicAdd(&c->edges, n_edges);
        atomicAdd(&c->items, n_items);
        atomicAdd(&c->stale, n_stale);
    }
}

__global__ void k_bfs_set_deadline(bfs_async_ctl* c, uint64_t after_ns) {
    if (blockIdx.x == 0 && threadIdx.x == 0) c->deadline_ns = gcq::globaltimer_ns() + after_ns;
}

template <int K>
__global__ void k_bfs_async_source(void* qv, unsigned int* level, int src, bfs_async_ctl* c) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        level[src] = 0;
        c->pending = 1;
        if (!async_q<K>::enq((typename async_q<K>::Q*)qv, (uint32_t)src, 0)) gcq::raise_error(&c->err, gcq::ERR_CAPACITY);
    }
}

// reached vertices and the largest level, for the asynchronous form
__global__ void k_bfs_summary(const int* __restrict__ level, int V, bfs_misc* m) {
    unsigned int reached = 0, maxl = 0;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += gridDim.x * blockDim.x) {
        const int l = level[v];
        if (l >= 0) {
            ++reached;
            maxl = max(maxl, (unsigned)l);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        reached += __shfl_xor_sync(0xffffffffu, reached, o);
        maxl = max(maxl, __shfl_xor_sync(0xffffffffu, maxl, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&m->reached, reached);
        atomicMax(&m->levels, maxl + 1);
    }
}

// Grid barrier for the persistent form: every block of a cooperative launch arrives
// once per phase; the wait is bounded and reports through m->err.
__device__ __forceinline__ bool grid_barrier(bfs_misc* m, uint64_t timeout_ns) {
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        ok = 1;
        const unsigned int gen = gcq::ld_acq(&m->bar_gen);
        if (atomicAdd(&m->bar_count, 1u) == gridDim.x - 1) {
            m->bar_count = 0;
            gcq::st_rel(&m->bar_gen, gen + 1u);
        } else {
            const uint64_t t0 = gcq::globaltimer_ns();
            uint32_t ns = 32;
            while (gcq::ld_acq(&m->bar_gen) == gen) {
                if (gcq::globaltimer_ns() - t0 > timeout_ns) { gcq::raise_error(&m->err, gcq::ERR_TIMEOUT); ok = 0; break; }
                __nanosleep(ns);
                ns = ns < 256 ? ns * 2 : ns;
            }
        }
    }
    __syncthreads();
    return ok != 0;
}

// The whole traversal in one cooperative launch: expand, hubs and the level
// bookkeeping of run_bfs (:583-623) separated by grid barriers.
template <int K>
__global__ void k_bfs_persistent(void* qa, void* qb, const int* __restrict__ off, const int* __restrict__ idx,
                                 int* __restrict__ level, int* __restrict__ hubs, bfs_misc* m, uint64_t timeout_ns) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    void* qin = qa;
    void* qout = qb;
    for (int curr = 0;; ++curr) {
        unsigned long long loc_edges = 0;
        unsigned int loc_next = 0;
        expand_level<K>(qin, qout, off, idx, level, curr, hubs, m, tid, loc_edges, loc_next);
        if (!grid_barrier(m, timeout_ns)) return;
        const unsigned int nhubs = gcq::ld_acq(&m->hub_count);
        expand_hubs<K>(qout, off, idx, level, curr, hubs, nhubs, m, tid, blockIdx.x, gridDim.x, loc_edges, loc_next);
        block_add(loc_edges, loc_next, m);
        if (!grid_barrier(m, timeout_ns)) return;
        const unsigned int next = gcq::ld_acq(&m->next_count);
        if (!grid_barrier(m, timeout_ns)) return;   // everyone has read next_count
        if (tid == 0) {
            m->reached += next;
            m->max_frontier = max(m->max_frontier, next);
            m->levels = curr + 1;
            m->next_count = 0;
            m->hub_count = 0;
        }
        if (next == 0) return;
        if (!grid_barrier(m, timeout_ns)) return;
        void* t = qin; qin = qout; qout = t;
    }
}

template <typename F>
int dispatch(int kind, F&& f) {
    switch (kind) {
        case GCQ_GWFQ: return f(std::integral_constant<int, GCQ_GWFQ>());
        case GCQ_GLFQ: return f(std::integral_constant<int, GCQ_GLFQ>());
        case GCQ_WFQ: return f(std::integral_constant<int, GCQ_WFQ>());
        case GCQ_SFQ: return f(std::integral_constant<int, GCQ_SFQ>());
    }
    return GCQ_EINVAL;
}

inline uint64_t mix(uint64_t x) { return gcqi::splitmix64(x); }
inline double unit(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace

extern "C" {

// Seeded grid graph (the benchmark graphs; the reference's build_grid,
// bfs_bench.cpp:245-256, keeps every 4-neighbour edge and has no shortcuts):
// vertex r*C + c; each right and down edge kept with probability keep_p; from each
// vertex, with probability diag_p, one diagonal shortcut to (r+1, c-1) or (r+1, c+1).
// Undirected, no duplicates or self loops; CSR built with neighbours in ascending
// order.  Arrays are allocated with malloc and released with gcq_free.
int gcq_graph_grid(uint32_t rows, uint32_t cols, double keep_p, double diag_p, uint64_t seed,
                   int32_t** offsets, int32_t** indices, int32_t* V_out, int64_t* E_out) {
    if (!offsets || !indices || !V_out || !E_out || rows == 0 || cols == 0) return GCQ_EINVAL;
    const uint64_t V = (uint64_t)rows * cols;
    if (V >= (1ull << 31)) return GCQ_EINVAL;
    std::vector<std::pair<int32_t, int32_t>> und;   // each undirected edge once (u < v)
    und.reserve((size_t)(V * (2 * keep_p + diag_p) * 1.05) + 16);
    for (uint32_t r = 0; r < rows; ++r) {
        for (uint32_t c = 0; c < cols; ++c) {
            const int32_t u = (int32_t)(r * cols + c);
            const uint64_t h = mix(seed ^ ((uint64_t)u * 0x9E3779B97F4A7C15ull));
            if (c + 1 < cols && unit(mix(h ^ 1)) < keep_p) und.emplace_back(u, u + 1);
            if (r + 1 < rows && unit(mix(h ^ 2)) < keep_p) und.emplace_back(u, u + (int32_t)cols);
            if (r + 1 < rows && diag_p > 0 && unit(mix(h ^ 3)) < diag_p) {
                const bool left = (mix(h ^ 4) & 1) && c > 0;
                const bool right = !left && c + 1 < cols;
                if (left) und.emplace_back(u, u + (int32_t)cols - 1);
                else if (right) und.emplace_back(u, u + (int32_t)cols + 1);
            }
        }
    }
    std::vector<int32_t> deg(V, 0);
    for (auto& e : und) { deg[e.first]++; deg[e.second]++; }
    int32_t* off = (int32_t*)malloc((V + 1) * sizeof(int32_t));
    const int64_t E = (int64_t)und.size() * 2;
    int32_t* idx = (int32_t*)malloc((size_t)std::max<int64_t>(E, 1) * sizeof(int32_t));
    if (!off || !idx) { free(off); free(idx); return GCQ_ENOMEM; }
    off[0] = 0;
    for (uint64_t v = 0; v < V; ++v) off[v + 1] = off[v] + deg[v];
    std::vector<int32_t> cur(off, off + V);
    for (auto& e : und) {
        idx[cur[e.first]++] = e.second;
        idx[cur[e.second]++] = e.first;
    }
    for (uint64_t v = 0; v < V; ++v) std::sort(idx + off[v], idx + off[v + 1]);
    *offsets = off;
    *indices = idx;
    *V_out = (int32_t)V;
    *E_out = E;
    return GCQ_OK;
}

void gcq_free(void* p) { free(p); }

// Upload a CSR graph and create the two frontier queues (bfs_bench.cpp:702-737).
// Capacity: 2^capacity_log2 per queue (0 picks the smallest power of two >= V,
// at least 2^15, the reference's 32768); a frontier larger than the queue is an
// error, not a silent drop as in the reference (:380, :404, :475).
int gcq_bfs_create(int kind, const int32_t* offsets, const int32_t* indices, int32_t V, int64_t E,
                   uint32_t threads, uint32_t capacity_log2, const gcq_knobs* knobs, gcq_bfs_ctx** out) {
    if (!offsets || !indices || !out || V <= 0 || E < 0 || threads == 0 || (threads & 31)) return GCQ_EINVAL;
    *out = nullptr;
    if (capacity_log2 == 0) {
        // the whole graph (a frontier never holds more), and at least the thread
        // count, which G-WFQ requires (max_threads <= capacity, gwf_queue.hpp:320)
        capacity_log2 = 15;
        while ((1ull << capacity_log2) < (uint64_t)V && capacity_log2 < 26) ++capacity_log2;
        if (kind == GCQ_GWFQ)
            while ((1ull << capacity_log2) < (uint64_t)threads && capacity_log2 < 26) ++capacity_log2;
        if (kind == GCQ_SFQ)   // SFQ's MAX_ID envelope: L <= 2^32 / (threads + 1)
            while (capacity_log2 > 10 && (1ull << capacity_log2) > (1ull << 32) / ((uint64_t)threads + 1))
                --capacity_log2;
    }
    gcq_knobs k;
    if (knobs) k = *knobs; else gcq_default_knobs(&k);
    if (kind == GCQ_WFQ) {
        // The reference sizes the pool once per traversal from V and E
        // (wf_queue_host_init_for_bfs, :694-760), but every dequeue that finds the
        // queue empty also consumes cells, about levels * threads * (patience + 1)
        // per traversal, so high-diameter graphs exhaust it and lose vertices.
        // Here the drained input queue is reset after every level, so the pool only
        // has to hold one level: the frontier plus each thread's failed dequeues.
        const uint64_t per_thread = (uint64_t)V / threads + 2ull * (k.ymc_patience + 2);
        k.ymc_ops_per_thread = (uint32_t)std::max<uint64_t>(64, per_thread);
    }
    gcq_bfs_ctx* c = new gcq_bfs_ctx();
    c->kind = kind; c->V = V; c->E = E; c->threads = threads;
    int rc = gcq_create(kind, capacity_log2, threads, &k, &c->qa);
    if (rc == GCQ_OK) rc = gcq_create(kind, capacity_log2, threads, &k, &c->qb);
    auto fail = [&](int r) {
        if (c->qa) gcq_destroy(c->qa);
        if (c->qb) gcq_destroy(c->qb);
        cudaFree(c->d_off); cudaFree(c->d_idx); cudaFree(c->d_level); cudaFree(c->d_hubs); cudaFree(c->d_misc);
        if (c->h_misc) cudaFreeHost(c->h_misc);
        if (c->stream) cudaStreamDestroy(c->stream);
        delete c;
        return r;
    };
    if (rc != GCQ_OK) return fail(rc);
    if (cudaMalloc(&c->d_off, (size_t)(V + 1) * 4) != cudaSuccess ||
        cudaMalloc(&c->d_idx, (size_t)std::max<int64_t>(E, 1) * 4) != cudaSuccess ||
        cudaMalloc(&c->d_level, (size_t)V * 4) != cudaSuccess ||
        cudaMalloc(&c->d_hubs, (size_t)V * 4) != cudaSuccess || cudaMalloc(&c->d_misc, 256) != cudaSuccess ||
        cudaMallocHost(&c->h_misc, 256) != cudaSuccess)
        return fail(GCQ_ENOMEM);
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(GCQ_ECUDA);
    if (cudaMemcpy(c->d_off, offsets, (size_t)(V + 1) * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        (E > 0 && cudaMemcpy(c->d_idx, indices, (size_t)E * 4, cudaMemcpyHostToDevice) != cudaSuccess))
        return fail(GCQ_ECUDA);
    *out = c;
    return GCQ_OK;
}

int gcq_bfs_destroy(gcq_bfs_ctx* c) {
    if (!c) return GCQ_EINVAL;
    gcq_destroy(c->qa);
    gcq_destroy(c->qb);
    cudaFree(c->d_off); cudaFree(c->d_idx); cudaFree(c->d_level); cudaFree(c->d_hubs); cudaFree(c->d_misc);
    cudaFreeHost(c->h_misc);
    cudaStreamDestroy(c->stream);
    delete c;
    return GCQ_OK;
}

// One traversal from `src` (run_bfs, bfs_bench.cpp:509-633).  persistent = 0: one
// expand + hub launch pair per level and a host read of the next frontier size per
// level, as the reference does; persistent = 1: a single cooperative launch.
// host_levels (V int32, may be NULL) receives the depths (-1 = unreached).
int gcq_bfs_run(gcq_bfs_ctx* c, int32_t src, uint32_t block, int persistent, int32_t* host_levels,
                gcq_bfs_result* out) {
    if (!c || !out || block == 0 || block > 1024 || (block & 31) || c->threads % block) return GCQ_EINVAL;
    if (src < 0 || src >= c->V) return GCQ_EINVAL;
    memset(out, 0, sizeof(*out));
    cudaStream_t s = c->stream;
    using clk = std::chrono::steady_clock;
    const auto t_total = clk::now();
    bfs_misc* m = (bfs_misc*)c->d_misc;
    bfs_misc* hm = (bfs_misc*)c->h_misc;
    GCQ_CUDA(cudaMemsetAsync(c->d_level, 0xFF, (size_t)c->V * 4, s));
    GCQ_CUDA(cudaMemsetAsync(m, 0, 256, s));
    int rc = gcq_reset(c->qa, s);
    if (rc == GCQ_OK) rc = gcq_reset(c->qb, s);
    if (rc != GCQ_OK) return rc;
    if (persistent != 2)   // the asynchronous form queues its own (level, vertex) source item
        rc = dispatch(c->kind, [&](auto kc) {
            constexpr int K = decltype(kc)::value;
            k_bfs_source<K><<<1, 32, 0, s>>>(c->qa->obj, c->d_level, src, m);
            return GCQ_OK;
        });
    GCQ_CUDA(cudaGetLastError());
    GCQ_CUDA(cudaStreamSynchronize(s));
    out->init_ms = std::chrono::duration<double, std::milli>(clk::now() - t_total).count();
    cudaEvent_t e0, e1;
    GCQ_CUDA(cudaEventCreate(&e0));
    GCQ_CUDA(cudaEventCreate(&e1));
    const unsigned grid = c->threads / block;
    double kernel_ms = 0;
    unsigned int reached = 1, levels = 0, max_frontier = 1;
    if (!persistent) {
        void* qin = c->qa->obj;
        void* qout = c->qb->obj;
        for (int curr = 0;; ++curr) {
            cudaEventRecord(e0, s);
            rc = dispatch(c->kind, [&](auto kc) {
                constexpr int K = decltype(kc)::value;
                k_bfs_expand<K><<<grid, block, 0, s>>>(qin, qout, c->d_off, c->d_idx, c->d_level, curr, c->d_hubs, m);
                k_bfs_hubs<K><<<grid, block, 0, s>>>(qout, c->d_off, c->d_idx, c->d_level, curr, c->d_hubs, m);
                return GCQ_OK;
            });
            cudaEventRecord(e1, s);
            GCQ_CUDA(cudaMemcpyAsync(hm, m, 64, cudaMemcpyDeviceToHost, s));
            // reset the per-level counters for the next level
            GCQ_CUDA(cudaMemsetAsync(m, 0, 8, s));
            GCQ_CUDA(cudaStreamSynchronize(s));
            GCQ_CUDA(cudaGetLastError());
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            kernel_ms += ms;
            levels = curr + 1;
            const unsigned int next = hm->next_count;
            reached += next;
            max_frontier = std::max(max_frontier, next);
            if (hm->err || hm->drops) break;
            if (next == 0) break;
            // YMC only: the input queue is drained; recycle its cells (see gcq_bfs_create)
            if (c->kind == GCQ_WFQ) {
                rc = gcq_reset(qin == c->qa->obj ? c->qa : c->qb, s);
                if (rc != GCQ_OK) return rc;
            }
            std::swap(qin, qout);
        }
        out->edges_scanned = hm->edges;
    } else if (persistent == 2) {
        // asynchronous label-correcting form: G-WFQ and G-LFQ (64-bit items)
        if (c->kind != GCQ_GWFQ && c->kind != GCQ_GLFQ) return GCQ_EUNSUPPORTED;
        bfs_async_ctl* ac = (bfs_async_ctl*)((char*)c->d_misc + 128);
        bfs_async_ctl hac;
        memset(&hac, 0, sizeof hac);
        hac.timeout_ns = 5000000000ull;
        GCQ_CUDA(cudaMemcpyAsync(ac, &hac, sizeof hac, cudaMemcpyHostToDevice, s));
        cudaEventRecord(e0, s);
        rc = dispatch(c->kind, [&](auto kc) {
            constexpr int K = decltype(kc)::value;
            if constexpr (K == GCQ_GWFQ || K == GCQ_GLFQ) {
                k_bfs_async_source<K><<<1, 32, 0, s>>>(c->qa->obj, (unsigned int*)c->d_level, src, ac);
                k_bfs_set_deadline<<<1, 32, 0, s>>>(ac, 60000000000ull);
                k_bfs_async<K><<<grid, block, 0, s>>>(c->qa->obj, c->d_off, c->d_idx, (unsigned int*)c->d_level, ac);
            }
            return GCQ_OK;
        });
        cudaEventRecord(e1, s);
        k_bfs_summary<<<gcqi::grid_for((uint64_t)c->V, 256), 256, 0, s>>>(c->d_level, c->V, m);
        GCQ_CUDA(cudaMemcpyAsync(hm, m, 64, cudaMemcpyDeviceToHost, s));
        GCQ_CUDA(cudaMemcpyAsync(&hac, ac, sizeof hac, cudaMemcpyDeviceToHost, s));
        GCQ_CUDA(cudaStreamSynchronize(s));
        GCQ_CUDA(cudaGetLastError());
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        kernel_ms = ms;
        levels = hm->levels;
        reached = hm->reached;
        max_frontier = 0;
        out->edges_scanned = hac.edges;
        hm->err |= hac.err;
    } else {
        if (c->kind == GCQ_WFQ) return GCQ_EUNSUPPORTED;   // needs the per-level pool reset
        // cooperative launch: all blocks must be resident for the grid barrier
        const void* kern = nullptr;
        dispatch(c->kind, [&](auto kc) {
            constexpr int K = decltype(kc)::value;
            kern = (const void*)k_bfs_persistent<K>;
            return GCQ_OK;
        });
        uint64_t res = 0;
        rc = gcqi::resident_threads(kern, (int)block, 0, &res);
        if (rc != GCQ_OK) return rc;
        if (c->threads > res) return GCQ_EUNSUPPORTED;
        void* qa = c->qa->obj;
        void* qb = c->qb->obj;
        uint64_t tmo = 5000000000ull;
        void* args[] = {&qa, &qb, &c->d_off, &c->d_idx, &c->d_level, &c->d_hubs, &m, &tmo};
        cudaEventRecord(e0, s);
        GCQ_CUDA(cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(block), args, 0, s));
        cudaEventRecord(e1, s);
        GCQ_CUDA(cudaMemcpyAsync(hm, m, 64, cudaMemcpyDeviceToHost, s));
        GCQ_CUDA(cudaStreamSynchronize(s));
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        kernel_ms = ms;
        levels = hm->levels;
        reached = 1 + hm->reached;
        max_frontier = std::max(1u, hm->max_frontier);
        out->edges_scanned = hm->edges;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    out->kernel_ms = kernel_ms;
    out->levels = (int32_t)levels;
    out->reached = reached;
    out->max_frontier = max_frontier;
    out->drops = hm->drops;
    if (host_levels) GCQ_CUDA(cudaMemcpyAsync(host_levels, c->d_level, (size_t)c->V * 4, cudaMemcpyDeviceToHost, s));
    GCQ_CUDA(cudaStreamSynchronize(s));
    out->total_ms = std::chrono::duration<double, std::milli>(clk::now() - t_total).count();
    uint32_t e1w = 0, e2w = 0;
    GCQ_CUDA(cudaMemcpy(&e1w, c->qa->err, 4, cudaMemcpyDeviceToHost));
    GCQ_CUDA(cudaMemcpy(&e2w, c->qb->err, 4, cudaMemcpyDeviceToHost));
    const uint32_t err = e1w | e2w | hm->err;
    if (hm->drops) return GCQ_ECAPACITY;
    if (err & GCQ_ERR_TIMEOUT) return GCQ_ETIMEDOUT;
    if (err & (GCQ_ERR_SPIN | GCQ_ERR_TID)) return GCQ_EDEVICE;
    if (err & (GCQ_ERR_POOL | GCQ_ERR_CAPACITY)) return GCQ_ECAPACITY;
    return GCQ_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ RMAT graphs
extern "C" {

// Seeded R-MAT graph (Chakrabarti, Zhan & Faloutsos, SDM 2004): 2^scale vertices,
// edge_factor * 2^scale generated edges, each placed by descending `scale` levels of
// the adjacency matrix with quadrant probabilities a, b, c, 1-a-b-c.  Self loops and
// duplicates are removed; the result is undirected CSR with ascending neighbours.
// Built in parallel on the host cores: edges are generated per thread from the edge
// index (so the graph does not depend on the thread count), scattered into CSR, and
// every adjacency list is sorted and deduplicated.  The reference has no generator
// (it loads .mtx/SNAP files, bfs_bench.cpp:202-243).
int gcq_graph_rmat(uint32_t scale, uint32_t edge_factor, double a, double b, double c, uint64_t seed,
                   int32_t** offsets, int32_t** indices, int32_t* V_out, int64_t* E_out) {
    if (!offsets || !indices || !V_out || !E_out || scale < 1 || scale > 30 || edge_factor == 0) return GCQ_EINVAL;
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return GCQ_EINVAL;
    const uint64_t V = 1ull << scale;
    const uint64_t M = (uint64_t)edge_factor * V;
    const double ab = a + b, abc = a + b + c;
    const unsigned nth = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    auto par = [&](uint64_t n, auto&& body) {
        std::vector<std::thread> ts;
        for (unsigned t = 0; t < nth; ++t)
            ts.emplace_back([&, t]() { for (uint64_t i = n * t / nth; i < n * (t + 1) / nth; ++i) body(i); });
        for (auto& th : ts) th.join();
    };
    std::vector<uint32_t> eu(M), ev(M);
    par(M, [&](uint64_t e) {
        uint64_t u = 0, v = 0;
        uint64_t h = mix(seed * 0xD1B54A32D192ED03ull + e);
        for (uint32_t l = 0; l < scale; ++l) {
            h = mix(h + 0x9E3779B97F4A7C15ull);
            const double r = unit(h);
            const uint64_t bit = 1ull << (scale - 1 - l);
            if (r < a) {}
            else if (r < ab) v |= bit;
            else if (r < abc) u |= bit;
            else { u |= bit; v |= bit; }
        }
        eu[e] = (uint32_t)u;
        ev[e] = (uint32_t)v;
    });
    std::vector<std::atomic<int32_t>> deg(V);
    par(V, [&](uint64_t v) { deg[v].store(0, std::memory_order_relaxed); });
    par(M, [&](uint64_t e) {
        if (eu[e] == ev[e]) return;
        deg[eu[e]].fetch_add(1, std::memory_order_relaxed);
        deg[ev[e]].fetch_add(1, std::memory_order_relaxed);
    });
    std::vector<int64_t> start(V + 1, 0);
    for (uint64_t v = 0; v < V; ++v) start[v + 1] = start[v] + deg[v].load(std::memory_order_relaxed);
    std::vector<int32_t> adj((size_t)std::max<int64_t>(start[V], 1));
    std::vector<std::atomic<int64_t>> cur(V);
    par(V, [&](uint64_t v) { cur[v].store(start[v], std::memory_order_relaxed); });
    par(M, [&](uint64_t e) {
        if (eu[e] == ev[e]) return;
        adj[cur[eu[e]].fetch_add(1, std::memory_order_relaxed)] = (int32_t)ev[e];
        adj[cur[ev[e]].fetch_add(1, std::memory_order_relaxed)] = (int32_t)eu[e];
    });
    std::vector<int32_t> ndeg(V);
    par(V, [&](uint64_t v) {
        int32_t* b0 = adj.data() + start[v];
        int32_t* e0 = adj.data() + start[v + 1];
        std::sort(b0, e0);
        ndeg[v] = (int32_t)(std::unique(b0, e0) - b0);
    });
    int32_t* off = (int32_t*)malloc((V + 1) * sizeof(int32_t));
    if (!off) return GCQ_ENOMEM;
    off[0] = 0;
    for (uint64_t v = 0; v < V; ++v) off[v + 1] = off[v] + ndeg[v];
    const int64_t E = off[V];
    int32_t* idx = (int32_t*)malloc((size_t)std::max<int64_t>(E, 1) * sizeof(int32_t));
    if (!idx) { free(off); return GCQ_ENOMEM; }
    par(V, [&](uint64_t v) { std::copy(adj.data() + start[v], adj.data() + start[v] + ndeg[v], idx + off[v]); });
    *offsets = off; *indices = idx; *V_out = (int32_t)V; *E_out = E;
    return GCQ_OK;
}

}  // extern "C"
