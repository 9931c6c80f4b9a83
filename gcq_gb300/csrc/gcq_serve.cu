// Served and batched BFS: one persistent kernel serves a stream of traversal
// requests over several resident graphs.  The reference runs one traversal per
// process (bfs_bench.cpp:327-496, host loop per level); this engine keeps every
// graph resident and overlaps many traversals on one worklist.
//
// Pipeline (all device-side, all through G-WFQ queues):
//   arrivals   requests carry arrival times on the device clock (an open-loop
//              schedule made by the caller, sorted by arrival); lane 0 of any warp
//              that sees the next arrival due moves it into its graph's submission
//              queue
//   admission  per graph, a pool of level-array slots sized by the HBM budget; a
//              warp admits a request when it can take a free slot of that graph and
//              reserve V(graph) entries of worklist room (admission by footprint:
//              level arrays in the slot pools, worklist items in the reservation)
//   work       one shared worklist carries (slot, level, vertex) items of every
//              admitted traversal.  Each traversal is a label-correcting BFS: a
//              neighbour whose level drops (atomicMin) is enqueued, a dequeued item
//              whose vertex already has a smaller level is stale, so the final
//              levels are exact hop distances whatever the processing order
//   completion a per-traversal pending count reaching zero ends the traversal; the
//              count is settled once per item (children - 1), so an item with one
//              child costs no counter update.  The level array is then swept by
//              cleanup items that fold a checksum of the levels and reset them; the
//              last sweep publishes the result and returns the slot
// Vertices of degree > 32 and cleanup sweeps are processed by the whole warp.
//
// Ray tiles of the benchmark scenes (gcq_rt_bounce_render's scenes) are served by
// the same kernel and worklist: a tile request takes a slot of its scene (ray and
// path storage for one tile) and worklist room for one item per pixel; a warp
// writes the tile's primary rays and queues one item per pixel; an item traces one
// bounce of its pixel's path and re-queues itself while the path continues; the
// tile's pending count reaching zero schedules one sweep that folds a checksum of
// the tile's pixels and returns the slot.  The pixels equal gcq_rt_bounce_render's.
// Every wait is bounded: a full worklist or an idle loop gives up after the
// configured timeout and reports through the control block's error word.
#include <algorithm>
#include <cstring>
#include <vector>

#include "gcq_scene.cuh"

namespace {

using gcq::gwf::mpmc;

constexpr uint32_t UNVISITED = 0x7F7F7F7Fu;   // byte-settable, above any level
constexpr uint32_t SLOT_BITS = 14, LVL_BITS = 18;
constexpr uint32_t CLEANUP = (1u << LVL_BITS) - 1;    // level field of a sweep item
constexpr uint32_t RAY = CLEANUP - 1;                 // level field of a ray item (vertex field: pixel in tile)
constexpr uint32_t RAY_GEN = CLEANUP - 2;             // level field of a tile's generation item
constexpr uint32_t MAX_LEVEL = CLEANUP - 3;
constexpr uint32_t MAX_SLOTS = 1u << SLOT_BITS;
constexpr uint32_t SWEEP = 1u << 13;                  // vertices per sweep item
constexpr int WARP_DEG = 32;
// A vertex of more than HUB_DEG neighbours is expanded as chunk items of
// CHUNK_EDGES edges (vertex field | CHUNK_BIT, chunk index in the level field), so
// many warps share a hub; a chunk relaxes with the vertex's current level.
constexpr int HUB_DEG = 2048;
constexpr int CHUNK_EDGES = 1024;
constexpr uint32_t CHUNK_BIT = 1u << 31;
constexpr int MAX_GRAPHS = 64;
constexpr uint32_t MAX_REQ = 1u << 20;
constexpr uint64_t MAX_ARRIVAL_NS = 60000000000ull;   // schedules span at most a minute
constexpr unsigned FULL = 0xffffffffu;
constexpr uint32_t POLL_TRIES = 2;    // fast-path attempts per poll of a server queue
constexpr uint32_t POLL_MISSES = 8;   // polls of an unfilled head slot before a worker dequeues anyway
// Patience of the worklist by default: its enqueues retry on the fast path and the
// wait-free slow path is not entered in practice (see gcq_serve_default_cfg).
constexpr uint32_t SERVER_PATIENCE = 1u << 16;

// A scene served as tiles: the renderer's parameters and geometry, and the image.
struct srv_scene {
    bparams P;
    const BSphere* sph;
    const BQuad* quad;
    float* img;
    int32_t ns, nq, tiles, _pad;
};

// A target of requests: a graph (scene == nullptr) or a scene.  For a scene, V is
// the pixels of a tile (its worklist reservation) and sweeps is 1.
struct srv_graph {
    const int32_t* off;
    const int32_t* idx;
    mpmc* subq;        // submitted requests of this target (request index)
    mpmc* slotq;       // free slots of this target (global slot index)
    const srv_scene* scene;
    int32_t V;
    uint32_t slot0, nslots, sweeps;
};

struct srv_req { int32_t graph; int32_t src; uint64_t arrival_ns; };
struct srv_res { uint64_t admit_ns, done_ns, finish_ns, checksum; uint32_t reached; int32_t max_level; };

struct alignas(128) srv_slot {
    gcq::u64a pending;      // items of the traversal not yet settled
    gcq::u64a checksum;
    gcq::u32a reached;
    gcq::u32a max_level;
    gcq::u32a sweeps_left;
    int32_t req;
    int32_t graph;          // target index
    int32_t src;            // tile index of a tile request
    uint64_t done_ns;
    int32_t* level;         // UNVISITED everywhere while the slot is free
    BRay* rays;             // a tile slot's rays and path states, one per pixel
    BPix* pix;
};

struct alignas(128) srv_ctl {
    gcq::u32a next_release;   // next request index to release
    char _p0[124];
    gcq::u32a completed;
    char _p1[124];
    gcq::u64a reserved;       // worklist entries reserved by admitted traversals
    char _p2[120];
    gcq::u64a t0;             // device clock at the start of the run
    uint64_t timeout_ns;
    uint64_t deadline_ns;     // the run gives up (ERR_TIMEOUT) after this, from t0
    uint64_t work_limit;      // reservations may not exceed this
    gcq::u32a err;
    uint32_t nreq;
    uint32_t ngraphs;
    uint32_t _pad;
    gcq::u64a stat[4];        // items, stale items, edges scanned, sweeps
    gcq::u64a stat2[4];       // rays traced
};

enum { ST_ITEMS, ST_STALE, ST_EDGES, ST_SWEEPS };
enum { ST_RAYS = 0 };   // index into srv_ctl::stat2

struct srv_ctx {
    mpmc* workq;
    srv_slot* slots;
    const srv_graph* graphs;
    const srv_req* reqs;
    srv_res* res;
    srv_ctl* ctl;
};

__device__ __forceinline__ uint64_t pack_item(uint32_t slot, uint32_t lvl, uint32_t v) {
    return ((uint64_t)slot << (32 + LVL_BITS)) | ((uint64_t)lvl << 32) | v;
}
__device__ __forceinline__ uint32_t item_slot(uint64_t x) { return (uint32_t)(x >> (32 + LVL_BITS)); }
__device__ __forceinline__ uint32_t item_lvl(uint64_t x) { return (uint32_t)(x >> 32) & CLEANUP; }
__device__ __forceinline__ uint32_t item_v(uint64_t x) { return (uint32_t)x; }

// Checksum of a traversal: sum (mod 2^64) over all vertices v of the graph of
// splitmix64(v << 32 | level(v)), level 0xFFFFFFFF for unreached vertices.
__device__ __forceinline__ uint64_t level_term(uint32_t v, uint32_t lvl) {
    return gcqi::splitmix64(((uint64_t)v << 32) | lvl);
}

// Checksum of a tile: sum (mod 2^64) over its pixels g (row-major in the image) and
// channels c of splitmix64((3g + c) << 32 | bits of the channel's float).
__device__ __forceinline__ uint64_t pixel_term(uint32_t g, int c, float v) {
    return gcqi::splitmix64(((uint64_t)(3u * g + (uint32_t)c) << 32) | (uint64_t)__float_as_uint(v));
}

__device__ __forceinline__ uint64_t now_ns(const srv_ctx& x) {
    return gcq::globaltimer_ns() - gcq::ld_rlx(&x.ctl->t0);
}

// Enqueue a work item; a full worklist is waited out (bounded), never dropped.
__device__ __forceinline__ void push_item(const srv_ctx& x, uint64_t it, uint32_t tid) {
    if (gcq::gwf::enqueue_ptr(x.workq, it, tid)) return;
    gcq::backoff bo;
    const uint64_t t0 = gcq::globaltimer_ns();
    do {
        if (gcq::globaltimer_ns() - t0 > x.ctl->timeout_ns) {
            gcq::raise_error(&x.ctl->err, gcq::ERR_CAPACITY);
            return;
        }
        bo.pause(2048);
    } while (!gcq::gwf::enqueue_ptr(x.workq, it, tid));
}

// The traversal in `slot` has no pending item: record the time, give back the
// worklist reservation and schedule the sweeps over its level array.
__device__ __noinline__ void traversal_done(const srv_ctx& x, uint32_t slot, uint32_t tid) {
    srv_slot* s = &x.slots[slot];
    const srv_graph& g = x.graphs[s->graph];
    s->done_ns = now_ns(x);
    gcq::fetch_add(&x.ctl->reserved, (uint64_t)0 - (uint64_t)g.V);
    gcq::st_rel(&s->sweeps_left, g.sweeps);
    for (uint32_t k = 0; k < g.sweeps; ++k) push_item(x, pack_item(slot, CLEANUP, k), tid);
}

// Settle one processed item that produced `children` new items (already counted
// for warp-wide expansions: pass children = 0 there after adding them).
__device__ __forceinline__ void settle(const srv_ctx& x, uint32_t slot, uint32_t children, uint32_t tid) {
    if (children == 1) return;   // the child inherits the item's count
    const uint64_t prev = gcq::fetch_add(&x.slots[slot].pending, (uint64_t)children - 1);
    if (children == 0 && prev == 1) traversal_done(x, slot, tid);
}

// Reserve `v` worklist entries if they fit under the limit.  A compare-and-swap
// that only ever adds what fits: an add-then-roll-back reservation livelocks when
// many control lanes overshoot the limit together and all of them roll back.
__device__ __forceinline__ bool reserve(srv_ctl* c, uint64_t v) {
    uint64_t cur = gcq::ld_rlx(&c->reserved);
    for (int k = 0; k < 8; ++k) {
        if (cur + v > c->work_limit) return false;
        const uint64_t seen = gcq::cas(&c->reserved, cur, cur + v);
        if (seen == cur) return true;
        cur = seen;
    }
    return false;
}

// Release due arrivals into their submission queues, then admit what fits.
// Called by lane 0 of a warp; `ctid` (the warp index) is its identity on the
// control queues.
__device__ __noinline__ void control(const srv_ctx& x, uint32_t ctid, uint32_t turn) {
    srv_ctl* c = x.ctl;
    const uint32_t nreq = c->nreq;
    for (int k = 0; k < 4; ++k) {
        const uint32_t i = gcq::ld_acq(&c->next_release);
        if (i >= nreq || x.reqs[i].arrival_ns > now_ns(x)) break;
        if (gcq::cas(&c->next_release, i, i + 1) == i)
            gcq::gwf::enqueue_ptr(x.graphs[x.reqs[i].graph].subq, i, ctid);
    }
    const uint32_t ng = c->ngraphs;
    int admitted = 0;
    for (uint32_t k = 0; k < ng && admitted < 2; ++k) {
        const uint32_t gi = (turn + ctid + k) % ng;
        const srv_graph& g = x.graphs[gi];
        // nothing submitted, or no free slot: read-only checks, no ticket taken
        if (!gcq::gwf::maybe_nonempty(&g.subq->aq) || !gcq::gwf::maybe_nonempty(&g.slotq->aq)) continue;
        const uint64_t V = (uint64_t)g.V;
        if (!reserve(c, V)) continue;
        uint64_t slot = 0, r = 0;
        if (!gcq::gwf::try_dequeue_ptr(g.slotq, &slot, ctid, POLL_TRIES)) {
            gcq::fetch_add(&c->reserved, (uint64_t)0 - V);
            continue;
        }
        if (!gcq::gwf::try_dequeue_ptr(g.subq, &r, ctid, POLL_TRIES)) {
            gcq::gwf::enqueue_ptr(g.slotq, slot, ctid);
            gcq::fetch_add(&c->reserved, (uint64_t)0 - V);
            continue;
        }
        srv_slot* s = &x.slots[slot];
        const int32_t src = x.reqs[r].src;
        s->req = (int32_t)r;
        s->graph = (int32_t)gi;
        s->src = src;
        gcq::st_rlx(&s->checksum, 0ull);
        gcq::st_rlx(&s->reached, 0u);
        gcq::st_rlx(&s->max_level, 0u);
        gcq::st_rlx(&s->pending, 1ull);
        x.res[r].admit_ns = now_ns(x);
        if (g.scene) {
            push_item(x, pack_item((uint32_t)slot, RAY_GEN, 0), ctid << 5);   // release publishes the slot
        } else {
            s->level[src] = 0;
            push_item(x, pack_item((uint32_t)slot, 0, (uint32_t)src), ctid << 5);
        }
        ++admitted;
    }
}

// One bounce of the path of pixel `i` of the tile in `slot`: the item re-queues
// itself while the path continues; a finished path writes its pixel, adds its rays
// to the tile's count and settles the item.
__device__ __noinline__ void serve_ray(const srv_ctx& x, uint64_t it, uint32_t slot, uint32_t i, uint32_t tid) {
    srv_slot* s = &x.slots[slot];
    const srv_scene* sc = x.graphs[s->graph].scene;
    BRay r = s->rays[i];
    BPix st = s->pix[i];
    const BHit hit = btrace(r, sc->sph, sc->ns, sc->quad, sc->nq);
    V3 c;
    if (bshade(r, st, hit, sc->P, &c)) {
        s->rays[i] = r;
        s->pix[i] = st;
        push_item(x, it, tid);   // the child inherits the item's count
        return;
    }
    float* o = sc->img + 3 * (size_t)r.pix;
    o[0] = c.x; o[1] = c.y; o[2] = c.z;
    atomicAdd((unsigned int*)&s->reached, r.depth + 1);
    atomicMax((unsigned int*)&s->max_level, r.depth + 1);
    settle(x, slot, 0, tid);
}

__global__ void __launch_bounds__(256, 3) k_serve(srv_ctx x) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t ctid = tid >> 5;
    const int lane = (int)(threadIdx.x & 31);
    srv_ctl* c = x.ctl;
    const uint32_t nreq = c->nreq;
    uint64_t n_items = 0, n_stale = 0, n_edges = 0, n_sweeps = 0, n_rays = 0;
    // stall detection: progress is any enqueue on the worklist (its Tail counter) or
    // a completion; one thread going without an item proves nothing
    uint64_t idle_since = 0, idle_mark = 0;
    uint32_t poll_misses = 0;
    gcq::backoff bo;
    for (uint32_t iter = 0;; ++iter) {
        uint32_t stop = 0;
        if (lane == 0) {
            stop = (gcq::ld_acq(&c->completed) >= nreq || gcq::ld_rlx(&c->err)) ? 1u : 0u;
            if (!stop && now_ns(x) > c->deadline_ns) {
                gcq::raise_error(&c->err, gcq::ERR_TIMEOUT);   // whole-run bound
                stop = 1;
            }
            if (!stop && (iter & 3) == 0) control(x, ctid, iter >> 2);
        }
        if (__shfl_sync(FULL, stop, 0)) break;

        uint64_t it = 0;
        // idle lanes poll through read-only hints: an empty worklist costs them two
        // loads, not a Head ticket and a marked slot each; and a Head ticket is taken
        // only once the head slot holds an entry (head_ready), or after POLL_MISSES
        // polls that saw Tail ahead with the head slot unfilled
        bool ready = false;
        if (gcq::gwf::maybe_nonempty(&x.workq->aq))
            ready = gcq::gwf::head_ready(&x.workq->aq) || ++poll_misses >= POLL_MISSES;
        const bool got = ready && gcq::gwf::try_dequeue_ptr(x.workq, &it, tid, POLL_TRIES);
        if (ready) poll_misses = 0;
        // 1: an edge range of one vertex (lvl = the level it gives), 2: a cleanup sweep,
        // 3: a tile's primary rays
        int big = 0;
        uint32_t slot = 0, lvl = 0, v = 0;
        int rb = 0, re = 0;
        if (got) {
            slot = item_slot(it);
            lvl = item_lvl(it);
            v = item_v(it);
            if (lvl == CLEANUP) {
                big = 2;
            } else if (lvl == RAY) {
                ++n_rays;
                serve_ray(x, it, slot, v, tid);
            } else if (lvl == RAY_GEN) {
                big = 3;
            } else if (v & CHUNK_BIT) {
                ++n_items;
                srv_slot* s = &x.slots[slot];
                const srv_graph& g = x.graphs[s->graph];
                const uint32_t u = v & ~CHUNK_BIT;
                rb = g.off[u] + (int)lvl * CHUNK_EDGES;
                re = min(g.off[u + 1], rb + CHUNK_EDGES);
                lvl = (uint32_t)gcq::ld_rlx((const int*)&s->level[u]) + 1;
                big = 1;
            } else {
                ++n_items;
                srv_slot* s = &x.slots[slot];
                int32_t* level = s->level;
                if ((uint32_t)gcq::ld_rlx((const int*)&level[v]) < lvl) {
                    ++n_stale;   // a shorter path reached v after this item was queued
                    settle(x, slot, 0, tid);
                } else {
                    const srv_graph& g = x.graphs[s->graph];
                    const int beg = g.off[v], end = g.off[v + 1];
                    if (end - beg > HUB_DEG) {
                        const uint32_t chunks = (uint32_t)((end - beg + CHUNK_EDGES - 1) / CHUNK_EDGES);
                        if (chunks >= CLEANUP) {
                            gcq::raise_error(&c->err, gcq::ERR_CAPACITY);
                            settle(x, slot, 0, tid);
                        } else {
                            // the chunks inherit this item's count
                            gcq::fetch_add(&s->pending, (uint64_t)chunks - 1);
                            for (uint32_t k = 0; k < chunks; ++k) push_item(x, pack_item(slot, k, v | CHUNK_BIT), tid);
                        }
                    } else if (end - beg > WARP_DEG) {
                        rb = beg;
                        re = end;
                        lvl = lvl + 1;
                        big = 1;
                    } else {
                        n_edges += (uint64_t)(end - beg);
                        const uint32_t lv = lvl + 1;
                        uint32_t won = 0;
                        if (lv > MAX_LEVEL) {
                            if (end > beg) gcq::raise_error(&c->err, gcq::ERR_CAPACITY);
                        } else {
                            for (int e = beg; e < end; ++e) {
                                const uint32_t w = (uint32_t)g.idx[e];
                                if ((uint32_t)atomicMin(&level[w], (int)lv) > lv) won |= 1u << (e - beg);
                            }
                        }
                        const uint32_t kids = (uint32_t)__popc(won);
                        if (kids > 1) gcq::fetch_add(&s->pending, (uint64_t)kids - 1);
                        for (uint32_t m = won; m; m &= m - 1)
                            push_item(x, pack_item(slot, lv, (uint32_t)g.idx[beg + __ffs(m) - 1]), tid);
                        if (kids == 0) settle(x, slot, 0, tid);
                    }
                }
            }
        }
        // warp-wide work, one owner lane at a time
        for (;;) {
            const unsigned want = __ballot_sync(FULL, big != 0);
            if (want == 0) break;
            const int owner = __ffs(want) - 1;
            const int kind = __shfl_sync(FULL, big, owner);
            const uint32_t os = __shfl_sync(FULL, slot, owner);
            const uint32_t ol = __shfl_sync(FULL, lvl, owner);
            const uint32_t ov = __shfl_sync(FULL, v, owner);
            const int beg = __shfl_sync(FULL, rb, owner), end = __shfl_sync(FULL, re, owner);
            srv_slot* s = &x.slots[os];
            const srv_graph& g = x.graphs[s->graph];
            int32_t* level = s->level;
            if (kind == 3) {
                // primary rays of the tile, one item per pixel
                const srv_scene* sc = g.scene;
                const bparams& P = sc->P;
                const int tile = s->src;
                const int x0 = (tile % P.tiles_x) * P.tile_w, y0 = (tile / P.tiles_x) * P.tile_h;
                const int tw = min(P.tile_w, P.img_w - x0), th = min(P.tile_h, P.img_h - y0);
                const int npx = tw * th;
                // count the children before any of them can be dequeued
                if (lane == owner) gcq::fetch_add(&s->pending, (uint64_t)npx);
                __syncwarp();
                for (int i = lane; i < npx; i += 32) {
                    const int px = x0 + i % tw, py = y0 + i / tw;
                    BRay r;
                    BPix st;
                    bprimary(P, px, py, (uint32_t)(py * P.img_w + px), &r, &st);
                    s->rays[i] = r;
                    s->pix[i] = st;
                    push_item(x, pack_item(os, RAY, (uint32_t)i), tid);
                }
                __syncwarp();
                if (lane == owner) settle(x, os, 0, tid);
            } else if (kind == 1) {
                const uint32_t lv = ol;   // the level this range's neighbours get
                if (lane == owner) n_edges += (uint64_t)(end - beg);
                if (lv > MAX_LEVEL) {
                    if (lane == owner) gcq::raise_error(&c->err, gcq::ERR_CAPACITY);
                } else {
                    for (int base = beg; base < end; base += 32) {
                        const int e = base + lane;
                        uint32_t w = 0;
                        bool won = false;
                        if (e < end) {
                            w = (uint32_t)g.idx[e];
                            won = (uint32_t)atomicMin(&level[w], (int)lv) > lv;
                        }
                        const unsigned wm = __ballot_sync(FULL, won);
                        // count the children before any of them can be dequeued
                        if (lane == owner && wm) gcq::fetch_add(&s->pending, (uint64_t)__popc(wm));
                        __syncwarp();
                        if (won) push_item(x, pack_item(os, lv, w), tid);
                    }
                }
                if (lane == owner) settle(x, os, 0, tid);
            } else {
                uint64_t sum = 0;
                uint32_t reached = 0, maxl = 0;
                if (g.scene) {
                    // a finished tile: checksum of its pixels (rays and path lengths are
                    // already counted)
                    const bparams& P = g.scene->P;
                    const float* img = g.scene->img;
                    const int tile = s->src;
                    const int x0 = (tile % P.tiles_x) * P.tile_w, y0 = (tile / P.tiles_x) * P.tile_h;
                    const int tw = min(P.tile_w, P.img_w - x0), th = min(P.tile_h, P.img_h - y0);
                    for (int i = lane; i < tw * th; i += 32) {
                        const uint32_t px = (uint32_t)((y0 + i / tw) * P.img_w + (x0 + i % tw));
                        for (int ch = 0; ch < 3; ++ch) sum += pixel_term(px, ch, img[3 * (size_t)px + ch]);
                    }
                } else {
                    // sweep ov: checksum and reset vertices [ov * SWEEP, +SWEEP)
                    const uint32_t lo = ov * SWEEP;
                    const uint32_t hi = min((uint32_t)g.V, lo + SWEEP);
                    for (uint32_t u = lo + (uint32_t)lane; u < hi; u += 32) {
                        const uint32_t l = (uint32_t)level[u];
                        const bool r = (l != UNVISITED);
                        sum += level_term(u, r ? l : 0xFFFFFFFFu);
                        reached += r ? 1u : 0u;
                        maxl = (r && l > maxl) ? l : maxl;
                        level[u] = (int32_t)UNVISITED;
                    }
                }
                for (int o = 16; o > 0; o >>= 1) {
                    sum += __shfl_xor_sync(FULL, sum, o);
                    reached += __shfl_xor_sync(FULL, reached, o);
                    maxl = max(maxl, __shfl_xor_sync(FULL, maxl, o));
                }
                if (lane == owner) {
                    ++n_sweeps;
                    atomicAdd((unsigned long long*)&s->checksum, (unsigned long long)sum);
                    atomicAdd((unsigned int*)&s->reached, reached);
                    atomicMax((unsigned int*)&s->max_level, maxl);
                    if (gcq::fetch_add(&s->sweeps_left, (uint32_t)-1) == 1) {
                        // last sweep: publish the result, return the slot
                        const int32_t r = s->req;
                        srv_res out;
                        out.admit_ns = x.res[r].admit_ns;
                        out.done_ns = s->done_ns;
                        out.finish_ns = now_ns(x);
                        out.checksum = gcq::ld_acq(&s->checksum);
                        out.reached = gcq::ld_acq(&s->reached);
                        out.max_level = (int32_t)gcq::ld_acq(&s->max_level);
                        x.res[r] = out;
                        gcq::gwf::enqueue_ptr(g.slotq, os, ctid);
                        gcq::fetch_add(&c->completed, 1u);
                    }
                }
            }
            if (lane == owner) big = 0;
        }

        if (got) {
            bo = gcq::backoff();
            idle_since = 0;
        } else {
            const uint64_t t = gcq::globaltimer_ns();
            const uint64_t mark = gcq::ld_rlx(&x.workq->aq.Tail) + gcq::ld_rlx(&c->completed);
            if (idle_since == 0 || mark != idle_mark) {
                idle_since = t;
                idle_mark = mark;
            } else if (t - idle_since > c->timeout_ns && gcq::ld_rlx(&c->next_release) >= nreq) {
                gcq::raise_error(&c->err, gcq::ERR_TIMEOUT);   // no progress anywhere: stuck
            }
            bo.pause(1024);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        n_items += __shfl_xor_sync(FULL, n_items, o);
        n_stale += __shfl_xor_sync(FULL, n_stale, o);
        n_edges += __shfl_xor_sync(FULL, n_edges, o);
        n_sweeps += __shfl_xor_sync(FULL, n_sweeps, o);
        n_rays += __shfl_xor_sync(FULL, n_rays, o);
    }
    if (lane == 0) {
        gcq::fetch_add_rlx(&c->stat[ST_ITEMS], n_items);
        gcq::fetch_add_rlx(&c->stat[ST_STALE], n_stale);
        gcq::fetch_add_rlx(&c->stat[ST_EDGES], n_edges);
        gcq::fetch_add_rlx(&c->stat[ST_SWEEPS], n_sweeps);
        if (n_rays) gcq::fetch_add_rlx(&c->stat2[ST_RAYS], n_rays);
    }
}

// Fill a graph's slot queue with its slot indices; tid < n <= the queue's threads.
__global__ void k_fill_slots(mpmc* q, uint32_t slot0, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) gcq::gwf::enqueue_ptr(q, slot0 + i, i);
}

__global__ void k_stamp_t0(srv_ctl* c) {
    if (threadIdx.x == 0 && blockIdx.x == 0) gcq::st_rel(&c->t0, gcq::globaltimer_ns());
}

// A CSR the kernel can index without bounds checks: offsets start at 0, never
// decrease and end at E; every neighbour is a vertex.
bool valid_csr(const int32_t* off, const int32_t* idx, int32_t V, int64_t E) {
    if (off[0] != 0 || (int64_t)off[V] != E) return false;
    for (int32_t v = 0; v < V; ++v)
        if (off[v + 1] < off[v]) return false;
    for (int64_t e = 0; e < E; ++e)
        if (idx[e] < 0 || idx[e] >= V) return false;
    return true;
}

uint32_t log2_ceil(uint64_t n) {
    uint32_t b = 0;
    while ((1ull << b) < n) ++b;
    return b;
}

}  // namespace

struct gcq_server {
    std::vector<srv_graph> graphs;     // targets: the graphs, then the scenes
    int ngraphs = 0, nscenes = 0;
    std::vector<float*> scene_img;
    std::vector<uint64_t> scene_px;
    std::vector<int32_t> scene_tiles;
    std::vector<void*> dev;            // device allocations
    std::vector<gcq_queue*> queues;    // workq first, then subq/slotq per graph
    srv_graph* d_graphs = nullptr;
    srv_slot* d_slots = nullptr;
    int32_t* d_levels = nullptr;
    uint64_t level_bytes = 0;
    srv_ctl* d_ctl = nullptr;
    uint32_t total_slots = 0, threads = 0, block = 256, grid = 0;
    uint64_t timeout_ns = 0, run_limit_ns = 0, work_cap = 0;
    bool dirty = false;                // level arrays need a reset before the next run
    ~gcq_server() {
        for (gcq_queue* q : queues) gcq_destroy(q);
        for (void* p : dev) cudaFree(p);
    }
};

namespace {
template <typename T>
int dev_alloc(gcq_server* s, T** p, size_t bytes) {
    if (cudaMalloc((void**)p, bytes) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return GCQ_ENOMEM;
    }
    s->dev.push_back(*p);
    return GCQ_OK;
}
}  // namespace

extern "C" {

void gcq_serve_default_cfg(gcq_serve_cfg* c) {
    if (!c) return;
    memset(c, 0, sizeof *c);
    c->budget_bytes = 150ull << 30;
    c->timeout_ns = 10000000000ull;
    c->run_limit_ns = 60000000000ull;
    c->max_slots = 1024;
    // The server polls its worklist from every resident thread; its workers take a
    // Head ticket only once the head slot holds an entry (gwf::head_ready), so a
    // slow-path enqueue's tickets are not lost to a crowd of pollers marking them
    // first.  With that hint the reference's patience (128 / 256, wait-free slow
    // path reachable) serves the benchmark mix on 65536 workers (317-329 against
    // 358-364 traversals/s here), but with every resident thread (~117 K) polling, a
    // slow-path request still stalls past the server's bound.  The default keeps
    // every operation on the fast path; callers choose the reference's patience
    // through work_knobs.
    gcq_default_knobs(&c->work_knobs);
    c->work_knobs.enq_patience = SERVER_PATIENCE;
    c->work_knobs.deq_patience = SERVER_PATIENCE;
    c->threads = 0;
    c->work_log2 = 0;
    c->rt_scenes = 0;
    c->rt_width = c->rt_height = 1024;
    c->rt_tile_px = 32;
    c->rt_max_bounces = 4;
    c->rt_slots = 1024;
    c->rt_seed = 1;
}

int gcq_serve_create(int ngraphs, const int32_t* const* offsets, const int32_t* const* indices,
                     const int32_t* V, const int64_t* E, const gcq_serve_cfg* cfg, gcq_server** out) {
    if (!out) return GCQ_EINVAL;
    *out = nullptr;
    if (!cfg || ngraphs < 0 || ngraphs > MAX_GRAPHS || (ngraphs > 0 && (!offsets || !indices || !V || !E)))
        return GCQ_EINVAL;
    if (ngraphs == 0 && cfg->rt_scenes == 0) return GCQ_EINVAL;
    if (cfg->rt_scenes > 2) return GCQ_EINVAL;
    if (cfg->rt_scenes && (cfg->rt_width == 0 || cfg->rt_height == 0 || cfg->rt_tile_px == 0 ||
                           cfg->rt_tile_px > 256 || cfg->rt_max_bounces > 1000 || cfg->rt_slots == 0 ||
                           (uint64_t)cfg->rt_width * cfg->rt_height > (1ull << 30)))
        return GCQ_EINVAL;
    if (ngraphs + (int)cfg->rt_scenes > MAX_GRAPHS) return GCQ_EINVAL;
    gcq_server* s = new gcq_server();
    auto fail = [&](int r) { delete s; return r; };
    int rc = GCQ_OK;
    int32_t maxV = 0;
    for (int g = 0; g < ngraphs; ++g) {
        if (!offsets[g] || V[g] <= 0 || V[g] >= INT32_MAX || E[g] < 0 || E[g] > INT32_MAX ||
            (E[g] > 0 && !indices[g]) || !valid_csr(offsets[g], indices[g], V[g], E[g]))
            return fail(GCQ_EINVAL);
        maxV = std::max(maxV, V[g]);
    }
    // persistent grid: every block resident
    s->block = 256;
    uint64_t res = 0;
    if ((rc = gcqi::resident_threads((const void*)k_serve, (int)s->block, 0, &res)) != GCQ_OK) return fail(rc);
    uint64_t threads = cfg->threads ? std::min<uint64_t>(cfg->threads, res) : res;
    threads = threads / s->block * s->block;
    if (threads == 0) return fail(GCQ_EINVAL);
    s->threads = (uint32_t)threads;
    s->grid = (uint32_t)(threads / s->block);
    s->timeout_ns = cfg->timeout_ns ? cfg->timeout_ns : 10000000000ull;
    s->run_limit_ns = cfg->run_limit_ns ? cfg->run_limit_ns : 60000000000ull;
    // slot pools: an even share of the budget per graph, at most max_slots each
    const uint32_t ntargets = (uint32_t)ngraphs + cfg->rt_scenes;
    const uint32_t per_graph_cap =
        std::min<uint32_t>(cfg->max_slots ? cfg->max_slots : 1024, MAX_SLOTS / ntargets);
    const uint64_t share = cfg->budget_bytes / (uint64_t)ntargets;
    uint64_t level_elems = 0;
    uint32_t ctl_threads = (uint32_t)(threads / 32);
    for (int g = 0; g < ngraphs; ++g) {
        const uint64_t bytes = (uint64_t)V[g] * 4;
        const uint32_t n = (uint32_t)std::min<uint64_t>(per_graph_cap, share / bytes);
        if (n == 0) return fail(GCQ_ECAPACITY);   // not even one level array fits the share
        srv_graph hg{};
        hg.V = V[g];
        hg.slot0 = s->total_slots;
        hg.nslots = n;
        hg.sweeps = (uint32_t)(((uint64_t)V[g] + SWEEP - 1) / SWEEP);
        s->total_slots += n;
        level_elems += (uint64_t)n * (uint64_t)V[g];
        ctl_threads = std::max(ctl_threads, n);
        s->graphs.push_back(hg);
    }
    // scenes: a tile slot holds a 32-byte ray and a 16-byte path state per pixel
    const uint32_t tile_px2 = cfg->rt_tile_px * cfg->rt_tile_px;
    uint64_t tile_elems = 0;
    for (uint32_t sc = 0; sc < cfg->rt_scenes; ++sc) {
        const uint64_t bytes = (uint64_t)tile_px2 * (sizeof(BRay) + sizeof(BPix));
        const uint32_t n = (uint32_t)std::min<uint64_t>(std::min<uint32_t>(cfg->rt_slots, MAX_SLOTS / ntargets),
                                                        share / bytes);
        if (n == 0) return fail(GCQ_ECAPACITY);
        srv_graph hg{};
        hg.V = (int32_t)tile_px2;
        hg.slot0 = s->total_slots;
        hg.nslots = n;
        hg.sweeps = 1;
        s->total_slots += n;
        tile_elems += (uint64_t)n * tile_px2;
        ctl_threads = std::max(ctl_threads, n);
        s->graphs.push_back(hg);
        maxV = std::max(maxV, (int32_t)tile_px2);
    }
    s->ngraphs = ngraphs;
    s->nscenes = (int)cfg->rt_scenes;
    for (uint32_t sc = 0; sc < cfg->rt_scenes; ++sc) {
        srv_scene hs{};
        memset(&hs, 0, sizeof hs);
        bparams& P = hs.P;
        P.img_w = (int)cfg->rt_width;
        P.img_h = (int)cfg->rt_height;
        P.tile_w = P.tile_h = (int)cfg->rt_tile_px;
        P.tiles_x = (P.img_w + P.tile_w - 1) / P.tile_w;
        P.threads_per_tile = 0;
        P.max_depth = (int)cfg->rt_max_bounces;
        P.seed = cfg->rt_seed;
        std::vector<BSphere> sph;
        std::vector<BQuad> quad;
        build_bscene((int)sc, cfg->rt_seed, sph, quad, P);
        hs.ns = (int32_t)sph.size();
        hs.nq = (int32_t)quad.size();
        hs.tiles = P.tiles_x * ((P.img_h + P.tile_h - 1) / P.tile_h);
        BSphere* d_sph = nullptr;
        BQuad* d_quad = nullptr;
        float* d_img = nullptr;
        srv_scene* d_sc = nullptr;
        const size_t img_bytes = (size_t)P.img_w * P.img_h * 12;
        if ((rc = dev_alloc(s, &d_sph, std::max<size_t>(1, sph.size()) * sizeof(BSphere))) != GCQ_OK ||
            (rc = dev_alloc(s, &d_quad, std::max<size_t>(1, quad.size()) * sizeof(BQuad))) != GCQ_OK ||
            (rc = dev_alloc(s, &d_img, img_bytes)) != GCQ_OK || (rc = dev_alloc(s, &d_sc, sizeof(srv_scene))) != GCQ_OK)
            return fail(rc);
        hs.sph = d_sph;
        hs.quad = d_quad;
        hs.img = d_img;
        if ((!sph.empty() && cudaMemcpy(d_sph, sph.data(), sph.size() * sizeof(BSphere), cudaMemcpyHostToDevice) != cudaSuccess) ||
            (!quad.empty() && cudaMemcpy(d_quad, quad.data(), quad.size() * sizeof(BQuad), cudaMemcpyHostToDevice) != cudaSuccess) ||
            cudaMemset(d_img, 0, img_bytes) != cudaSuccess ||
            cudaMemcpy(d_sc, &hs, sizeof hs, cudaMemcpyHostToDevice) != cudaSuccess)
            return fail(gcqi::cuda_fail(cudaGetLastError(), "scene upload", __FILE__, __LINE__));
        s->graphs[ngraphs + sc].scene = d_sc;
        s->scene_img.push_back(d_img);
        s->scene_px.push_back((uint64_t)P.img_w * P.img_h);
        s->scene_tiles.push_back(hs.tiles);
    }
    // graphs
    for (int g = 0; g < ngraphs; ++g) {
        int32_t* d_off = nullptr;
        int32_t* d_idx = nullptr;
        if ((rc = dev_alloc(s, &d_off, (size_t)(V[g] + 1) * 4)) != GCQ_OK) return fail(rc);
        if ((rc = dev_alloc(s, &d_idx, (size_t)std::max<int64_t>(E[g], 1) * 4)) != GCQ_OK) return fail(rc);
        if (cudaMemcpy(d_off, offsets[g], (size_t)(V[g] + 1) * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
            (E[g] > 0 && cudaMemcpy(d_idx, indices[g], (size_t)E[g] * 4, cudaMemcpyHostToDevice) != cudaSuccess))
            return fail(gcqi::cuda_fail(cudaGetLastError(), "graph upload", __FILE__, __LINE__));
        s->graphs[g].off = d_off;
        s->graphs[g].idx = d_idx;
    }
    // queues: the worklist holds at least twice the largest graph and every thread;
    // control queues are used by one lane per warp (identity = warp index)
    gcq_knobs k = cfg->work_knobs;   // the control queues follow the worklist's knobs
    // reservations may reach half the worklist, and that half holds two traversals
    // of the largest graph, so no graph waits for the worklist to drain completely
    uint32_t work_log2 = cfg->work_log2 ? cfg->work_log2 : 25;
    work_log2 = std::max({work_log2, log2_ceil((uint64_t)maxV) + 2, log2_ceil(threads)});
    if (work_log2 > 29) return fail(GCQ_ECAPACITY);   // the G-WFQ ring's limit
    s->work_cap = 1ull << work_log2;
    gcq_queue* q = nullptr;
    if ((rc = gcq_create(GCQ_GWFQ, work_log2, s->threads, &cfg->work_knobs, &q)) != GCQ_OK) return fail(rc);
    s->queues.push_back(q);
    const uint32_t ctl_log2 = std::max<uint32_t>(log2_ceil(ctl_threads), 10);
    for (uint32_t g = 0; g < ntargets; ++g) {
        const uint32_t sub_log2 = std::max<uint32_t>(ctl_log2, 16);
        if ((rc = gcq_create(GCQ_GWFQ, sub_log2, ctl_threads, &k, &q)) != GCQ_OK) return fail(rc);
        s->queues.push_back(q);
        s->graphs[g].subq = (mpmc*)q->obj;
        if ((rc = gcq_create(GCQ_GWFQ, std::max(ctl_log2, log2_ceil(s->graphs[g].nslots)), ctl_threads, &k, &q)) !=
            GCQ_OK)
            return fail(rc);
        s->queues.push_back(q);
        s->graphs[g].slotq = (mpmc*)q->obj;
    }
    if ((rc = dev_alloc(s, &s->d_graphs, sizeof(srv_graph) * ntargets)) != GCQ_OK) return fail(rc);
    if (cudaMemcpy(s->d_graphs, s->graphs.data(), sizeof(srv_graph) * ntargets, cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(gcqi::cuda_fail(cudaGetLastError(), "graph table", __FILE__, __LINE__));
    // level arrays (UNVISITED) and slot headers
    s->level_bytes = level_elems * 4;
    if ((rc = dev_alloc(s, &s->d_levels, (size_t)std::max<uint64_t>(s->level_bytes, 4))) != GCQ_OK) return fail(rc);
    if (cudaMemset(s->d_levels, 0x7F, (size_t)s->level_bytes) != cudaSuccess)
        return fail(gcqi::cuda_fail(cudaGetLastError(), "level reset", __FILE__, __LINE__));
    BRay* d_rays = nullptr;
    BPix* d_pix = nullptr;
    if (tile_elems) {
        if ((rc = dev_alloc(s, &d_rays, tile_elems * sizeof(BRay))) != GCQ_OK ||
            (rc = dev_alloc(s, &d_pix, tile_elems * sizeof(BPix))) != GCQ_OK)
            return fail(rc);
    }
    std::vector<srv_slot> hs(s->total_slots);
    memset((void*)hs.data(), 0, sizeof(srv_slot) * hs.size());
    uint64_t off = 0, toff = 0;
    for (const srv_graph& g : s->graphs) {
        if (g.scene) {
            for (uint32_t i = 0; i < g.nslots; ++i, toff += (uint64_t)g.V) {
                hs[g.slot0 + i].rays = d_rays + toff;
                hs[g.slot0 + i].pix = d_pix + toff;
            }
        } else {
            for (uint32_t i = 0; i < g.nslots; ++i, off += (uint64_t)g.V) hs[g.slot0 + i].level = s->d_levels + off;
        }
    }
    if ((rc = dev_alloc(s, &s->d_slots, sizeof(srv_slot) * hs.size())) != GCQ_OK) return fail(rc);
    if (cudaMemcpy(s->d_slots, hs.data(), sizeof(srv_slot) * hs.size(), cudaMemcpyHostToDevice) != cudaSuccess)
        return fail(gcqi::cuda_fail(cudaGetLastError(), "slot table", __FILE__, __LINE__));
    if ((rc = dev_alloc(s, &s->d_ctl, sizeof(srv_ctl))) != GCQ_OK) return fail(rc);
    *out = s;
    return GCQ_OK;
}

int gcq_serve_image(const gcq_server* s, int scene, float* image) {
    if (!s || !image || scene < 0 || scene >= s->nscenes) return GCQ_EINVAL;
    GCQ_CUDA(cudaMemcpy(image, s->scene_img[scene], s->scene_px[scene] * 12, cudaMemcpyDeviceToHost));
    return GCQ_OK;
}

int gcq_serve_destroy(gcq_server* s) {
    if (!s) return GCQ_EINVAL;
    delete s;
    return GCQ_OK;
}

int gcq_serve_info(const gcq_server* s, int graph, uint32_t* slots, uint32_t* threads, uint64_t* level_bytes) {
    if (!s || graph < -1 || graph >= (int)s->graphs.size()) return GCQ_EINVAL;
    if (slots) *slots = graph < 0 ? s->total_slots : s->graphs[graph].nslots;
    if (threads) *threads = s->threads;
    if (level_bytes) *level_bytes = s->level_bytes;
    return GCQ_OK;
}

int gcq_serve_run(gcq_server* s, const gcq_serve_req* reqs, uint32_t nreq, gcq_serve_res* res,
                  gcq_serve_stats* stats) {
    static_assert(sizeof(gcq_serve_req) == sizeof(srv_req), "request layout");
    static_assert(sizeof(gcq_serve_res) == sizeof(srv_res), "result layout");
    if (!s || !reqs || !res || nreq == 0 || nreq > MAX_REQ) return GCQ_EINVAL;
    for (uint32_t i = 0; i < nreq; ++i) {
        const int g = reqs[i].graph;
        if (g < 0 || g >= (int)s->graphs.size()) return GCQ_EINVAL;
        const int32_t lim = g < s->ngraphs ? s->graphs[g].V : s->scene_tiles[g - s->ngraphs];
        if (reqs[i].src < 0 || reqs[i].src >= lim) return GCQ_EINVAL;
        if (i && reqs[i].arrival_ns < reqs[i - 1].arrival_ns) return GCQ_EINVAL;   // sorted by arrival
        if (reqs[i].arrival_ns > MAX_ARRIVAL_NS) return GCQ_EINVAL;
    }
    // a submission queue holds every request of its graph at once
    std::vector<uint32_t> per_graph(s->graphs.size(), 0);
    for (uint32_t i = 0; i < nreq; ++i) ++per_graph[reqs[i].graph];
    for (size_t g = 0; g < s->graphs.size(); ++g)
        if (per_graph[g] > (1u << s->queues[1 + 2 * g]->order)) return GCQ_ECAPACITY;
    if (s->dirty) {
        GCQ_CUDA(cudaMemset(s->d_levels, 0x7F, (size_t)s->level_bytes));
        s->dirty = false;
    }
    srv_req* d_req = nullptr;
    srv_res* d_res = nullptr;
    GCQ_CUDA(cudaMalloc(&d_req, sizeof(srv_req) * nreq));
    if (cudaMalloc(&d_res, sizeof(srv_res) * nreq) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(d_req);
        return GCQ_ENOMEM;
    }
    int rc = GCQ_OK;
    auto finish = [&](int r) {
        cudaFree(d_req);
        cudaFree(d_res);
        if (r != GCQ_OK) s->dirty = true;
        return r;
    };
    if (cudaMemcpy(d_req, reqs, sizeof(srv_req) * nreq, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(d_res, 0, sizeof(srv_res) * nreq) != cudaSuccess)
        return finish(gcqi::cuda_fail(cudaGetLastError(), "request upload", __FILE__, __LINE__));
    for (gcq_queue* q : s->queues)
        if ((rc = gcq_reset(q, nullptr)) != GCQ_OK) return finish(rc);
    for (size_t g = 0; g < s->graphs.size(); ++g) {
        const srv_graph& hg = s->graphs[g];
        k_fill_slots<<<(hg.nslots + 255) / 256, 256>>>(hg.slotq, hg.slot0, hg.nslots);
    }
    srv_ctl hc;
    memset((void*)&hc, 0, sizeof hc);
    hc.nreq = nreq;
    hc.ngraphs = (uint32_t)s->graphs.size();
    hc.timeout_ns = s->timeout_ns;
    hc.deadline_ns = reqs[nreq - 1].arrival_ns + s->run_limit_ns;
    hc.work_limit = s->work_cap / 2;   // room for re-queued (label-correcting) items
    if (cudaMemcpy(s->d_ctl, &hc, sizeof hc, cudaMemcpyHostToDevice) != cudaSuccess)
        return finish(gcqi::cuda_fail(cudaGetLastError(), "control block", __FILE__, __LINE__));
    srv_ctx x;
    x.workq = (mpmc*)s->queues[0]->obj;
    x.slots = s->d_slots;
    x.graphs = s->d_graphs;
    x.reqs = d_req;
    x.res = d_res;
    x.ctl = s->d_ctl;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    k_stamp_t0<<<1, 32>>>(s->d_ctl);
    cudaEventRecord(e0);
    k_serve<<<s->grid, s->block>>>(x);
    cudaEventRecord(e1);
    cudaError_t ke = cudaGetLastError();
    if (ke == cudaSuccess) ke = cudaEventSynchronize(e1);
    float ms = 0;
    if (ke == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (ke != cudaSuccess) return finish(gcqi::cuda_fail(ke, "k_serve", __FILE__, __LINE__));
    if (cudaMemcpy(res, d_res, sizeof(srv_res) * nreq, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(&hc, s->d_ctl, sizeof hc, cudaMemcpyDeviceToHost) != cudaSuccess)
        return finish(gcqi::cuda_fail(cudaGetLastError(), "results", __FILE__, __LINE__));
    uint32_t err = hc.err;
    for (gcq_queue* q : s->queues) {
        uint32_t e = 0;
        if (cudaMemcpy(&e, q->err, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            return finish(gcqi::cuda_fail(cudaGetLastError(), "queue error word", __FILE__, __LINE__));
        err |= e;
    }
    if (stats) {
        memset(stats, 0, sizeof *stats);
        stats->kernel_ms = ms;
        stats->items = hc.stat[ST_ITEMS];
        stats->stale = hc.stat[ST_STALE];
        stats->edges = hc.stat[ST_EDGES];
        stats->sweeps = hc.stat[ST_SWEEPS];
        stats->rays = hc.stat2[ST_RAYS];
        stats->completed = hc.completed;
        stats->error_word = err;
        stats->released = hc.next_release;
        stats->reserved = hc.reserved;
        gcq::gwf::mpmc wq;
        if (cudaMemcpy(&wq, s->queues[0]->obj, sizeof wq, cudaMemcpyDeviceToHost) == cudaSuccess) {
            const gcq::gwf::ring* rings[2] = {&wq.aq, &wq.fq};
            for (int i = 0; i < 2; ++i) {
                stats->work_tail[i] = rings[i]->Tail >> rings[i]->thr_bits;
                stats->work_head[i] = rings[i]->Head >> rings[i]->thr_bits;
                stats->work_threshold[i] = rings[i]->Threshold;
            }
        }
        std::vector<srv_slot> hs(s->total_slots);
        if (cudaMemcpy(hs.data(), s->d_slots, sizeof(srv_slot) * hs.size(), cudaMemcpyDeviceToHost) == cudaSuccess)
            for (const srv_slot& sl : hs) stats->inflight += (sl.pending != 0 || sl.sweeps_left != 0) ? 1u : 0u;
    }
    if (err & GCQ_ERR_TIMEOUT) return finish(GCQ_ETIMEDOUT);
    if (err & GCQ_ERR_CAPACITY) return finish(GCQ_ECAPACITY);
    if (err) return finish(GCQ_EDEVICE);
    if (hc.completed != nreq) return finish(GCQ_ETIMEDOUT);
    return finish(GCQ_OK);
}

}  // extern "C"
