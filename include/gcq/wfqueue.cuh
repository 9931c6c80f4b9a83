// WFQ-YMC for sm_103a: the GPU adaptation of Yang & Mellor-Crummey's wait-free
// queue in wfqueue_hip_opt.hpp (segmented cells, per-thread handles with enqueue
// and dequeue requests, fast path / slow path / helping, preallocated cell pool
// without reclamation).
//
// Kept from the reference: sentinels BOTTOM=0, TOP=~0, RETRY=~0-1, EMPTY=0
// (:41-58); request state = pending<<63 | id (:124-129); find_cell over a flat
// preallocated pool returning null when exhausted (:208-237); enq_fast/enq_slow/
// enq_commit (:259-318); help_enq (:320-413); deq_fast/help_deq/deq_slow
// (:416-524); the patience loops of wf_enqueue/wf_dequeue (:527-555); the pool size
// threads * (3 * ops + 128) cells plus 8 spare segments (:594-599).
// Changed for GB300:
//   * a cell is 32 bytes {val, enq, deq, pad}, one sector, instead of 24;
//   * cell.enq / cell.deq name a request by handle index (2 + h; 0 null, 1 top)
//     rather than by pointer;
//   * find_cell no longer does atomicMax(active_segments) on every access (:229-232):
//     every cell an operation touches is below max(T, H), which the reset kernel
//     reads instead;
//   * advance_end is one atom.max instead of a CAS loop (:192-199);
//   * the T and H tickets are warp-aggregated;
//   * request publication is release/acquire; loops are bounded.
#pragma once

#include <stdint.h>
#include <string.h>
#include "gcq_atomics.cuh"

#ifndef WF_SEGMENT_SIZE
#define WF_SEGMENT_SIZE 1024u
#endif
#ifndef WF_PATIENCE
#define WF_PATIENCE 16
#endif
#ifndef WF_PREALLOC_OPS_PER_THREAD
#define WF_PREALLOC_OPS_PER_THREAD 512
#endif
#ifndef WF_SEGMENT_SAFETY
#define WF_SEGMENT_SAFETY 8
#endif
#ifndef WF_EMPTY
#define WF_EMPTY 0ull
#endif

namespace gcq {
namespace ymc {

constexpr uint64_t BOTTOM = 0ULL;
constexpr uint64_t TOP = ~0ULL;
constexpr uint64_t EMPTY = WF_EMPTY;
constexpr uint64_t RETRY = ~0ULL - 1;
constexpr uint64_t REQ_NULL = 0, REQ_TOP = 1;   // cell.enq / cell.deq markers

__host__ __device__ __forceinline__ uint64_t pack_state(int pending, uint64_t low63) {
    return ((uint64_t)pending << 63) | (low63 & ((1ULL << 63) - 1));
}
__host__ __device__ __forceinline__ int state_pending(uint64_t s) { return (int)(s >> 63); }
__host__ __device__ __forceinline__ uint64_t state_low(uint64_t s) { return s & ((1ULL << 63) - 1); }

struct alignas(32) cell {
    u64a val;   // data, BOTTOM or TOP
    u64a enq;   // REQ_NULL, REQ_TOP or 2 + handle index
    u64a deq;
    u64a _pad;
};

// Per-thread handle (wfqueue_hip_opt.hpp:161-178).  The request words are shared;
// the cursors are private to the owning thread.
struct alignas(64) handle {
    u64a enq_val, enq_state;   // enqueue request
    u64a deq_id, deq_state;    // dequeue request
    uint32_t next;             // next handle in the ring (read-only after init)
    uint32_t enq_peer, deq_peer;
    uint32_t _pad;
    uint64_t enq_id_last;
};

struct alignas(128) queue {
    u64a T;
    char _pad0[GCQ_HOT_STRIDE - 8];
    u64a H;
    char _pad1[GCQ_HOT_STRIDE - 8];
    cell* cells;
    handle* handles;
    u32a* err;
    uint64_t cap_cells;   // pool size (cells)
    uint32_t nhandles;
    uint32_t patience;
    char _pad2[88];
};

struct ctx {
    queue* q;
    cell* cells;
    handle* hs;
    u32a* err;
    uint64_t cap;
    __device__ __forceinline__ cell* find_cell(uint64_t id) const {
        if (id >= cap) { raise_error(err, ERR_POOL); return nullptr; }
        return &cells[id];
    }
    __device__ __forceinline__ uint64_t req_of(uint32_t h) const { return 2ULL + h; }
};

__device__ __forceinline__ ctx load_ctx(queue* q) {
    ctx c;
    c.q = q; c.cells = q->cells; c.hs = q->handles; c.err = q->err; c.cap = q->cap_cells;
    return c;
}

// wf_init_kernel (:571-591) and the pool clearing of wf_clear_pool_kernel (:646-663),
// as one grid-stride slice over `ncells` cells and the handles.
__device__ inline void init_slice(queue* q, uint64_t ncells, uint64_t gid, uint64_t nthreads) {
    for (uint64_t i = gid; i < ncells; i += nthreads) {
        cell* c = &q->cells[i];
        c->val = BOTTOM; c->enq = REQ_NULL; c->deq = REQ_NULL; c->_pad = 0;
    }
    const uint32_t n = q->nhandles;
    for (uint64_t i = gid; i < n; i += nthreads) {
        handle* h = &q->handles[i];
        h->enq_val = 0; h->enq_state = pack_state(0, 0);
        h->deq_id = 0; h->deq_state = pack_state(0, 0);
        h->next = (uint32_t)((i + 1) % n);
        h->enq_peer = h->next;
        h->deq_peer = h->next;
        h->enq_id_last = 0;
    }
    if (gid == 0) { q->T = 0; q->H = 0; }
}

// advance_end_for_linearizability (:192-199): monotone raise of T or H.
__device__ __forceinline__ void advance_end(u64a* e, uint64_t cid) { fetch_max(e, cid); }

__device__ __forceinline__ bool try_to_claim_req(u64a* state, uint64_t expect_id, uint64_t cell_id) {
    return cas_ok(state, pack_state(1, expect_id), pack_state(0, cell_id));
}

__device__ __forceinline__ void enq_commit(const ctx& x, cell* c, uint64_t v, uint64_t cid) {
    advance_end(&x.q->T, cid + 1);
    exchange(&c->val, v);
}

__device__ __forceinline__ bool enq_fast(const ctx& x, uint64_t v, uint64_t* cid) {
    const uint64_t i = warp_fetch_add(&x.q->T, 1);
    cell* c = x.find_cell(i);
    if (c && cas_ok(&c->val, BOTTOM, v)) return true;
    *cid = i;
    return false;
}

__device__ inline bool enq_slow(const ctx& x, uint32_t hid, uint64_t v, uint64_t cell_id) {
    handle* h = &x.hs[hid];
    st_rlx(&h->enq_val, v);
    st_rel(&h->enq_state, pack_state(1, cell_id));
    for (uint32_t spin = 0; spin < GCQ_SPIN_LIMIT; ++spin) {
        const uint64_t i = fetch_add(&x.q->T, 1);
        cell* c = x.find_cell(i);
        if (!c) break;
        if (cas(&c->enq, REQ_NULL, x.req_of(hid)) == REQ_NULL) {
            const uint64_t cur = ld_acq(&c->val);
            if (cur == BOTTOM || cur == TOP) {
                try_to_claim_req(&h->enq_state, cell_id, i);
                break;
            }
        }
        if (!state_pending(ld_acq(&h->enq_state))) break;
    }
    const uint64_t final_id = state_low(ld_acq(&h->enq_state));
    cell* d = x.find_cell(final_id);
    if (d) {
        // The value goes into the claimed cell before the enqueue returns, as in
        // Yang & Mellor-Crummey's enq_slow.  wfqueue_hip_opt.hpp:313-314 commits only
        // when the cell already reads TOP; a cell still at BOTTOM then waits for a
        // dequeuer to commit the request's value, which this handle's next slow
        // enqueue overwrites, and the value is lost.
        enq_commit(x, d, v, final_id);
        return true;
    }
    return false;   // pool exhausted: the value was dropped, as in the reference
}

__device__ inline uint64_t help_enq(const ctx& x, uint32_t hid, cell* c, uint64_t i) {
    handle* h = &x.hs[hid];
    const uint64_t old = cas(&c->val, BOTTOM, TOP);
    if (old != BOTTOM && old != TOP) return old;
    uint64_t ce = ld_acq(&c->enq);
    if (ce == REQ_NULL) {
        uint32_t p = h->enq_peer;
        uint64_t s = ld_acq(&x.hs[p].enq_state);
        uint64_t rid = state_low(s);
        int pend = state_pending(s);
        if (h->enq_id_last != 0 && h->enq_id_last != rid) {
            h->enq_id_last = 0;
            p = x.hs[p].next;
            h->enq_peer = p;
            s = ld_acq(&x.hs[p].enq_state);
            rid = state_low(s);
            pend = state_pending(s);
        }
        if (pend && rid > 0 && rid <= i) {
            const uint64_t prev = cas(&c->enq, REQ_NULL, x.req_of(p));
            if (prev != REQ_NULL && prev != x.req_of(p)) {
                ce = prev;
                h->enq_id_last = rid;
            } else {
                ce = x.req_of(p);
                h->enq_id_last = 0;
                h->enq_peer = x.hs[p].next;
            }
        } else {
            h->enq_id_last = 0;
            h->enq_peer = x.hs[p].next;
        }
        if (ce == REQ_NULL) {
            const uint64_t prev = cas(&c->enq, REQ_NULL, REQ_TOP);
            ce = (prev == REQ_NULL) ? REQ_TOP : prev;
        }
    }
    if (ce == REQ_TOP) return ld_acq(&x.q->T) <= i ? EMPTY : RETRY;
    handle* rh = &x.hs[ce - 2];
    const uint64_t s = ld_acq(&rh->enq_state);
    const int pend = state_pending(s);
    const uint64_t rid = state_low(s);
    const uint64_t v = ld_rlx(&rh->enq_val);
    if (!pend) {
        if (rid == i) {
            if (ld_acq(&c->val) == TOP) enq_commit(x, c, v, i);
            return ld_acq(&c->val);
        }
        // Bound to a request that took another cell: the cell is dead (TOP), not
        // evidence of an empty queue, as in Yang & Mellor-Crummey's help_enq.
        // wfqueue_hip_opt.hpp:394-395 returns EMPTY here when T <= i, which lets a
        // dequeue request complete empty at this cell past a value cell behind it.
        return ld_acq(&c->val);
    }
    if (rid > i) return ld_acq(&x.q->T) <= i ? EMPTY : RETRY;
    if (try_to_claim_req(&rh->enq_state, rid, i) || ld_acq(&rh->enq_state) == pack_state(0, i)) {
        if (ld_acq(&c->val) == TOP) enq_commit(x, c, v, i);
    }
    return ld_acq(&c->val);
}

__device__ __forceinline__ uint64_t deq_fast(const ctx& x, uint32_t hid, uint64_t* id_out) {
    const uint64_t i = warp_fetch_add(&x.q->H, 1);
    cell* c = x.find_cell(i);
    if (!c) { *id_out = i; return EMPTY; }
    const uint64_t v = help_enq(x, hid, c, i);
    if (v == EMPTY) return EMPTY;
    if (v != TOP && v != RETRY && cas(&c->deq, REQ_NULL, REQ_TOP) == REQ_NULL) return v;
    *id_out = i;
    return RETRY;
}

__device__ inline void help_deq(const ctx& x, uint32_t hid, uint32_t helpee) {
    handle* r = &x.hs[helpee];
    uint64_t s = ld_acq(&r->deq_state);
    const uint64_t id = ld_rlx(&r->deq_id);
    if (!state_pending(s) || state_low(s) < id) return;
    uint64_t prior = id, i = id, cand = 0;
    for (uint32_t spin = 0; spin < GCQ_SPIN_LIMIT; ++spin) {
        s = ld_acq(&r->deq_state);
        if (!state_pending(s) || ld_rlx(&r->deq_id) != id) return;
        while (!cand && state_pending(s) && state_low(s) == prior) {
            cell* c = x.find_cell(++i);
            if (!c) break;
            advance_end(&x.q->H, i + 1);
            const uint64_t v = help_enq(x, hid, c, i);
            if (v == EMPTY || (v != TOP && v != RETRY && ld_acq(&c->deq) == REQ_NULL)) {
                cand = i;
                break;
            }
            s = ld_acq(&r->deq_state);
            if (!state_pending(s) || ld_rlx(&r->deq_id) != id) return;
        }
        if (cand) {
            // The candidate is kept when a smaller cell is announced instead: that cell
            // is tried first, and if its claim fails this one is announced next (Yang &
            // Mellor-Crummey's "if (idx >= new) new = 0").  Dropping it, as
            // wfqueue_hip_opt.hpp:474-479 does, resumes the scan past it, and its value
            // is left behind the request's cell.
            const uint64_t seen = cas(&r->deq_state, pack_state(1, prior), pack_state(1, cand));
            if (seen == pack_state(1, prior) || !state_pending(seen) || state_low(seen) >= cand) cand = 0;
        }
        s = ld_acq(&r->deq_state);
        if (!state_pending(s) || ld_rlx(&r->deq_id) != id) return;
        const uint64_t aidx = state_low(s);
        cell* c = x.find_cell(aidx);
        if (!c) return;
        // Claimed for this request by this helper or by another one: the value the
        // CAS found is compared, as Yang & Mellor-Crummey's help_deq does.
        // wfqueue_hip_opt.hpp:489-492 compares a value loaded before the CAS, so a
        // helper that loses the claim to another helper of the same request moves
        // on, announces a later cell, and the claimed cell's value is orphaned.
        bool claimed = ld_acq(&c->val) == TOP;
        if (!claimed) {
            const uint64_t prev = cas(&c->deq, REQ_NULL, x.req_of(helpee));
            claimed = prev == REQ_NULL || prev == x.req_of(helpee);
        }
        if (claimed) {
            cas(&r->deq_state, s, pack_state(0, aidx));
            return;
        }
        prior = aidx;
        if (aidx >= i) i = aidx;
    }
    raise_error(x.err, ERR_SPIN);
}

__device__ inline uint64_t deq_slow(const ctx& x, uint32_t hid, uint64_t cid) {
    handle* h = &x.hs[hid];
    st_rlx(&h->deq_id, cid);
    st_rel(&h->deq_state, pack_state(1, cid));
    help_deq(x, hid, hid);
    const uint64_t idx = state_low(ld_acq(&h->deq_state));
    cell* c = x.find_cell(idx);
    if (!c) {
        advance_end(&x.q->H, idx + 1);
        return EMPTY;
    }
    const uint64_t v = ld_acq(&c->val);
    advance_end(&x.q->H, idx + 1);
    return v == TOP ? EMPTY : v;
}

// wf_enqueue, :527-536.  `v` must not be 0, ~0 or ~0-1.
__device__ inline bool enqueue(queue* q, uint32_t hid, uint64_t v) {
    const ctx x = load_ctx(q);
    const int patience = (int)q->patience;
    for (int p = patience; p >= 0; --p) {
        uint64_t cid = 0;
        if (enq_fast(x, v, &cid)) return true;
        if (p == 0) return enq_slow(x, hid, v, cid);
    }
    return false;
}

// wf_dequeue, :538-555.  Returns the value or EMPTY.
__device__ inline uint64_t dequeue(queue* q, uint32_t hid) {
    const ctx x = load_ctx(q);
    const int patience = (int)q->patience;
    uint64_t v = RETRY, cid = 0;
    for (int p = patience; p >= 0; --p) {
        v = deq_fast(x, hid, &cid);
        if (v != RETRY) break;
    }
    if (v == RETRY) v = deq_slow(x, hid, cid);
    if (v != EMPTY) {
        handle* h = &x.hs[hid];
        help_deq(x, hid, h->deq_peer);
        h->deq_peer = x.hs[h->deq_peer].next;
    }
    return v;
}

// Dequeue for polling consumers (the reference has none): it never moves H past T.
// The lanes of a warp that call it together take consecutive H tickets with one
// CAS by their leader, and only as many as T - H; each winner then reads its cell,
// whose enqueuer holds the matching T ticket, until the value lands.  A polling
// consumer of wf_dequeue on an empty queue takes an H ticket past T every poll and
// the cell behind it is lost to the pool (no reclamation, wfqueue_hip_opt.hpp:
// 208-237); with this one the pool holds one cell per enqueue.  Meant for
// workloads whose enqueues use the fast path (no consumer marks a cell, so
// enq_fast's CAS succeeds); a cell found marked TOP belongs to an enqueue that went
// elsewhere, and the lane returns empty-handed.  false: nothing taken.
__device__ inline bool try_dequeue(queue* q, uint64_t* out) {
    const unsigned active = __activemask();
    const unsigned peers = __match_any_sync(active, (unsigned long long)(uintptr_t)q);
    const int leader = __ffs(peers) - 1;
    const unsigned rank = __popc(peers & lanemask_lt());
    uint64_t base = 0, n = 0;
    if ((int)lane_id() == leader) {
        uint64_t h = ld_acq(&q->H);
        for (int k = 0; k < 8; ++k) {
            const uint64_t t = ld_acq(&q->T);
            if (t <= h) break;
            const uint64_t want = t - h < (uint64_t)__popc(peers) ? t - h : (uint64_t)__popc(peers);
            const uint64_t old = cas(&q->H, h, h + want);
            if (old == h) {
                base = h;
                n = want;
                break;
            }
            h = old;
        }
    }
    base = __shfl_sync(peers, base, leader);
    n = __shfl_sync(peers, n, leader);
    if (rank >= n) return false;
    const ctx x = load_ctx(q);
    cell* c = x.find_cell(base + rank);
    if (!c) return false;   // past the pool: the enqueue holding this ticket failed too (ERR_POOL)
    backoff bo;
    for (uint32_t k = 0; k < GCQ_SPIN_LIMIT; ++k) {
        const uint64_t v = ld_acq(&c->val);
        if (v == TOP) return false;
        if (v != BOTTOM) {
            *out = v;
            return true;
        }
        bo.pause(256);
    }
    raise_error(x.err, ERR_SPIN);
    return false;
}

}  // namespace ymc
}  // namespace gcq

// -----------------------------------------------------------------------------
// Reference-named device and host API (wfqueue_hip_opt.hpp:161-189, 527-764).
//
// wf_queue is the library's queue object and wf_handle its per-thread handle; a
// handle passed to wf_enqueue/wf_dequeue must be an element of the array the queue
// was initialised with (wf_init_kernel), which is how the reference's harnesses
// use them (&handles[tid]).  The host helpers allocate the queue object, its error
// word and its cell pool in one cudaMalloc, and the handles in another, as the
// reference allocates the queue and the handles apart; the pool is device memory,
// not managed memory (the reference's hipMallocManaged + prefetch,
// wfqueue_hip_opt.hpp:604-640).  They return the first failing CUDA call's error
// instead of printing, and the reference's pool sizes: threads * (3 * ops + 128)
// cells plus WF_SEGMENT_SAFETY segments, or for BFS 1.2 * (V + E / chunk) + 10000
// cells plus the same spare.
// -----------------------------------------------------------------------------
typedef gcq::ymc::queue wf_queue;
typedef gcq::ymc::handle wf_handle;

// wf_enqueue, wfqueue_hip_opt.hpp:527-536.  `value` must not be 0, ~0 or ~0-1.
__device__ __forceinline__ bool wf_enqueue(wf_queue* q, wf_handle* h, uint64_t value) {
    return gcq::ymc::enqueue(q, (uint32_t)(h - q->handles), value);
}
// wf_dequeue, wfqueue_hip_opt.hpp:538-555.  WF_EMPTY (0) when empty.
__device__ __forceinline__ uint64_t wf_dequeue(wf_queue* q, wf_handle* h) {
    return gcq::ymc::dequeue(q, (uint32_t)(h - q->handles));
}
// wf_dequeue_bfs, wfqueue_hip_opt.hpp:557-568: fast-path attempts only, giving up
// as soon as the queue looks empty (T <= H + 1); no slow path, no helping.
__device__ inline uint64_t wf_dequeue_bfs(wf_queue* q, wf_handle* h) {
    const gcq::ymc::ctx x = gcq::ymc::load_ctx(q);
    const uint32_t hid = (uint32_t)(h - q->handles);
    uint64_t cid = 0;
    for (int p = (int)q->patience; p >= 0; --p) {
        const uint64_t v = gcq::ymc::deq_fast(x, hid, &cid);
        if (v != gcq::ymc::RETRY) return v;
        if (gcq::ld_acq(&q->T) <= gcq::ld_acq(&q->H) + 1) return WF_EMPTY;
    }
    return WF_EMPTY;
}

// wf_init_kernel, wfqueue_hip_opt.hpp:571-591: handle i links to handle i + 1 (mod
// num_threads); thread 0 records the array in the queue.
static __global__ void wf_init_kernel(wf_queue* q, wf_handle* handles, int num_threads) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid == 0) {
        q->handles = handles;
        q->nhandles = (uint32_t)num_threads;
    }
    if (tid >= num_threads) return;
    wf_handle* h = &handles[tid];
    h->enq_val = 0; h->enq_state = gcq::ymc::pack_state(0, 0);
    h->deq_id = 0; h->deq_state = gcq::ymc::pack_state(0, 0);
    h->next = (uint32_t)((tid + 1) % num_threads);
    h->enq_peer = h->next;
    h->deq_peer = h->next;
    h->_pad = 0;
    h->enq_id_last = 0;
}

// wf_clear_pool_kernel, wfqueue_hip_opt.hpp:646-663: clear the cells an operation
// can have touched -- every cell below max(T, H) + 1 (the reference clears its
// active segments).
static __global__ void wf_clear_pool_kernel(wf_queue* q) {
    const uint64_t t = q->T, hh = q->H;
    const uint64_t span = (t > hh ? t : hh) + 1;
    const uint64_t used = span < q->cap_cells ? span : q->cap_cells;
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < used; i += (uint64_t)gridDim.x * blockDim.x) {
        gcq::ymc::cell* c = &q->cells[i];
        c->val = gcq::ymc::BOTTOM; c->enq = gcq::ymc::REQ_NULL; c->deq = gcq::ymc::REQ_NULL; c->_pad = 0;
    }
}

static inline cudaError_t wf_queue_host_alloc(wf_queue** d_q, wf_handle** d_handles, int num_threads,
                                              uint64_t cells) {
    if (!d_q || !d_handles || num_threads <= 0) return cudaErrorInvalidValue;
    cells += (uint64_t)WF_SEGMENT_SAFETY * WF_SEGMENT_SIZE;
    const uint64_t head_bytes = (sizeof(wf_queue) + 255) / 256 * 256;
    const uint64_t bytes = head_bytes + 256 + cells * sizeof(gcq::ymc::cell);
    char* base = nullptr;
    cudaError_t e = cudaMalloc((void**)&base, bytes);
    if (e != cudaSuccess) return e;
    e = cudaMalloc((void**)d_handles, sizeof(wf_handle) * (size_t)num_threads);
    if (e != cudaSuccess) { cudaFree(base); return e; }
    wf_queue h;
    memset(&h, 0, sizeof h);
    h.cells = (gcq::ymc::cell*)(base + head_bytes + 256);
    h.err = (gcq::u32a*)(base + head_bytes);
    h.handles = *d_handles;
    h.cap_cells = cells;
    h.nhandles = (uint32_t)num_threads;
    h.patience = WF_PATIENCE;
    if ((e = cudaMemcpy(base, &h, sizeof h, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemset(base + head_bytes, 0, 256 + cells * sizeof(gcq::ymc::cell))) != cudaSuccess) {
        cudaFree(*d_handles);
        cudaFree(base);
        return e;
    }
    *d_q = (wf_queue*)base;
    const int block = 256;
    wf_init_kernel<<<(num_threads + block - 1) / block, block>>>(*d_q, *d_handles, num_threads);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return cudaDeviceSynchronize();
}
// wf_queue_host_init_ex, wfqueue_hip_opt.hpp:594-644
static inline cudaError_t wf_queue_host_init_ex(wf_queue** d_q, wf_handle** d_handles, int num_threads,
                                                int ops_per_thread) {
    if (ops_per_thread < 0) return cudaErrorInvalidValue;
    return wf_queue_host_alloc(d_q, d_handles, num_threads, (uint64_t)num_threads * (3ull * ops_per_thread + 128));
}
// wf_queue_host_init, wfqueue_hip_opt.hpp:762-764
static inline cudaError_t wf_queue_host_init(wf_queue** d_q, wf_handle** d_handles, int num_threads) {
    return wf_queue_host_init_ex(d_q, d_handles, num_threads, WF_PREALLOC_OPS_PER_THREAD);
}
// wf_queue_host_init_for_bfs, wfqueue_hip_opt.hpp:697-760
static inline cudaError_t wf_queue_host_init_for_bfs(wf_queue** d_q, wf_handle** d_handles, int num_threads,
                                                     long long graph_edges, int graph_vertices, int chunk_size) {
    if (graph_edges < 0 || graph_vertices < 0 || chunk_size <= 0) return cudaErrorInvalidValue;
    const uint64_t work_items = ((uint64_t)graph_edges + chunk_size - 1) / chunk_size;
    const uint64_t cells = (uint64_t)(((uint64_t)graph_vertices + work_items) * 1.20) + 10000;
    return wf_queue_host_alloc(d_q, d_handles, num_threads, cells);
}
// wf_queue_reset_for_bfs, wfqueue_hip_opt.hpp:665-695: clear the used cells, zero
// T and H, re-initialise the handles.
static inline cudaError_t wf_queue_reset_for_bfs(wf_queue* d_q, wf_handle* d_handles, int num_threads) {
    wf_clear_pool_kernel<<<152 * 8, 256>>>(d_q);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemset((void*)&d_q->T, 0, sizeof(d_q->T));
    if (e == cudaSuccess) e = cudaMemset((void*)&d_q->H, 0, sizeof(d_q->H));
    if (e != cudaSuccess) return e;
    const int block = 256;
    wf_init_kernel<<<(num_threads + block - 1) / block, block>>>(d_q, d_handles, num_threads);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return cudaDeviceSynchronize();
}
// Free what the host initialisers allocated (the reference leaves this to hipFree).
static inline void wf_queue_host_destroy(wf_queue* d_q, wf_handle* d_handles) {
    if (d_q) cudaFree(d_q);
    if (d_handles) cudaFree(d_handles);
}
