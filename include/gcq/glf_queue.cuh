// G-LFQ for sm_103a: the lock-free SCQ queue of glf_queue.hpp with
// warp-aggregated tickets, 64-bit entries {Cycle, Safe1, Index32}, no slow path.
//
// Kept from the reference: entry layout and INIT (glf_queue.hpp:66-90), modular
// cycles (:96-110), the line-spreading slot permutation (:116-120), ring and
// indirection layout (:126-138), enqueue/dequeue loops (:467-560), 64-bit payload
// indirection (:566-582).
// Changed for GB300: the cycle tag is 16 bits by default (FQ_CYCLE_BITS; the
// reference's knob, whose default of 8 bits wraps once an operation holds a ticket
// 128 cycles behind the counters -- a stale entry then compares as current and a
// value is lost or taken twice on rings of a few times the thread count); ring
// capacity and the permutation are runtime header fields;
// the enqueue CAS is tried first against the steady-state free slot, and a
// dequeuer waits briefly for the enqueuer holding its ticket before marking the
// slot (deq_wait);
// the slot permutation (128-byte lines, 16 entries) is a knob, identity by default
// (with warp-aggregated tickets contiguous slots coalesce in L2); Tail, Head
// and Threshold sit GCQ_HOT_STRIDE apart; loads are acquire/relaxed loads instead of
// atomicAdd(p, 0) (:144-148); retry loops are bounded (GCQ_SPIN_LIMIT) and report
// through the header's error word instead of spinning forever.
#pragma once

#include <stdint.h>
#include "gcq_atomics.cuh"

#ifndef FQ_N
#define FQ_N 32768
#endif
#ifndef FQ_CYCLE_BITS
#define FQ_CYCLE_BITS 16
#endif

namespace gcq {
namespace glf {

constexpr uint32_t CYCLE_MASK = (1u << FQ_CYCLE_BITS) - 1;
constexpr uint32_t HALF_CYCLE = 1u << (FQ_CYCLE_BITS - 1);
constexpr uint32_t BOT = 0xFFFFFFFEu;
constexpr uint32_t BOT_C = 0xFFFFFFFFu;

namespace ent {
constexpr int CYCLE_SHIFT = 48, SAFE_SHIFT = 47;
static_assert(FQ_CYCLE_BITS >= 4 && CYCLE_SHIFT + FQ_CYCLE_BITS <= 64, "the cycle tag must fit above bit 48");
constexpr uint64_t SAFE_BIT = 1ULL << SAFE_SHIFT;
constexpr uint64_t CONSUME_MASK = (uint64_t)BOT_C;
constexpr uint64_t INIT = SAFE_BIT | (uint64_t)BOT;
__host__ __device__ __forceinline__ uint32_t cycle(uint64_t e) { return (uint32_t)(e >> CYCLE_SHIFT) & CYCLE_MASK; }
__host__ __device__ __forceinline__ bool safe(uint64_t e) { return (e >> SAFE_SHIFT) & 1; }
__host__ __device__ __forceinline__ uint32_t index(uint64_t e) { return (uint32_t)e; }
__host__ __device__ __forceinline__ uint64_t pack(uint32_t c, bool s, uint32_t i) {
    return ((uint64_t)(c & CYCLE_MASK) << CYCLE_SHIFT) | ((uint64_t)s << SAFE_SHIFT) | (uint64_t)i;
}
}  // namespace ent

__host__ __device__ __forceinline__ int cycle_cmp(uint32_t a, uint32_t b) {
    const uint32_t d = (a - b) & CYCLE_MASK;
    return d == 0 ? 0 : (d < HALF_CYCLE ? 1 : -1);
}

struct alignas(128) ring {
    u64a Tail;
    char _pad0[GCQ_HOT_STRIDE - 8];
    u64a Head;
    char _pad1[GCQ_HOT_STRIDE - 8];
    int Threshold;
    char _pad2[GCQ_HOT_STRIDE - 4];
    u64a* Entry;          // 2N slots
    u32a* err;
    uint32_t order;       // log2 N
    uint32_t line_log2;   // log2 entries per line for the permutation; 0 = identity
    uint32_t deq_wait;    // re-reads of a not-yet-filled slot before marking it
    char _pad3[100];
};

struct alignas(128) mpmc {
    ring aq;
    ring fq;
    u64a* data;
    u32a* err;
};

struct cfg {
    u64a* entry;
    u32a* err;
    uint32_t order, line_log2, deq_wait;
    __host__ __device__ __forceinline__ uint32_t slots() const { return 2u << order; }
    __host__ __device__ __forceinline__ int32_t threshold_max() const { return 3 * (int32_t)(1u << order) - 1; }
    __host__ __device__ __forceinline__ uint32_t cycle_of(uint64_t t) const { return (uint32_t)(t >> (order + 1)) & CYCLE_MASK; }
    // cache_remap, glf_queue.hpp:116-120
    __host__ __device__ __forceinline__ uint32_t slot_of(uint64_t t) const {
        const uint32_t pos = (uint32_t)t & (slots() - 1);
        if (line_log2 == 0 || slots() <= (1u << line_log2)) return pos;
        const uint32_t per = 1u << line_log2;
        return (pos & (per - 1)) * (slots() >> line_log2) + (pos >> line_log2);
    }
    __host__ __device__ __forceinline__ uint32_t pos_of_slot(uint32_t s) const {
        if (line_log2 == 0 || slots() <= (1u << line_log2)) return s;
        const uint32_t stride = slots() >> line_log2;
        return (s % stride) * (1u << line_log2) + s / stride;
    }
};

__device__ __forceinline__ cfg load_cfg(const ring* q) {
    cfg c;
    c.entry = q->Entry; c.err = q->err; c.order = q->order; c.line_log2 = q->line_log2;
    c.deq_wait = q->deq_wait;
    return c;
}

// fq_ring_init_empty / fq_ring_init_full (glf_queue.hpp:418-435), split over a
// grid-stride group; each slot's final value is computed directly.
__device__ inline void init_slice(ring* q, bool full, uint64_t gid, uint64_t nthreads) {
    const cfg c = load_cfg(q);
    const uint32_t slots = c.slots(), n = 1u << c.order;
    for (uint64_t s = gid; s < slots; s += nthreads) {
        const uint32_t pos = c.pos_of_slot((uint32_t)s);
        c.entry[s] = (full && pos < n) ? ent::pack(c.cycle_of((uint64_t)slots + pos), true, pos) : ent::INIT;
    }
    if (gid == 0) {
        q->Head = slots;
        q->Tail = full ? (uint64_t)slots + n : (uint64_t)slots;
        q->Threshold = full ? c.threshold_max() : -1;
    }
}

// catchup, glf_queue.hpp:447-455
__device__ inline void catchup(ring* q, uint64_t tail, uint64_t head) {
    for (int i = 0; i < 32; i++) {
        if (cas_ok(&q->Tail, tail, head)) break;
        head = ld_acq(&q->Head);
        tail = ld_acq(&q->Tail);
        if (tail >= head) break;
    }
}

// fq_enqueue, glf_queue.hpp:467-500.  Returns false only if the retry bound was
// reached (error word set).  Publish: as gwf::try_enq (acq_rel entry CAS when the
// caller wrote what the index refers to, acquire only when it ordered its accesses
// itself).
template <bool Publish = true>
__device__ inline bool enqueue(ring* q, uint32_t index) {
    const cfg c = load_cfg(q);
    for (uint32_t spin = 0; spin < GCQ_SPIN_LIMIT; ++spin) {
        const uint64_t T = warp_ticket(&q->Tail, 1);
        const uint32_t tcyc = c.cycle_of(T);
        const uint32_t j = c.slot_of(T);
        // CAS first against the steady-state free slot (previous cycle, safe,
        // consumed); a mismatch returns the current value for the loop below.
        uint64_t E = ent::pack(tcyc - 1, true, BOT_C);
        if (cas_upd_ord<Publish>(&c.entry[j], &E, ent::pack(tcyc, true, index))) {
            reset_threshold(&q->Threshold, c.threshold_max());
            return true;
        }
        for (;; ++spin) {
            const uint32_t ecyc = ent::cycle(E), eidx = ent::index(E);
            if (cycle_cmp(ecyc, tcyc) >= 0 || eidx < BOT) break;
            if (!ent::safe(E)) {
                dekker_fence();
                if (ld_rlx(&q->Head) > T) break;
            }
            if (!cas_upd_ord<Publish>(&c.entry[j], &E, ent::pack(tcyc, true, index))) {
                if (spin >= GCQ_SPIN_LIMIT) break;
                continue;
            }
            reset_threshold(&q->Threshold, c.threshold_max());
            return true;
        }
    }
    raise_error(c.err, ERR_SPIN);
    return false;
}

#ifndef GCQ_GLF_EMPTY_CHECK
#define GCQ_GLF_EMPTY_CHECK 1
#endif
// fq_dequeue, glf_queue.hpp:510-560.  Returns the index or BOT when empty.
__device__ inline uint32_t dequeue(ring* q) {
    if (ld_rlx(&q->Threshold) < 0) return BOT;
    const cfg c = load_cfg(q);
    for (uint32_t spin = 0; spin < GCQ_SPIN_LIMIT; ++spin) {
        const uint64_t H = warp_ticket(&q->Head, 1);
        const uint32_t hcyc = c.cycle_of(H);
        const uint32_t j = c.slot_of(H);
        uint64_t E = ld_acq(&c.entry[j]);   // acquire: the payload reads follow a consume
        // bounded wait for the enqueuer holding this ticket (see gwf::try_deq)
        if (c.deq_wait && cycle_cmp(ent::cycle(E), hcyc) < 0 && ent::index(E) >= BOT) {
            uint32_t ns = 32;
            for (uint32_t w = 0; w < c.deq_wait; ++w) {
                __nanosleep(ns);
                ns = ns < 1024 ? ns * 2 : ns;
                E = ld_acq(&c.entry[j]);
                if (!(cycle_cmp(ent::cycle(E), hcyc) < 0 && ent::index(E) >= BOT)) break;
            }
        }
        for (bool acquired = true;; ++spin) {
            const uint32_t ecyc = ent::cycle(E), eidx = ent::index(E);
            if (cycle_cmp(ecyc, hcyc) == 0 && eidx < BOT) {
                // E was read with acquire semantics (or is fenced now), so the OR that
                // marks the slot consumed is issued without waiting for it
                if (!acquired) fence_acq_rel();
                red_or_rlx(&c.entry[j], ent::CONSUME_MASK);
                return eidx;
            }
            if (cycle_cmp(ecyc, hcyc) >= 0 || spin >= GCQ_SPIN_LIMIT) break;
            const uint64_t nw = (eidx >= BOT) ? ent::pack(hcyc, ent::safe(E), BOT) : ent::pack(ecyc, false, eidx);
            if (cas_upd_rlx(&c.entry[j], &E, nw)) break;
            acquired = false;
        }
        dekker_fence();
        const uint64_t T = ld_rlx(&q->Tail);
        if (T <= H + 1) {
            catchup(q, T, H + 1);
            fetch_add(&q->Threshold, -1);
            return BOT;
        }
        if (fetch_add(&q->Threshold, -1) <= 0) return BOT;
        // the empty exit before a retry ticket, as G-WFQ's (gwf::seen_empty)
        if (GCQ_GLF_EMPTY_CHECK) {
            const uint64_t h = ld_acq(&q->Head);
            const uint64_t t = ld_rlx(&q->Tail);
            if (t <= h) {
                if (t < h) catchup(q, t, h);
                return BOT;
            }
        }
    }
    raise_error(c.err, ERR_SPIN);
    return BOT;
}

// fq_enqueue_ptr / fq_dequeue_ptr, glf_queue.hpp:566-582.  The payload is written
// before an acq_rel index enqueue (the release publishes it) and read after the
// dequeue's acquire; the index's return to fq is an acq_rel CAS, whose release
// orders the read before the next producer's write (GCQ_ACQUIRE_ONLY_RETURN).
// (Payloads in flagged 128-bit cells, written by an exchange the producer does not
// wait for, with an acquire-only index enqueue, measured slower: 52.6 against 60.1
// Gops/s balanced at 262144 threads.)  They work on the two rings and the payload
// array, so the library's queue (mpmc) and the self-contained fq_mpmc_t below run
// the same code.
__device__ __forceinline__ bool enqueue_ptr(ring* aq, ring* fq, u64a* data, uint64_t value) {
    const uint32_t idx = dequeue(fq);
    if (idx == BOT) return false;
    st_rlx(&data[idx], value);
    return enqueue(aq, idx);
}
__device__ __forceinline__ bool dequeue_ptr(ring* aq, ring* fq, u64a* data, uint64_t* out) {
    const uint32_t idx = dequeue(aq);
    if (idx == BOT) return false;
    *out = ld_acq(&data[idx]);
    enqueue<!GCQ_ACQUIRE_ONLY_RETURN>(fq, idx);
    return true;
}
__device__ __forceinline__ bool enqueue_ptr(mpmc* q, uint64_t value) { return enqueue_ptr(&q->aq, &q->fq, q->data, value); }
__device__ __forceinline__ bool dequeue_ptr(mpmc* q, uint64_t* out) { return dequeue_ptr(&q->aq, &q->fq, q->data, out); }

}  // namespace glf
}  // namespace gcq

// -----------------------------------------------------------------------------
// Reference-named device API (glf_queue.hpp:32-46, 126-138, 418-582).
//
// fq_ring_t and fq_mpmc_t are self-contained, as in the reference: a caller
// allocates sizeof(fq_mpmc_t) and runs fq_init on one thread.  A ring is the
// library's ring header (Tail, Head and Threshold GCQ_HOT_STRIDE apart, then the
// parameters) followed by its FQ_SLOTS entries; fq_ring_init_* point the header at
// them.  The payload array is the reference's data[FQ_N].
// -----------------------------------------------------------------------------
static constexpr uint32_t FQ_SLOTS = 2 * FQ_N;
static constexpr int32_t FQ_THRESH_MAX = 3 * (int32_t)FQ_N - 1;
static constexpr uint32_t FQ_BOT = gcq::glf::BOT;
static constexpr uint32_t FQ_BOT_C = gcq::glf::BOT_C;
static_assert((FQ_N & (FQ_N - 1)) == 0, "FQ_N must be a power of two");

struct fq_ring_t : gcq::glf::ring {
    // The reference's Entry[FQ_SLOTS]; the header's own Entry pointer (gcq::glf::ring::Entry),
    // hidden by this name, is set to it by the initialisers.
    unsigned long long Entry[FQ_SLOTS];
    gcq::u32a err_word;
};
struct fq_mpmc_t {
    fq_ring_t aq;   // allocated indices
    fq_ring_t fq;   // free indices
    uint64_t data[FQ_N];
};

// fq_ring_init_empty / fq_ring_init_full, glf_queue.hpp:418-435 (one thread).
__device__ inline void fq_ring_setup(fq_ring_t* q) {
    gcq::glf::ring* h = q;
    h->Entry = q->Entry;
    q->err_word = 0;
    h->err = &q->err_word;
    h->order = 31 - __clz(FQ_N);
#ifdef FQ_CACHE_REMAP
    h->line_log2 = 3;   // the reference's cache_remap: 8 entries per 64-byte line (glf_queue.hpp:116-120)
#else
    h->line_log2 = 0;   // identity, the library's default (contiguous tickets coalesce in L2)
#endif
    h->deq_wait = 0;
}
__device__ inline void fq_ring_init_empty(fq_ring_t* q) {
    fq_ring_setup(q);
    gcq::glf::init_slice(q, false, 0, 1);
    __threadfence();
}
__device__ inline void fq_ring_init_full(fq_ring_t* q) {
    fq_ring_setup(q);
    gcq::glf::init_slice(q, true, 0, 1);
    __threadfence();
}
// fq_init, glf_queue.hpp:437-440
__device__ inline void fq_init(fq_mpmc_t* q) {
    fq_ring_init_empty(&q->aq);
    fq_ring_init_full(&q->fq);
}
// fq_enqueue / fq_dequeue, glf_queue.hpp:467-560, on a self-contained ring or a
// ring header of the library's queues (gcq::glf::ring).
__device__ __forceinline__ void fq_enqueue(gcq::glf::ring* q, uint32_t index) { gcq::glf::enqueue(q, index); }
__device__ __forceinline__ uint32_t fq_dequeue(gcq::glf::ring* q) { return gcq::glf::dequeue(q); }
// fq_enqueue_ptr / fq_dequeue_ptr, glf_queue.hpp:566-582
__device__ __forceinline__ bool fq_enqueue_ptr(fq_mpmc_t* q, uint64_t v) {
    return gcq::glf::enqueue_ptr(&q->aq, &q->fq, (gcq::u64a*)q->data, v);
}
__device__ __forceinline__ bool fq_dequeue_ptr(fq_mpmc_t* q, uint64_t* out) {
    return gcq::glf::dequeue_ptr(&q->aq, &q->fq, (gcq::u64a*)q->data, out);
}
__device__ __forceinline__ bool fq_enqueue_ptr(gcq::glf::mpmc* q, uint64_t v) { return gcq::glf::enqueue_ptr(q, v); }
__device__ __forceinline__ bool fq_dequeue_ptr(gcq::glf::mpmc* q, uint64_t* out) { return gcq::glf::dequeue_ptr(q, out); }
