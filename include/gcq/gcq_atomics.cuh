// gpu-scope memory operations, warp-aggregated tickets and bounded waits shared by
// the four gCQ queues on sm_103a.
//
// The reference relies on HIP's atomics being sequentially consistent
// (gwf_ring.hpp:15-17) and on __threadfence for publication.  On NVIDIA GPUs plain
// atomicCAS/atomicAdd are relaxed, so every shared queue word here goes through an
// explicitly ordered PTX operation at .gpu scope:
//   * the fast paths use the weakest order each step needs: relaxed tickets and
//     entry loads, a release CAS where an enqueue publishes (it makes the payload
//     written before it visible), an acquire OR where a dequeue consumes (it makes
//     the payload visible to the reads after it), relaxed marking CASes;
//   * the slow paths and request records keep acq_rel read-modify-writes and
//     acquire/release loads and stores;
//   * the two store->load (Dekker) points of the SCQ emptiness argument get a
//     fence.sc (GCQ_SC_FENCES, on by default): a dequeuer's read of Tail after its
//     fetch-and-add on Head, and an enqueuer's read of Head after its add on Tail.
// All queue memory is global (device) memory.
#pragma once

#include <stdint.h>
#include <cuda_runtime.h>

#ifndef GCQ_SC_FENCES
#define GCQ_SC_FENCES 1
#endif

// Distance in bytes between the hot words of one queue header (ticket counters,
// threshold, close flag).  On GB300, counters on adjacent 128-B lines land in the
// same L2 slice, whose atomic unit then serves every ticket and threshold access
// of the queue; 4 KB apart they spread over slices.  Balanced G-WFQ at 262144
// threads: 21.4 Gops/s with 128 B, 34.2 with 4 KB (16 KB: no further gain).
#ifndef GCQ_HOT_STRIDE
#define GCQ_HOT_STRIDE 4096
#endif

// Upper bound on any retry loop inside one queue operation; reaching it marks the
// queue's error word and makes the operation fail instead of spinning forever.
#ifndef GCQ_SPIN_LIMIT
#define GCQ_SPIN_LIMIT (1u << 22)
#endif

namespace gcq {

typedef unsigned long long u64a;   // type of 64-bit atomic words
typedef unsigned int u32a;         // type of 32-bit atomic words

// ---- error word bits (queue header `err`, read by the host after a launch) ----
enum : unsigned int {
    ERR_SPIN = 1u << 0,       // a retry loop reached GCQ_SPIN_LIMIT
    ERR_TIMEOUT = 1u << 1,    // a blocking wait passed its deadline
    ERR_TID = 1u << 2,        // a thread index at or above the record count
    ERR_POOL = 1u << 3,       // YMC segment pool exhausted
    ERR_CAPACITY = 1u << 4,   // harness-level overflow (frontier larger than the queue)
};

// ---------------------------------------------------------------- loads/stores
__device__ __forceinline__ uint64_t ld_acq(const u64a* p) {
    uint64_t v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint64_t ld_rlx(const u64a* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t ld_acq(const u32a* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ uint32_t ld_rlx(const u32a* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int32_t ld_acq(const int* p) {
    int32_t v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ int32_t ld_rlx(const int* p) {
    int32_t v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_rel(u64a* p, uint64_t v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_rlx(u64a* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_rel(u32a* p, uint32_t v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void st_rlx(u32a* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// ---------------------------------------------------------------- read-modify-write
__device__ __forceinline__ uint64_t fetch_add(u64a* p, uint64_t v) {
    uint64_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}
__device__ __forceinline__ uint64_t fetch_add_rlx(u64a* p, uint64_t v) {
    uint64_t old;
    asm volatile("atom.relaxed.gpu.global.add.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}
__device__ __forceinline__ uint32_t fetch_add(u32a* p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ int32_t fetch_add(int* p, int32_t v) {
    int32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.s32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ int32_t exchange(int* p, int32_t v) {
    int32_t old;
    asm volatile("atom.acq_rel.gpu.global.exch.b32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ uint64_t exchange(u64a* p, uint64_t v) {
    uint64_t old;
    asm volatile("atom.acq_rel.gpu.global.exch.b64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}
// compare-and-swap; returns the previous value
__device__ __forceinline__ uint64_t cas(u64a* p, uint64_t expect, uint64_t desired) {
    uint64_t old;
    asm volatile("atom.acq_rel.gpu.global.cas.b64 %0, [%1], %2, %3;"
                 : "=l"(old) : "l"(p), "l"(expect), "l"(desired) : "memory");
    return old;
}
__device__ __forceinline__ uint32_t cas(u32a* p, uint32_t expect, uint32_t desired) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.cas.b32 %0, [%1], %2, %3;"
                 : "=r"(old) : "l"(p), "r"(expect), "r"(desired) : "memory");
    return old;
}
__device__ __forceinline__ uint64_t cas_rel(u64a* p, uint64_t expect, uint64_t desired) {
    uint64_t old;
    asm volatile("atom.release.gpu.global.cas.b64 %0, [%1], %2, %3;"
                 : "=l"(old) : "l"(p), "l"(expect), "l"(desired) : "memory");
    return old;
}
__device__ __forceinline__ uint64_t cas_rlx(u64a* p, uint64_t expect, uint64_t desired) {
    uint64_t old;
    asm volatile("atom.relaxed.gpu.global.cas.b64 %0, [%1], %2, %3;"
                 : "=l"(old) : "l"(p), "l"(expect), "l"(desired) : "memory");
    return old;
}
__device__ __forceinline__ bool cas_upd_rel(u64a* p, uint64_t* expect, uint64_t desired) {
    const uint64_t old = cas_rel(p, *expect, desired);
    const bool ok = (old == *expect);
    *expect = old;
    return ok;
}
__device__ __forceinline__ uint64_t cas_acq(u64a* p, uint64_t expect, uint64_t desired) {
    uint64_t old;
    asm volatile("atom.acquire.gpu.global.cas.b64 %0, [%1], %2, %3;"
                 : "=l"(old) : "l"(p), "l"(expect), "l"(desired) : "memory");
    return old;
}
// CAS with acq_rel (Release) or acquire ordering, refreshing `expect`.  A release
// costs the issuing thread an extra L2 round trip on this GPU; acquire does not.
template <bool Release>
__device__ __forceinline__ bool cas_upd_ord(u64a* p, uint64_t* expect, uint64_t desired) {
    const uint64_t old = Release ? cas(p, *expect, desired) : cas_acq(p, *expect, desired);
    const bool ok = (old == *expect);
    *expect = old;
    return ok;
}
__device__ __forceinline__ bool cas_upd_rlx(u64a* p, uint64_t* expect, uint64_t desired) {
    const uint64_t old = cas_rlx(p, *expect, desired);
    const bool ok = (old == *expect);
    *expect = old;
    return ok;
}
// OR without a returned value: the issuing thread does not wait for it.
__device__ __forceinline__ void red_or_rlx(u64a* p, uint64_t v) {
    asm volatile("red.relaxed.gpu.global.or.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
// Reset an SCQ Threshold to its maximum after a successful enqueue (SCQ's
// "if Threshold != 3n-1 then Threshold = 3n-1"): a load of the hot word (served by
// L2 for every lane of a warp at once) and an exchange only when it moved.  A
// non-returning red.max in its place -- 3n-1 is the largest value the word holds,
// so max is the exchange and the enqueuer would not wait for the load -- measured
// 23.3 against 35.0 Gops/s (balanced G-WFQ, 262144 threads) and 21.1 against 61.7
// (G-LFQ): every enqueue then sends an atomic to the one word, and the L2 slice
// serialises them.
__device__ __forceinline__ void reset_threshold(int* thr, int32_t thr_max) {
    if (ld_rlx(thr) != thr_max) exchange(thr, thr_max);
}

// Order of an MPMC queue's index return to its free ring.  A consumer's read of a
// payload must come before the next producer's write to it.  The return is an
// acq_rel CAS and the producer obtains the index with an acquire read of the free
// ring's entry, so under the PTX model the read precedes the write in causality
// order.  GCQ_ACQUIRE_ONLY_RETURN=1 makes the return acquire-only and the payload
// read an acquire load: the read is then performed before the CAS is issued, which
// orders it on this hardware, but the PTX model gives no cross-thread order
// without the release.  Off by default.
#ifndef GCQ_ACQUIRE_ONLY_RETURN
#define GCQ_ACQUIRE_ONLY_RETURN 0
#endif
// CAS that reports success and refreshes `expect` with the observed value
// (the C11 compare_exchange contract used by gwf_ring.hpp:93-99).
__device__ __forceinline__ bool cas_upd(u64a* p, uint64_t* expect, uint64_t desired) {
    uint64_t old = cas(p, *expect, desired);
    bool ok = (old == *expect);
    *expect = old;
    return ok;
}
__device__ __forceinline__ bool cas_ok(u64a* p, uint64_t expect, uint64_t desired) {
    return cas(p, expect, desired) == expect;
}
__device__ __forceinline__ uint64_t fetch_or(u64a* p, uint64_t v) {
    uint64_t old;
    asm volatile("atom.acq_rel.gpu.global.or.b64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}
__device__ __forceinline__ uint32_t fetch_or(u32a* p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.or.b32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ uint64_t fetch_max(u64a* p, uint64_t v) {
    uint64_t old;
    asm volatile("atom.acq_rel.gpu.global.max.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
    return old;
}

// ---------------------------------------------------------------- fences, time
__device__ __forceinline__ void fence_sc() { asm volatile("fence.sc.gpu;" ::: "memory"); }
__device__ __forceinline__ void fence_acq_rel() { asm volatile("fence.acq_rel.gpu;" ::: "memory"); }
// Full fence at the store->load points of the emptiness argument (see header).
__device__ __forceinline__ void dekker_fence() {
#if GCQ_SC_FENCES
    fence_sc();
#endif
}
__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint32_t lane_id() {
    uint32_t l;
    asm("mov.u32 %0, %%laneid;" : "=r"(l));
    return l;
}
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Record an error in a queue's error word (sticky until the host resets it).  The
// word is read first so that a condition hit by every thread (an exhausted YMC
// pool) does not turn into one single-address atomic per operation.
__device__ __forceinline__ void raise_error(u32a* err, unsigned int bits) {
    if (err && (ld_rlx(err) & bits) != bits) fetch_or(err, bits);
}


// ---------------------------------------------------------------- tickets
// Warp-aggregated fetch-and-add: the lanes that are executing this call together
// and name the same counter get consecutive values from one L2 atomic issued by
// the lowest such lane.  The group is formed from __activemask() and narrowed by
// __match_any_sync on the address, and every shuffle uses exactly that group, so
// the result is well defined under independent thread scheduling however the
// warp has diverged (the reference shuffles with a full mask under a partial
// __activemask(), glf_queue.hpp:245-246 with :392-404).
__device__ __forceinline__ uint64_t warp_fetch_add(u64a* p, uint64_t step) {
    const unsigned active = __activemask();
    const unsigned peers = __match_any_sync(active, (unsigned long long)(uintptr_t)p);
    const int leader = __ffs(peers) - 1;
    const unsigned rank = __popc(peers & lanemask_lt());
    uint64_t base = 0;
    if ((int)lane_id() == leader) base = fetch_add(p, step * (uint64_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + (uint64_t)rank * step;
}
// The same with a relaxed fetch-and-add: a ticket orders nothing by itself (the
// entry it selects is read through its address), so the fast paths take their
// tickets without a fence; the store->load points have their own fence.sc.
__device__ __forceinline__ uint64_t warp_ticket(u64a* p, uint64_t step) {
    const unsigned active = __activemask();
    const unsigned peers = __match_any_sync(active, (unsigned long long)(uintptr_t)p);
    const int leader = __ffs(peers) - 1;
    const unsigned rank = __popc(peers & lanemask_lt());
    uint64_t base = 0;
    if ((int)lane_id() == leader) base = fetch_add_rlx(p, step * (uint64_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    return base + (uint64_t)rank * step;
}

// A warp-aggregated ticket in two halves, so that the fetch-and-add's round trip
// can overlap another memory access of the same lanes: ticket_issue sends the
// leader's relaxed fetch-and-add and returns without waiting for it; the caller
// issues its other access; ticket_take distributes the result (the first use of the
// returned value, where the leader waits).  Both halves must run on the same lanes.
struct ticket_req {
    unsigned peers;
    int leader;
    unsigned rank;
    uint64_t base;   // the leader's pending fetch-and-add result
};
__device__ __forceinline__ ticket_req ticket_issue(u64a* p, uint64_t step) {
    ticket_req t;
    const unsigned active = __activemask();
    t.peers = __match_any_sync(active, (unsigned long long)(uintptr_t)p);
    t.leader = __ffs(t.peers) - 1;
    t.rank = __popc(t.peers & lanemask_lt());
    t.base = 0;
    if ((int)lane_id() == t.leader) t.base = fetch_add_rlx(p, step * (uint64_t)__popc(t.peers));
    return t;
}
__device__ __forceinline__ uint64_t ticket_take(const ticket_req& t, uint64_t step) {
    return __shfl_sync(t.peers, t.base, t.leader) + (uint64_t)t.rank * step;
}

// ---------------------------------------------------------------- waiting
// Deadline-bounded back-off used by every blocking wait: starts with a few spins,
// then sleeps with exponentially growing __nanosleep up to max_ns.
struct backoff {
    uint32_t ns = 0;
    __device__ __forceinline__ void pause(uint32_t max_ns = 2048) {
        if (ns == 0) { ns = 32; return; }
        __nanosleep(ns);
        ns = ns < max_ns ? ns * 2 : max_ns;
    }
};

}  // namespace gcq
