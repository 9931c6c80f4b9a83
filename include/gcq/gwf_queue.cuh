// G-WFQ types for sm_103a: the wait-free queue of gwf_queue.hpp (wCQ squeezed into
// 64-bit words), laid out for GB300.
//
// Kept from the reference (same bit layouts, same names):
//   * global counter word {Counter, ThrIdx}          gwf_queue.hpp:31-92
//   * modular cycle comparison                         gwf_queue.hpp:110-136
//   * entry {Note, Cycle, Safe1, Enq1, Index32}        gwf_queue.hpp:149-189
//   * local counter {cnt<<2 | INC | FIN}               gwf_queue.hpp:202-216
//   * per-thread help request and phase-2 record       gwf_queue.hpp:242-288
//   * ring {Tail, Head, Threshold, Entry[2N], Record}  gwf_queue.hpp:313-332
//   * indirection {aq, fq, data[N]}                    gwf_queue.hpp:338-345
// Changed for GB300:
//   * Note and Cycle are 15 bits each by default (WF_CYCLE_BITS), not 8: they fill
//     the 14 bits the reference's entry leaves zero (gwf_queue.hpp:140-146).  An
//     8-bit tag wraps when an operation still holds a ticket 128 cycles behind the
//     ring's counters (128 x 2N tickets), after which a stale entry compares as
//     current; on rings of a few times the thread count that happens, and values
//     are lost or taken twice.  WF_CYCLE_BITS=8 gives the reference's layout;
//   * ring parameters (capacity, ThrIdx width, patience, help delay, slot remap) are
//     runtime fields of the ring header, so one compiled kernel serves every
//     capacity and thread count; the templates below fix them at compile time for
//     callers that embed a queue in their own structures, as the reference does;
//   * Tail, Head and Threshold each own a 128-byte line;
//   * the private help countdown (nextCheck/nextTid) lives in a dense per-thread
//     array apart from the shared record, so a warp reads it in one coalesced access
//     and helpers never share its line;
//   * a per-slot owner table names the record of the slow-path enqueuer that
//     produced an Enq=0 entry, so finalize_request goes to that record directly
//     instead of scanning all max_threads records (gwf_ring.hpp:316-327), which at
//     2^18 threads costs 2^18 dependent loads per consume.
#pragma once

#include <stdint.h>
#include "gcq_atomics.cuh"

#ifndef WF_CYCLE_BITS
#define WF_CYCLE_BITS 15
#endif
#ifndef WF_HELP_DELAY
#define WF_HELP_DELAY 64
#endif
#ifndef WF_ENQ_PATIENCE
#define WF_ENQ_PATIENCE 128
#endif
#ifndef WF_DEQ_PATIENCE
#define WF_DEQ_PATIENCE 256
#endif
#ifndef GPU_CACHELINE_BYTES
#define GPU_CACHELINE_BYTES 128
#endif

namespace gcq {
namespace gwf {

constexpr uint32_t CYCLE_RANGE = 1u << WF_CYCLE_BITS;
constexpr uint32_t CYCLE_MASK = CYCLE_RANGE - 1;
constexpr uint32_t HALF_CYCLE = CYCLE_RANGE >> 1;
constexpr uint32_t ENTRIES_PER_LINE = GPU_CACHELINE_BYTES / 8;

// Three-way modular cycle comparison: -1 behind, 0 equal, +1 ahead.
__host__ __device__ __forceinline__ int cycle_cmp(uint32_t a, uint32_t b) {
    const uint32_t d = (a - b) & CYCLE_MASK;
    return d == 0 ? 0 : (d < HALF_CYCLE ? 1 : -1);
}

namespace entry {
// Note and Cycle at the top of the word, Safe and Enq below them; 8 bits each
// gives the reference's shifts 56 / 48 / 47 / 46.
constexpr int NOTE_SHIFT = 64 - WF_CYCLE_BITS, CYCLE_SHIFT = 64 - 2 * WF_CYCLE_BITS;
constexpr int SAFE_SHIFT = CYCLE_SHIFT - 1, ENQ_SHIFT = CYCLE_SHIFT - 2;
static_assert(WF_CYCLE_BITS >= 4 && ENQ_SHIFT >= 32, "Note and Cycle must fit above the 32-bit index");
constexpr uint32_t NOTE_NONE = CYCLE_MASK;  // Note = -1: no dequeuer has marked the slot
constexpr uint64_t SAFE_BIT = 1ULL << SAFE_SHIFT;
constexpr uint64_t ENQ_BIT = 1ULL << ENQ_SHIFT;
constexpr uint32_t BOT = 0xFFFFFFFEu;    // empty
constexpr uint32_t BOT_C = 0xFFFFFFFFu;  // consumed
constexpr uint64_t CONSUME_MASK = ENQ_BIT | (uint64_t)BOT_C;
constexpr uint64_t INIT = ((uint64_t)NOTE_NONE << NOTE_SHIFT) | SAFE_BIT | ENQ_BIT | BOT;
__host__ __device__ __forceinline__ uint32_t note(uint64_t e) { return (uint32_t)(e >> NOTE_SHIFT) & CYCLE_MASK; }
__host__ __device__ __forceinline__ uint32_t cycle(uint64_t e) { return (uint32_t)(e >> CYCLE_SHIFT) & CYCLE_MASK; }
__host__ __device__ __forceinline__ bool safe(uint64_t e) { return (e >> SAFE_SHIFT) & 1; }
__host__ __device__ __forceinline__ bool enq(uint64_t e) { return (e >> ENQ_SHIFT) & 1; }
__host__ __device__ __forceinline__ uint32_t index(uint64_t e) { return (uint32_t)e; }
__host__ __device__ __forceinline__ bool empty_index(uint32_t i) { return i >= BOT; }
__host__ __device__ __forceinline__ uint64_t pack(uint32_t n, uint32_t c, bool s, bool q, uint32_t i) {
    return ((uint64_t)(n & CYCLE_MASK) << NOTE_SHIFT) | ((uint64_t)(c & CYCLE_MASK) << CYCLE_SHIFT) |
           ((uint64_t)s << SAFE_SHIFT) | ((uint64_t)q << ENQ_SHIFT) | (uint64_t)i;
}
}  // namespace entry

namespace local {
constexpr uint64_t FIN = 1, INC = 2, CNT_MASK = ~3ULL;
}

// Operation counters of a ring, kept when the library is built with GCQ_STATS=1
// (the reference's GWF_PROFILE counters, gwf_ring.hpp:23-36, which it declares
// but never defines).
namespace stat {
enum : int {
    TRY_ENQ = 0,      // fast-path enqueue attempts
    TRY_DEQ = 1,      // fast-path dequeue attempts
    DEQ_RETRY = 2,    // fast-path dequeue attempts that found nothing and retried
    ENQ_SLOW = 3,     // enqueues that entered the slow path
    DEQ_SLOW = 4,     // dequeues that entered the slow path
    FINALIZE = 5,     // finalize_request calls (consumed Enq=0 entries)
    FINALIZE_SCAN = 6,// finalize_request calls that fell back to the record scan
    DEQ_WAITED = 7,   // dequeues that found their slot filled while waiting for it
    COUNT = 8
};
}
#ifndef GCQ_STATS
#define GCQ_STATS 0
#endif
#if GCQ_STATS
#define GCQ_STAT(c, k) do { if ((c).stats) atomicAdd((unsigned long long*)&(c).stats[k], 1ull); } while (0)
#else
#define GCQ_STAT(c, k) do { } while (0)
#endif

// Shared part of a thread's record: help request + phase-2 record, one 128-B line.
struct alignas(128) record {
    u32a seq1, enqueue, pending, index;
    u64a localTail, initTail, localHead, initHead;
    u32a seq2, _pad0;
    u32a p2_seq1, _pad1;
    u64a p2_local;   // address of the localTail/localHead being incremented
    u64a p2_cnt;
    u32a p2_seq2, _pad2;
};
static_assert(sizeof(record) == 128, "record is one line");

// Private help countdown of a thread (gwf_queue.hpp:260-261).
struct helper_state {
    int32_t nextCheck;
    uint32_t nextTid;
};

// Ring header.  The three hot words sit GCQ_HOT_STRIDE apart; the parameters
// after them are written once by init and only read afterwards.
struct alignas(128) ring {
    u64a Tail;
    char _pad0[GCQ_HOT_STRIDE - 8];
    u64a Head;
    char _pad1[GCQ_HOT_STRIDE - 8];
    int Threshold;
    char _pad2[GCQ_HOT_STRIDE - 4];
    u64a* Entry;            // 2N slots
    record* Record;         // max_threads shared records
    helper_state* Help;     // max_threads private countdowns
    u32a* err;              // sticky error word
    u32a* Owner;            // 2N: 1 + index of the record whose slow-path enqueue last
                            // produced an Enq=0 entry in the slot (0 = none)
    uint32_t order;         // log2 N
    uint32_t thr_bits;      // width of the ThrIdx field
    uint32_t max_threads;   // number of records; thread indices must be below it
    uint32_t help_delay, enq_patience, deq_patience;
    uint32_t remap;         // 1: spread consecutive tickets over different lines
    uint32_t deq_wait;      // re-reads of a not-yet-filled slot before marking it
    uint32_t _pad4;
    u64a* stats;            // operation counters (GCQ_STATS builds), see stat::
};

// Indirection queue with 64-bit payloads (gwf_queue.hpp:338-345): data[N] holds
// the payload of each index.
struct alignas(128) mpmc {
    ring aq;   // allocated indices, starts empty
    ring fq;   // free indices, starts holding 0..N-1
    u64a* data;
    u32a* err;
};

// Parameters of a ring, read once per operation.
struct cfg {
    u64a* entry;
    record* rec;
    helper_state* help;
    u32a* err;
    u32a* owner;
    uint32_t order, thr_bits, max_threads;
    uint32_t help_delay, enq_patience, deq_patience, remap, deq_wait;
    u64a* stats;
    __host__ __device__ __forceinline__ uint32_t slots() const { return 2u << order; }
    __device__ __forceinline__ uint64_t cinc() const { return 1ULL << thr_bits; }
    __device__ __forceinline__ uint64_t null_tid() const { return (1ULL << thr_bits) - 1; }
    __device__ __forceinline__ int32_t threshold_max() const { return 3 * (int32_t)(1u << order) - 1; }
    __device__ __forceinline__ uint64_t counter(uint64_t g) const { return g >> thr_bits; }
    __device__ __forceinline__ uint32_t thridx(uint64_t g) const { return (uint32_t)(g & null_tid()); }
    __device__ __forceinline__ uint64_t pack_global(uint64_t cnt, uint64_t t) const {
        return (cnt << thr_bits) | (t & null_tid());
    }
    __device__ __forceinline__ uint32_t cycle_of(uint64_t t) const { return (uint32_t)(t >> (order + 1)) & CYCLE_MASK; }
    // slot of a ticket: identity (the reference's G-WFQ, CACHE_REMAP unset at
    // gwf_ring.hpp:43-50) or the line-spreading permutation of gwf_queue.hpp:226-230
    __device__ __forceinline__ uint32_t slot_of(uint64_t t) const {
        const uint32_t pos = (uint32_t)t & (slots() - 1);
        if (!remap || slots() < ENTRIES_PER_LINE) return pos;
        return (pos & (ENTRIES_PER_LINE - 1)) * (slots() / ENTRIES_PER_LINE) + pos / ENTRIES_PER_LINE;
    }
    // inverse of slot_of: the ticket position (mod 2N) that maps to slot s
    __host__ __device__ __forceinline__ uint32_t pos_of_slot(uint32_t s) const {
        if (!remap || slots() < ENTRIES_PER_LINE) return s;
        const uint32_t stride = slots() / ENTRIES_PER_LINE;
        return (s % stride) * ENTRIES_PER_LINE + s / stride;
    }
};

__device__ __forceinline__ cfg load_cfg(const ring* q) {
    cfg c;
    c.entry = q->Entry; c.rec = q->Record; c.help = q->Help; c.err = q->err; c.owner = q->Owner;
    c.order = q->order; c.thr_bits = q->thr_bits; c.max_threads = q->max_threads;
    c.help_delay = q->help_delay; c.enq_patience = q->enq_patience; c.deq_patience = q->deq_patience;
    c.remap = q->remap;
    c.deq_wait = q->deq_wait;
    c.stats = q->stats;
    return c;
}

}  // namespace gwf
}  // namespace gcq

// -----------------------------------------------------------------------------
// Compile-time face with the reference's names (gwf_queue.hpp:31-103, 313-345).
// -----------------------------------------------------------------------------
template <int THRIDX_BITS = 14>
struct wf_config {
    static constexpr int COUNTER_BITS = 64 - THRIDX_BITS;
    static constexpr uint32_t MAX_THREADS = (1u << THRIDX_BITS) - 1;
    static constexpr uint64_t NULL_TID = (1ULL << THRIDX_BITS) - 1;
    static constexpr uint64_t THRIDX_MASK = NULL_TID;
    static constexpr uint64_t COUNTER_INC = 1ULL << THRIDX_BITS;
    static constexpr int BITS = THRIDX_BITS;
    static_assert(THRIDX_BITS >= 5 && THRIDX_BITS <= 20, "THRIDX_BITS in [5, 20]");
    static_assert(COUNTER_BITS >= 44, "need at least 44 counter bits");
    __host__ __device__ static uint64_t pack_global(uint64_t counter, uint32_t t) {
        return (counter << THRIDX_BITS) | ((uint64_t)t & THRIDX_MASK);
    }
    __host__ __device__ static uint64_t unpack_counter(uint64_t g) { return g >> THRIDX_BITS; }
    __host__ __device__ static uint32_t unpack_thridx(uint64_t g) { return (uint32_t)(g & THRIDX_MASK); }
    __host__ __device__ static bool has_active_phase2(uint64_t g) { return unpack_thridx(g) != (uint32_t)NULL_TID; }
};
using gwf_1k = wf_config<10>;
using gwf_2k = wf_config<11>;
using gwf_4k = wf_config<12>;
using gwf_8k = wf_config<13>;
using gwf_16k = wf_config<14>;
using gwf_32k = wf_config<15>;
using gwf_64k = wf_config<16>;
using gwf_128k = wf_config<17>;
using gwf_256k = wf_config<18>;
using gwf_512k = wf_config<19>;

namespace wf_entry = gcq::gwf::entry;
namespace wf_local_ptr = gcq::gwf::local;

template <typename Config, uint32_t N_PARAM>
struct wf_t {
    static constexpr uint32_t N = N_PARAM;
    static constexpr uint32_t SLOTS = 2 * N;
    static constexpr int32_t THRESHOLD_MAX = 3 * (int32_t)N - 1;
    static_assert((N & (N - 1)) == 0, "N must be a power of two");
    static_assert(Config::MAX_THREADS <= N, "wf requires k <= n");
    static_assert(gcq::gwf::CYCLE_RANGE > 2u * (WF_HELP_DELAY * (uint64_t)Config::MAX_THREADS / (2 * N) + 3),
                  "cycle bits insufficient for this thread/buffer configuration");
    // Patience 1 would start the slow path without a failed ticket of its own (at
    // counter 0, the same start for every request of a thread); the library's
    // gcq_create refuses it as well.
    static_assert(WF_ENQ_PATIENCE >= 2 && WF_DEQ_PATIENCE >= 2 && WF_HELP_DELAY >= 1,
                  "WF_ENQ_PATIENCE and WF_DEQ_PATIENCE must be at least 2, WF_HELP_DELAY at least 1");
    gcq::gwf::ring hdr;
    gcq::u32a err;
    unsigned long long Entry[SLOTS];
    gcq::gwf::record Record[Config::MAX_THREADS];
    gcq::gwf::helper_state Help[Config::MAX_THREADS];
    gcq::u32a Owner[SLOTS];
};

// Indirection queue (gwf_queue.hpp:338-345) as one object a caller can allocate
// with sizeof and initialise with wf_mpmc_init, with the reference's data[N];
// Enqueue_Ptr/Dequeue_Ptr run the library's code on it.
template <typename Config, uint32_t N_PARAM>
struct wf_mpmc_t {
    using queue_type = wf_t<Config, N_PARAM>;
    queue_type aq;
    queue_type fq;
    gcq::u64a data[N_PARAM];
};
