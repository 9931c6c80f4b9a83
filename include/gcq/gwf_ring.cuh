// G-WFQ algorithm for sm_103a: fast path (SCQ with warp-aggregated tickets),
// cooperative slow path (wCQ's two-phase fetch-and-add), helping, and the 64-bit
// payload indirection.  Every function names the reference routine it restates.
//
// Thread identity: the per-thread calls take the caller's thread index `tid`
// explicitly (it selects the help record; it must be below the ring's
// max_threads).  The reference-named wrappers at the end use wf_tid(), the global
// x index, or WF_TID_EXPR when defined (gwf_ring.hpp:53-63).
#pragma once

#include "gwf_queue.cuh"

namespace gcq {
namespace gwf {

using entry::BOT;
using entry::BOT_C;

// ------------------------------------------------------------------ init
// Thread `gid` of a `nthreads`-wide grid-stride group initialises its share of the
// ring; the reference does the same serially on one thread (gwf_ring.hpp:229-276).
// With `full` the ring starts holding indices 0..N-1 at tickets 2N..3N-1, as
// wf_mpmc_init does for fq (gwf_ring.hpp:278-298).  Each slot's final value is
// computed from the slot itself (inverse of slot_of), so no two threads write the
// same word and no grid-wide ordering is needed.
__device__ inline void init_slice(ring* q, bool full, uint64_t gid, uint64_t nthreads) {
    const cfg c = load_cfg(q);
    const uint32_t slots = c.slots();
    const uint32_t n = 1u << c.order;
    for (uint64_t s = gid; s < slots; s += nthreads) {
        const uint32_t pos = c.pos_of_slot((uint32_t)s);
        c.entry[s] = (full && pos < n)
                         ? entry::pack(entry::NOTE_NONE, c.cycle_of((uint64_t)slots + pos), true, true, pos)
                         : entry::INIT;
        c.owner[s] = 0;
    }
    for (uint64_t i = gid; i < c.max_threads; i += nthreads) {
        record* r = &c.rec[i];
        r->seq1 = 1; r->enqueue = 0; r->pending = 0; r->index = 0;
        r->localTail = 0; r->initTail = 0; r->localHead = 0; r->initHead = 0;
        r->seq2 = 0;
        r->p2_seq1 = 1; r->p2_local = 0; r->p2_cnt = 0; r->p2_seq2 = 0;
        c.help[i].nextCheck = (int32_t)c.help_delay;
        c.help[i].nextTid = (uint32_t)i;
    }
    if (gid == 0) {
        const uint64_t start = slots;
        q->Head = c.pack_global(start, c.null_tid());
        q->Tail = c.pack_global(full ? start + n : start, c.null_tid());
        q->Threshold = full ? c.threshold_max() : -1;
    }
}

// ------------------------------------------------------------------ consume etc.
// finalize_request, gwf_ring.hpp:309-328: set FIN on the slow-path enqueuer whose
// localTail holds ticket h.  The slot's owner entry names that record; the scan of
// all records remains as the fallback when it no longer matches.  A localTail whose
// counter is h with INC set belongs to a request that tried to claim h in the
// cooperative fetch-and-add and lost; the holder has h without INC from before it
// produced the entry until FIN.  The reference's scan stops at the first counter
// match (:322-325): when that is such a loser, the holder never gets FIN while its
// producer is delayed, its helpers take the consumed slot as produced until the slot
// is reused a cycle later, then move on and produce the index a second time.  Both
// lookups here match h without INC.
__device__ inline void finalize_request(const cfg& c, uint64_t h_raw, uint32_t j, uint32_t tid) {
    GCQ_STAT(c, stat::FINALIZE);
    const uint64_t h_local = h_raw << 2;
    // the entry was read relaxed; this fence makes the owner store that preceded
    // the producing (release) CAS visible, so the lookup does not miss and scan
    fence_acq_rel();
    const uint32_t own = ld_rlx(&c.owner[j]);
    if (own != 0 && own <= c.max_threads) {
        const uint64_t lt = ld_acq(&c.rec[own - 1].localTail);
        if ((lt & ~local::FIN) == h_local) {
            cas(&c.rec[own - 1].localTail, h_local, h_local | local::FIN);
            return;
        }
    }
    GCQ_STAT(c, stat::FINALIZE_SCAN);
    uint32_t i = (tid + 1 == c.max_threads) ? 0 : tid + 1;
    while (i != tid) {
        const uint64_t lt = ld_acq(&c.rec[i].localTail);
        if ((lt & ~local::FIN) == h_local) {
            cas(&c.rec[i].localTail, h_local, h_local | local::FIN);
            return;
        }
        i = (i + 1 == c.max_threads) ? 0 : i + 1;
    }
}

// consume, gwf_ring.hpp:335-341.  The caller read `e` with acquire semantics (an
// acquire load, or a relaxed access followed by an acq_rel fence), which orders
// the payload reads after the enqueuer's release; the OR that marks the slot
// consumed needs no ordering of its own, so it is issued without waiting for it
// (an acquire RMW here costs a second L2 round trip on every dequeue).
__device__ __forceinline__ void consume(const cfg& c, uint64_t h_raw, uint32_t j, uint64_t e, uint32_t tid) {
    if (!entry::enq(e)) finalize_request(c, h_raw, j, tid);
    red_or_rlx(&c.entry[j], entry::CONSUME_MASK);
}

// catchup, gwf_ring.hpp:348-371
__device__ inline void catchup(ring* q, const cfg& c, uint64_t tail_raw, uint64_t head_raw) {
    for (int i = 0; i < 32; i++) {
        uint64_t cur = ld_acq(&q->Tail);
        const uint64_t cur_cnt = c.counter(cur);
        if (cur_cnt >= head_raw) break;
        if (cur_cnt != tail_raw) {
            tail_raw = cur_cnt;
            head_raw = c.counter(ld_acq(&q->Head));
            if (tail_raw >= head_raw) break;
            continue;
        }
        if (cas_ok(&q->Tail, cur, c.pack_global(head_raw, c.thridx(cur)))) break;
        head_raw = c.counter(ld_acq(&q->Head));
        tail_raw = c.counter(ld_acq(&q->Tail));
        if (tail_raw >= head_raw) break;
    }
}

// ------------------------------------------------------------------ fast path
// try_enq, gwf_ring.hpp:382-414, on ticket T (a Tail counter value).  0 on
// success, else T.
// Publish: the caller wrote what the index refers to before this call, and the
// entry CAS is acq_rel -- release orders those writes before the index, acquire
// orders the Threshold reset after the CAS.  Without Publish the caller has ordered
// its earlier accesses itself, and the CAS is acquire only: a release costs a
// further L2 round trip on this GPU, an acquire nothing measurable.
template <bool Publish = true>
__device__ inline uint64_t try_enq_at(ring* q, const cfg& c, uint32_t index, uint64_t T) {
    GCQ_STAT(c, stat::TRY_ENQ);
    const uint32_t tcyc = c.cycle_of(T);
    const uint32_t j = c.slot_of(T);
    // In steady state the slot holds the previous cycle's consumed entry (Note
    // untouched by any slow path, safe, index consumed): try the CAS against that
    // value first.  A match means the enqueue conditions hold; a mismatch returns
    // the slot's current value, exactly what the load of gwf_ring.hpp:394 would
    // have read, so the code below continues from it.  Saves one L2 round trip.
    uint64_t E = entry::pack(entry::NOTE_NONE, tcyc - 1, true, true, BOT_C);
    if (cas_upd_ord<Publish>(&c.entry[j], &E, entry::pack(entry::NOTE_NONE, tcyc, true, true, index))) {
        reset_threshold(&q->Threshold, c.threshold_max());
        return 0;
    }
    for (uint32_t spin = 0; spin < GCQ_SPIN_LIMIT; ++spin) {
        const uint32_t ecyc = entry::cycle(E);
        const uint32_t eidx = entry::index(E);
        if (cycle_cmp(ecyc, tcyc) >= 0 || !entry::empty_index(eidx)) return T;
        if (!entry::safe(E)) {
            dekker_fence();
            if (c.counter(ld_rlx(&q->Head)) > T) return T;
        }
        const uint64_t nw = entry::pack(entry::note(E), tcyc, true, true, index);
        if (!cas_upd_ord<Publish>(&c.entry[j], &E, nw)) continue;
        reset_threshold(&q->Threshold, c.threshold_max());
        return 0;
    }
    raise_error(c.err, ERR_SPIN);
    return T;
}
template <bool Publish = true>
__device__ __forceinline__ uint64_t try_enq(ring* q, const cfg& c, uint32_t index) {
    return try_enq_at<Publish>(q, c, index, c.counter(warp_ticket(&q->Tail, c.cinc())));
}

// An enqueue ticket taken ahead of need and then not used (the operation it was for
// found the queue full): the slot is marked passed at the ticket's cycle, as the
// dequeuer holding the same ticket would mark it, so that dequeuer does not wait
// for an index that will not come.  A slot holding an older index is left for that
// dequeuer.  Not waited for; a failed CAS means the slot moved on and needs nothing.
// The dequeuer that reaches the ticket fails there and spends one unit of Threshold
// with no element behind it, a failure SCQ's 3n - 1 bound does not count; the
// abandoning thread resets Threshold, as an enqueue does, so the bound still holds
// from there on (callers also take such tickets at most once per thread between two
// successful enqueues, see enqueue_ptr).
__device__ inline void abandon_enq_ticket(ring* q, uint64_t T_raw) {
    const cfg c = load_cfg(q);
    const uint64_t T = c.counter(T_raw);
    const uint32_t tcyc = c.cycle_of(T);
    const uint32_t j = c.slot_of(T);
    const uint64_t E = ld_rlx(&c.entry[j]);
    if (cycle_cmp(entry::cycle(E), tcyc) < 0 && entry::empty_index(entry::index(E)))
        cas_rlx(&c.entry[j], E, entry::pack(entry::note(E), tcyc, entry::safe(E), true, BOT));
    reset_threshold(&q->Threshold, c.threshold_max());
}

// try_deq, gwf_ring.hpp:421-472.  0 when finished (*out = index, or BOT if the
// queue is empty), else the ticket tried.
// With PF the same lanes also take a ticket of the counter pf_ctr (another ring's
// Tail, for the enqueue that follows this dequeue): its fetch-and-add is issued
// together with this ticket's slot load, so its round trip overlaps the load's;
// *pf_raw receives the raw counter word.
template <bool PF = false>
__device__ inline uint64_t try_deq(ring* q, const cfg& c, uint32_t* out, uint32_t tid, u64a* pf_ctr = nullptr,
                                   uint64_t* pf_raw = nullptr) {
    GCQ_STAT(c, stat::TRY_DEQ);
    const uint64_t H = c.counter(warp_ticket(&q->Head, c.cinc()));
    const uint32_t hcyc = c.cycle_of(H);
    const uint32_t j = c.slot_of(H);
    ticket_req pf;
    if (PF && pf_ctr) pf = ticket_issue(pf_ctr, c.cinc());
    uint64_t E = ld_acq(&c.entry[j]);   // acquire: see consume
    if (PF && pf_ctr) *pf_raw = ticket_take(pf, c.cinc());
    // The slot of an earlier cycle with no index: the enqueuer holding this ticket
    // may be about to fill it.  Marking it now would make that enqueuer retry with a
    // new ticket, and this dequeuer too; re-reading it a few times first (bounded,
    // so the operation stays wait-free) avoids that collision.
    if (c.deq_wait && cycle_cmp(entry::cycle(E), hcyc) < 0 && entry::empty_index(entry::index(E))) {
        uint32_t ns = 32;
        for (uint32_t w = 0; w < c.deq_wait; ++w) {
            __nanosleep(ns);
            ns = ns < 1024 ? ns * 2 : ns;
            E = ld_acq(&c.entry[j]);
            if (!(cycle_cmp(entry::cycle(E), hcyc) < 0 && entry::empty_index(entry::index(E)))) {
                GCQ_STAT(c, stat::DEQ_WAITED);
                break;
            }
        }
    }
    uint32_t spin = 0;
    for (;; ++spin) {
        const uint32_t ecyc = entry::cycle(E);
        const uint32_t eidx = entry::index(E);
        if (cycle_cmp(ecyc, hcyc) == 0 && !entry::empty_index(eidx)) {
            if (spin) fence_acq_rel();   // E came from a relaxed CAS
            consume(c, H, j, E, tid);
            *out = eidx;
            return 0;
        }
        if (cycle_cmp(ecyc, hcyc) >= 0) break;
        if (spin >= GCQ_SPIN_LIMIT) { raise_error(c.err, ERR_SPIN); break; }
        const uint64_t nw = entry::empty_index(eidx)
                                ? entry::pack(entry::note(E), hcyc, entry::safe(E), true, BOT)
                                : entry::pack(entry::note(E), ecyc, false, entry::enq(E), eidx);
        if (cas_upd_rlx(&c.entry[j], &E, nw)) break;
    }
    dekker_fence();
    const uint64_t T = c.counter(ld_rlx(&q->Tail));
    if (T <= H + 1) {
        catchup(q, c, T, H + 1);
        fetch_add(&q->Threshold, -1);
        *out = BOT;
        return 0;
    }
    if (fetch_add(&q->Threshold, -1) <= 0) {
        *out = BOT;
        return 0;
    }
    GCQ_STAT(c, stat::DEQ_RETRY);
    return H;
}

// ------------------------------------------------------------------ slow path
// prepare_phase2, gwf_ring.hpp:486-504: publish (local, cnt) under a sequence pair.
__device__ __forceinline__ void prepare_phase2(record* me, u64a* localp, uint64_t cnt_local) {
    const uint32_t seq = ld_rlx(&me->p2_seq1) + 1;
    st_rlx(&me->p2_seq1, seq);
    fence_acq_rel();
    st_rlx(&me->p2_local, (uint64_t)(uintptr_t)localp);
    st_rlx(&me->p2_cnt, cnt_local);
    st_rel(&me->p2_seq2, seq);
}

// slow_faa, gwf_ring.hpp:523-639: cooperative fetch-and-add on Tail/Head that
// increments the global counter exactly once per helper group.  Returns false
// when the request was finalised (FIN), true when *v holds a fresh ticket.
__device__ inline bool slow_faa(ring* q, const cfg& c, u64a* globalp, u64a* localp, uint64_t* v,
                                int* thld, uint32_t tid) {
    record* my = &c.rec[tid];
    uint64_t cnt_local = 0, cnt_raw = 0;
    bool global_ok = false;
    uint32_t spin = 0;
    do {
        if (++spin > GCQ_SPIN_LIMIT) {
            raise_error(c.err, ERR_SPIN);
            *v = ld_acq(localp) | local::FIN;
            return false;
        }
        const uint64_t lc = ld_acq(localp);
        if (lc & local::FIN) { *v = lc; return false; }
        uint64_t gp = ld_acq(globalp);
        const uint32_t gt = c.thridx(gp);
        if (gt != (uint32_t)c.null_tid()) {
            // help the phase-2 request named by the global word (gwf_ring.hpp:550-590).
            // A thread has one phase-2 record for both counters, and a counter word
            // keeps a thread index after that thread's own clean-up CAS lost to a
            // fetch-and-add, so the record read here may describe an increment of
            // the other counter, or a later one of this counter whose CAS has not
            // happened.  Clearing INC for it hands that thread a ticket the counter
            // also gives to a fast-path operation: two enqueuers on one ticket lose
            // a value, two dequeuers duplicate one (the reference clears it whenever
            // the record's seqlock matches).  INC is cleared only when the record's
            // local is fed by this counter and the word, read again after the
            // record, still names the thread past the record's count -- true for the
            // phase 2 of that thread's successful CAS until its index is cleaned,
            // and the first cleaner clears INC before it cleans.
            record* hr = &c.rec[gt];
            const uint32_t seq = ld_acq(&hr->p2_seq2);
            u64a* p2_local = (u64a*)(uintptr_t)ld_rlx(&hr->p2_local);
            const uint64_t p2_cnt = ld_rlx(&hr->p2_cnt);
            fence_acq_rel();
            const uint32_t seq1 = ld_acq(&hr->p2_seq1);
            bool help_ok = seq1 == seq && p2_local;
            if (help_ok) {
                const uint64_t g2 = ld_acq(globalp);
                const uintptr_t base = (uintptr_t)(globalp == &q->Tail ? &c.rec[0].localTail : &c.rec[0].localHead);
                const uintptr_t a = (uintptr_t)p2_local;
                help_ok = a >= base && (a - base) % sizeof(record) == 0 && (a - base) / sizeof(record) < c.max_threads &&
                          c.thridx(g2) == gt && c.counter(g2) > (p2_cnt >> 2);
            }
            if (help_ok) cas(p2_local, p2_cnt | local::INC, p2_cnt);
            const uint64_t clean = c.pack_global(c.counter(gp), c.null_tid());
            if (!cas_ok(globalp, gp, clean)) continue;
            gp = clean;
        }
        cnt_raw = c.counter(gp);
        cnt_local = cnt_raw << 2;
        uint64_t vc = *v;
        if (!cas_upd(localp, &vc, cnt_local | local::INC)) {
            *v = vc;
            if (vc & local::FIN) return false;
            if (!(vc & local::INC)) return true;
            cnt_local = vc & local::CNT_MASK;
            cnt_raw = cnt_local >> 2;
        } else {
            *v = cnt_local | local::INC;
        }
        prepare_phase2(my, localp, cnt_local);
        global_ok = cas_ok(globalp, c.pack_global(cnt_raw, c.null_tid()), c.pack_global(cnt_raw + 1, tid));
    } while (!global_ok);
    if (thld) fetch_add(thld, -1);
    cas(localp, cnt_local | local::INC, cnt_local);
    cas(globalp, c.pack_global(cnt_raw + 1, tid), c.pack_global(cnt_raw + 1, c.null_tid()));
    *v = cnt_local;
    return true;
}

// try_enq_slow, gwf_ring.hpp:650-705
__device__ inline bool try_enq_slow(ring* q, const cfg& c, uint64_t T_raw, uint32_t index, record* r) {
    const uint32_t tcyc = c.cycle_of(T_raw);
    const uint32_t j = c.slot_of(T_raw);
    uint64_t P = ld_acq(&c.entry[j]);
    for (uint32_t spin = 0; spin < GCQ_SPIN_LIMIT; ++spin) {
        const uint32_t ecyc = entry::cycle(P), enote = entry::note(P), eidx = entry::index(P);
        if (cycle_cmp(ecyc, tcyc) < 0 && cycle_cmp(enote, tcyc) < 0) {
            bool skip = !entry::empty_index(eidx);
            if (!skip && !entry::safe(P)) {
                dekker_fence();
                skip = c.counter(ld_acq(&q->Head)) > T_raw;
            }
            if (skip) {
                // advance Note so later helpers skip this slot too
                const uint64_t nn = entry::pack(tcyc, ecyc, entry::safe(P), entry::enq(P), eidx);
                if (!cas_upd(&c.entry[j], &P, nn)) continue;
                return false;
            }
            // two-step insertion: Enq=0 first, flipped to 1 once FIN is set; the
            // owner entry is published by the release half of the CAS below
            st_rlx(&c.owner[j], (uint32_t)(r - c.rec) + 1u);
            const uint64_t nn = entry::pack(enote, tcyc, true, false, index);
            if (!cas_upd(&c.entry[j], &P, nn)) continue;
            const uint64_t T_local = T_raw << 2;
            if (cas_ok(&r->localTail, T_local, T_local | local::FIN))
                cas(&c.entry[j], nn, entry::pack(enote, tcyc, true, true, index));
            reset_threshold(&q->Threshold, c.threshold_max());
            return true;
        }
        // The slot is at our cycle: produced for this request (our index, or
        // consumed since, index ⊥c) -- or passed by the dequeuer that holds the same
        // ticket, which marks it ⊥ at our cycle.  gwf_ring.hpp:697-704 takes every
        // cycle match as "already produced", which loses the element in the second
        // case; here it fails the ticket, as the fast path does, and the request
        // takes another.
        return cycle_cmp(ecyc, tcyc) == 0 && (eidx == index || eidx == BOT_C);
    }
    raise_error(c.err, ERR_SPIN);
    return true;
}

// try_deq_slow, gwf_ring.hpp:712-769
__device__ inline bool try_deq_slow(ring* q, const cfg& c, uint64_t H_raw, record* r) {
    const uint32_t hcyc = c.cycle_of(H_raw);
    const uint32_t j = c.slot_of(H_raw);
    uint64_t P = ld_acq(&c.entry[j]);
    for (uint32_t spin = 0;; ++spin) {
        if (spin >= GCQ_SPIN_LIMIT) { raise_error(c.err, ERR_SPIN); break; }
        const uint32_t ecyc = entry::cycle(P), enote = entry::note(P), eidx = entry::index(P);
        if (cycle_cmp(ecyc, hcyc) == 0 && !entry::empty_index(eidx)) {
            const uint64_t H_local = H_raw << 2;
            const uint64_t prev = cas(&r->localHead, H_local, H_local | local::FIN);
            return prev == H_local || (prev & local::FIN) != 0;
        }
        uint32_t n_note = enote;
        uint64_t val = entry::pack(n_note, hcyc, entry::safe(P), true, BOT);
        if (!entry::empty_index(eidx)) {
            if (cycle_cmp(ecyc, hcyc) < 0 && cycle_cmp(enote, hcyc) < 0) {
                const uint64_t nn = entry::pack(hcyc, ecyc, entry::safe(P), entry::enq(P), eidx);
                if (!cas_upd(&c.entry[j], &P, nn)) continue;
                n_note = hcyc;
            }
            val = entry::pack(n_note, ecyc, false, entry::enq(P), eidx);
        }
        if (cycle_cmp(ecyc, hcyc) < 0) {
            if (!cas_upd(&c.entry[j], &P, val)) continue;
        }
        break;
    }
    dekker_fence();
    const uint64_t T = c.counter(ld_acq(&q->Tail));
    if (T <= H_raw + 1) catchup(q, c, T, H_raw + 1);
    // Done only when the request is finished: at this ticket (this CAS) or already
    // (FIN).  gwf_ring.hpp:763-766 reports done whatever the CAS found; when another
    // helper has moved the request to a later ticket, the owner then stops and
    // gathers at that unfinished ticket (empty), and the helper that finishes the
    // request there later claims an element nobody returns.
    if (ld_acq(&q->Threshold) < 0) {
        const uint64_t H_local = H_raw << 2;
        const uint64_t prev = cas(&r->localHead, H_local, H_local | local::FIN);
        return prev == H_local || (prev & local::FIN) != 0;
    }
    return false;
}

// enqueue_slow / dequeue_slow, gwf_ring.hpp:775-802.  A helper (seq != NO_SEQ)
// stops once the request it read is over: a request's localTail is published with
// a release store after the previous request's seq1 increment, so a helper that
// obtained a ticket from a newer request sees seq1 moved and does not produce the
// old request's index there.
constexpr uint32_t NO_SEQ = 0xFFFFFFFFu;
__device__ inline void enqueue_slow(ring* q, const cfg& c, uint64_t v, uint32_t index, record* r, uint32_t tid,
                                    uint32_t seq = NO_SEQ) {
    while (slow_faa(q, c, &q->Tail, &r->localTail, &v, nullptr, tid)) {
        if (seq != NO_SEQ && ld_acq(&r->seq1) != seq) break;
        if (try_enq_slow(q, c, v >> 2, index, r)) break;
    }
}
__device__ inline void dequeue_slow(ring* q, const cfg& c, uint64_t v, record* r, uint32_t tid) {
    while (slow_faa(q, c, &q->Head, &r->localHead, &v, &q->Threshold, tid))
        if (try_deq_slow(q, c, v >> 2, r)) break;
}

// ------------------------------------------------------------------ helping
// help_enqueue / help_dequeue / help_threads, gwf_ring.hpp:808-861
__device__ inline void help_enqueue(ring* q, const cfg& c, record* thr, uint32_t tid) {
    const uint32_t seq = ld_acq(&thr->seq2);
    const uint32_t is_enq = ld_rlx(&thr->enqueue);
    const uint32_t idx = ld_rlx(&thr->index);
    const uint64_t init_tail = ld_rlx(&thr->initTail);
    fence_acq_rel();
    if (is_enq && ld_rlx(&thr->seq1) == seq) enqueue_slow(q, c, init_tail, idx, thr, tid, seq);
}
__device__ inline void help_dequeue(ring* q, const cfg& c, record* thr, uint32_t tid) {
    const uint32_t seq = ld_acq(&thr->seq2);
    const uint32_t is_enq = ld_rlx(&thr->enqueue);
    const uint64_t init_head = ld_rlx(&thr->initHead);
    fence_acq_rel();
    if (!is_enq && ld_rlx(&thr->seq1) == seq) dequeue_slow(q, c, init_head, thr, tid);
}
// With `reg` the countdown is the caller's copy (a thread_ctx below, kept in
// registers for the kernel's duration) instead of the thread's slot in c.help.
__device__ __forceinline__ void help_threads(ring* q, const cfg& c, uint32_t tid, helper_state* reg = nullptr) {
    helper_state hs = reg ? *reg : c.help[tid];
    if (--hs.nextCheck != 0) {
        if (reg) reg->nextCheck = hs.nextCheck;
        else c.help[tid].nextCheck = hs.nextCheck;
        return;
    }
    record* thr = &c.rec[hs.nextTid];
    if (ld_acq(&thr->pending)) {
        if (ld_rlx(&thr->enqueue)) help_enqueue(q, c, thr, tid);
        else help_dequeue(q, c, thr, tid);
    }
    hs.nextCheck = (int32_t)c.help_delay;
    hs.nextTid = (hs.nextTid + 1 == c.max_threads) ? 0 : hs.nextTid + 1;
    if (reg) *reg = hs;
    else c.help[tid] = hs;
}

// ------------------------------------------------------------------ top level
// Enqueue_wf, gwf_ring.hpp:1234-1284 (Publish: see try_enq).  first_raw, when
// not 0, is a Tail ticket the caller already took (try_deq's prefetch): the first
// fast-path attempt uses it.  Tickets start at 2N, so 0 never names one.
// HelpAfter moves the operation's help check (help_threads) from before its own
// work to after it.  A release CAS waits for every earlier write of the thread, and
// the help check writes the thread's countdown: after the CAS, that store is not
// waited for.  Each operation still makes one help check, so a peer's request is
// still visited within help_delay operations of every thread.
template <bool Publish = true, bool HelpAfter = false>
__device__ inline void enqueue(ring* q, uint32_t index, uint32_t tid, uint64_t first_raw = 0,
                               helper_state* hs = nullptr) {
    const cfg c = load_cfg(q);
    if (tid >= c.max_threads) { raise_error(c.err, ERR_TID); return; }
    if (!HelpAfter) help_threads(q, c, tid, hs);
    uint64_t tail = 0;
    for (uint32_t count = c.enq_patience; --count != 0;) {
        if (first_raw) {
            tail = try_enq_at<Publish>(q, c, index, c.counter(first_raw));
            first_raw = 0;
        } else {
            tail = try_enq<Publish>(q, c, index);
        }
        if (tail == 0) {
            if (HelpAfter) help_threads(q, c, tid, hs);
            return;
        }
    }
    GCQ_STAT(c, stat::ENQ_SLOW);
    record* r = &c.rec[tid];
    const uint32_t seq = ld_rlx(&r->seq1);
    const uint64_t tail_local = tail << 2;
    st_rel(&r->localTail, tail_local);   // after the previous request's seq1 increment
    st_rlx(&r->initTail, tail_local);
    st_rlx(&r->index, index);
    st_rlx(&r->enqueue, 1u);
    st_rel(&r->seq2, seq);
    st_rel(&r->pending, 1u);
    enqueue_slow(q, c, tail_local, index, r, tid);
    st_rel(&r->pending, 0u);
    st_rel(&r->seq1, seq + 1);
    if (HelpAfter) help_threads(q, c, tid, hs);
}

// Dequeue_wf, gwf_ring.hpp:1286-1356.  Returns the index or BOT when empty.
// With PF the first fast-path attempt also takes a ticket of pf_ctr into *pf_raw
// (see try_deq); *pf_raw stays 0 when the dequeue returns before taking one.
// Empty exit before a Head ticket (GCQ_DEQ_EMPTY_CHECK): the dequeue returns BOT
// when no enqueue ticket lies beyond the Head counter (Head read with acquire, then
// Tail).  At the Tail read Tail <= Head: every entry whose enqueue has completed has
// a dequeuer holding its ticket, concurrent with this operation, so the queue is
// empty at that instant -- the exit SCQ takes after a failed ticket when
// Tail <= H + 1 (gwf_ring.hpp:452-460), taken without spending a ticket.  It is
// taken before every retry, and before the first ticket when the caller says its
// previous dequeue on this ring found the queue empty (first_check, from a
// thread_ctx).  Without it, consumers that outnumber producers spend tickets on an
// empty queue, drive Head ahead of Tail and make the producers' tickets fail in
// turn: split mode with 25 % producers at 8192 threads ran at 81 Mops/s with 115 M
// retries in 130 M attempts, against 1072 Mops/s and 456 retries with the exit
// before every ticket.  Before every first ticket unconditionally, the dependent
// loads halved balanced mode (18.8 against 35.8 Gops/s at 262144 threads), and
// triggered by the ring's Threshold being below its maximum they sent balanced
// mode at 262144 threads, stochastically, into a regime of 5.2 ms per chunk
// against 1.9.  0 turns it off.
#ifndef GCQ_DEQ_EMPTY_CHECK
#define GCQ_DEQ_EMPTY_CHECK 1
#endif
// When Head is ahead of Tail (dequeuers spent tickets past the last enqueue), the
// exit moves Tail up to Head, as SCQ's failing dequeuer does (catchup): otherwise the
// producers' next tickets land on the passed slots and fail one by one.
__device__ __forceinline__ bool seen_empty(ring* q, const cfg& c) {
    const uint64_t h = c.counter(ld_acq(&q->Head));
    const uint64_t t = c.counter(ld_rlx(&q->Tail));
    if (t > h) return false;
    if (t < h) catchup(q, c, t, h);
    return true;
}
// hs: the caller's register copy of its help countdown (thread_ctx), or null.
// skip_check: the thread's own last operation on this ring was an enqueue that
// left Threshold at its maximum, so the pre-check is skipped; it is a hint that
// spares tickets on an empty queue, and the dequeue stays correct without it.
// first_check: the thread's last dequeue on this ring found it empty, so the empty
// exit is tried before the first ticket too.
template <bool PF = false>
__device__ inline uint32_t dequeue(ring* q, uint32_t tid, u64a* pf_ctr = nullptr, uint64_t* pf_raw = nullptr,
                                   helper_state* hs = nullptr, bool skip_check = false, bool first_check = false) {
    const cfg c = load_cfg(q);
    if (!skip_check && ld_rlx(&q->Threshold) < 0) return BOT;
    if (GCQ_DEQ_EMPTY_CHECK && first_check && seen_empty(q, c)) return BOT;
    if (tid >= c.max_threads) { raise_error(c.err, ERR_TID); return BOT; }
    help_threads(q, c, tid, hs);
    uint32_t out = BOT;
    uint64_t head = 0;
    if (PF) {
        head = try_deq<true>(q, c, &out, tid, pf_ctr, pf_raw);
        if (head == 0) return out;
        if (GCQ_DEQ_EMPTY_CHECK && seen_empty(q, c)) return BOT;
    }
    for (uint32_t count = c.deq_patience - (PF ? 1u : 0u); --count != 0;) {
        head = try_deq(q, c, &out, tid);
        if (head == 0) return out;
        if (GCQ_DEQ_EMPTY_CHECK && seen_empty(q, c)) return BOT;
    }
    GCQ_STAT(c, stat::DEQ_SLOW);
    record* r = &c.rec[tid];
    const uint32_t seq = ld_rlx(&r->seq1);
    const uint64_t head_local = head << 2;
    st_rlx(&r->localHead, head_local);
    st_rlx(&r->initHead, head_local);
    st_rlx(&r->enqueue, 0u);
    st_rel(&r->seq2, seq);
    st_rel(&r->pending, 1u);
    dequeue_slow(q, c, head_local, r, tid);
    st_rel(&r->pending, 0u);
    st_rel(&r->seq1, seq + 1);
    // gather the slow-path result (gwf_ring.hpp:1340-1355)
    const uint64_t h_raw = ld_acq(&r->localHead) >> 2;
    const uint32_t j = c.slot_of(h_raw);
    const uint64_t e = ld_acq(&c.entry[j]);
    if (cycle_cmp(entry::cycle(e), c.cycle_of(h_raw)) == 0 && !entry::empty_index(entry::index(e))) {
        consume(c, h_raw, j, e, tid);
        return entry::index(e);
    }
    return BOT;
}

// A hint for polling consumers, not a queue operation (the reference has none):
// true when the ring's Tail counter is ahead of its Head counter.  It reads two
// words and changes nothing, so a consumer that polls an idle queue through it
// takes no Head ticket, marks no slot and leaves the Threshold alone.  An entry
// enqueued at ticket T and not yet dequeued implies Head <= T < Tail, so the hint
// turns true once such an entry exists; it may also be true for an empty queue
// (a dequeue then simply fails).
__device__ __forceinline__ bool maybe_nonempty(const ring* q) {
    const uint32_t b = q->thr_bits;
    return (ld_rlx(&q->Tail) >> b) > (ld_rlx(&q->Head) >> b);
}

// A stronger poll hint (the reference has none): true when the slot of the next
// Head ticket already holds an index of that ticket's cycle, an entry a dequeue
// would take now.  A poller that takes Head tickets only then does not race the
// enqueuers for slots they are still filling -- each such race marks the slot and
// makes both sides retry, and a slow-path enqueue, whose tickets come one CAS at a
// time, can lose every one of them to a crowd of pollers.  An enqueuer can also
// give a ticket up and leave its slot empty for good, so a poller that keeps
// seeing Tail ahead of Head with an unfilled head slot should dequeue anyway after
// a few polls (the dequeue marks the slot and moves on).
__device__ __forceinline__ bool head_ready(const ring* q) {
    const cfg c = load_cfg(q);
    const uint64_t h = c.counter(ld_rlx(&q->Head));
    const uint64_t e = ld_rlx(&c.entry[c.slot_of(h)]);
    return cycle_cmp(entry::cycle(e), c.cycle_of(h)) == 0 && !entry::empty_index(entry::index(e));
}

// Dequeue for polling consumers (the reference has none): at most `tries` fast-path
// attempts, no help record, no slow path.  BOT when they find the queue empty or
// run out; the caller polls again.  A consumer that polls an idle queue through
// the wait-free dequeue publishes a slow-path request after deq_patience failures,
// and with many pollers those requests race the dequeue front without end.
__device__ inline uint32_t try_dequeue(ring* q, uint32_t tid, uint32_t tries) {
    if (ld_rlx(&q->Threshold) < 0) return BOT;
    const cfg c = load_cfg(q);
    uint32_t out = BOT;
    for (uint32_t k = 0; k < tries; ++k)
        if (try_deq(q, c, &out, tid) == 0) return out;
    return BOT;
}

// Enqueue_Ptr / Dequeue_Ptr, gwf_ring.hpp:1362-1380.  false = full / empty.
// The reference stores the payload, fences, then enqueues the index, so a consumer
// that dequeues a value also sees every write the producer made before its
// Enqueue_Ptr (a queue of pointers to filled records).  Here the index's enqueue
// to aq is an acq_rel CAS: its release orders the producer's earlier writes and
// the payload store before the index, and the consumer's acquire load of the aq
// entry orders its payload read and later reads after them.  The index's return
// to fq carries a release too (it orders the consumer's payload read before the
// next producer's store; see take_and_return).  Measured against the earlier form
// -- payloads in flagged 128-bit cells written by an exchange the producer did not
// wait for, and an acquire-only aq enqueue that published nothing else -- this one
// is faster as well: 1.70 against 1.99 ms per chunk (balanced, 262144 threads,
// capacity 2^20, L2 flushed).
// With GCQ_TICKET_PREFETCH (default) each operation takes its second ring's ticket
// while the first ring's access is in flight: Enqueue_Ptr issues the aq Tail
// fetch-and-add beside the fq slot load, Dequeue_Ptr issues the fq Tail
// fetch-and-add beside the payload read.  Each saves one dependent L2 round trip.
//
// The operations work on a view of an indirection queue -- its two rings, its
// payload array and its error word -- so the library's queue (mpmc) and the
// compile-time wf_mpmc_t below run the same code.
#ifndef GCQ_TICKET_PREFETCH
#define GCQ_TICKET_PREFETCH 1
#endif
struct mpmc_view {
    ring* aq;
    ring* fq;
    u64a* data;
    u32a* err;
};
__device__ __forceinline__ mpmc_view view_of(mpmc* q) { return mpmc_view{&q->aq, &q->fq, q->data, q->err}; }

// Per-thread state of a thread that runs many operations on one queue within a
// kernel: its two help countdowns (the reference keeps them in the thread's record,
// gwf_queue.hpp:260-261; here they stay in registers between ctx_load and
// ctx_store) and, per ring, whether its last operation there was an enqueue that
// left Threshold at its maximum (the next dequeue skips the pre-check).
struct thread_ctx {
    helper_state help_aq, help_fq;
    bool aq_fresh, fq_fresh;   // last operation on the ring: this thread's enqueue
    bool aq_empty, fq_empty;   // last dequeue on the ring: found it empty
};
__device__ __forceinline__ thread_ctx ctx_load(const mpmc_view& q, uint32_t tid) {
    thread_ctx x;
    x.help_aq = q.aq->Help[tid];
    x.help_fq = q.fq->Help[tid];
    x.aq_fresh = x.fq_fresh = false;
    x.aq_empty = x.fq_empty = false;
    return x;
}
__device__ __forceinline__ void ctx_store(const mpmc_view& q, uint32_t tid, const thread_ctx& x) {
    q.aq->Help[tid] = x.help_aq;
    q.fq->Help[tid] = x.help_fq;
}

__device__ __forceinline__ bool enqueue_ptr(const mpmc_view& q, uint64_t value, uint32_t tid,
                                            thread_ctx* x = nullptr) {
#if GCQ_TICKET_PREFETCH
    // The aq ticket is taken ahead of need only by a thread with a context whose last
    // free-ring dequeue succeeded.  A ticket taken for an operation that then finds
    // the queue full is abandoned; a thread that kept prefetching while the queue
    // stayed full would drive Tail ahead of the elements by one abandoned ticket per
    // attempt, the dequeuers failing on them would spend Threshold below zero, and
    // dequeues would report a full queue empty (a CPU model of this path lost values
    // that way).  So a thread abandons at most one ticket between two successful
    // enqueues, and callers without a context take no aq ticket ahead of need.
    uint64_t aq_raw = 0;
    const bool pf = x && !x->fq_empty;
    const uint32_t idx = dequeue<true>(q.fq, tid, pf ? &q.aq->Tail : nullptr, &aq_raw, x ? &x->help_fq : nullptr,
                                       x && x->fq_fresh, x && x->fq_empty);
    if (x) {
        x->fq_fresh = false;
        x->fq_empty = (idx == BOT);
    }
    if (idx == BOT) {
        if (aq_raw) abandon_enq_ticket(q.aq, aq_raw);
        return false;
    }
    st_rlx(&q.data[idx], value);
    enqueue<true>(q.aq, idx, tid, aq_raw, x ? &x->help_aq : nullptr);
    if (x) x->aq_fresh = true;
#else
    const uint32_t idx = dequeue(q.fq, tid, nullptr, nullptr, x ? &x->help_fq : nullptr, x && x->fq_fresh,
                                 x && x->fq_empty);
    if (x) {
        x->fq_fresh = false;
        x->fq_empty = (idx == BOT);
    }
    if (idx == BOT) return false;
    st_rlx(&q.data[idx], value);
    enqueue<true>(q.aq, idx, tid, 0, x ? &x->help_aq : nullptr);
    if (x) x->aq_fresh = true;
#endif
    return true;
}
// Read the payload of index idx and return idx to fq.  The return's release is
// that of an acq_rel CAS.  (An acq_rel fence right after the read, then an acquire
// CAS, measured slower.)  The return's help check runs after its CAS
// (GCQ_RETURN_HELP_AFTER), so the release does not wait for the store of the help
// countdown.
#ifndef GCQ_RETURN_HELP_AFTER
#define GCQ_RETURN_HELP_AFTER 1
#endif
__device__ __forceinline__ uint64_t take_and_return(const mpmc_view& q, uint32_t idx, uint32_t tid,
                                                    thread_ctx* x = nullptr) {
    // the aq entry's acquire load (or, opt-in, this acquire) orders the read
#if GCQ_TICKET_PREFETCH
    const uint64_t inc = 1ULL << q.fq->thr_bits;
    const ticket_req t = ticket_issue(&q.fq->Tail, inc);
    const uint64_t v = GCQ_ACQUIRE_ONLY_RETURN ? ld_acq(&q.data[idx]) : ld_rlx(&q.data[idx]);
    const uint64_t fq_raw = ticket_take(t, inc);
#else
    const uint64_t v = GCQ_ACQUIRE_ONLY_RETURN ? ld_acq(&q.data[idx]) : ld_rlx(&q.data[idx]);
    const uint64_t fq_raw = 0;
#endif
    enqueue<!GCQ_ACQUIRE_ONLY_RETURN, GCQ_RETURN_HELP_AFTER>(q.fq, idx, tid, fq_raw, x ? &x->help_fq : nullptr);
    if (x) x->fq_fresh = true;
    return v;
}
__device__ __forceinline__ bool dequeue_ptr(const mpmc_view& q, uint64_t* out, uint32_t tid,
                                            thread_ctx* x = nullptr) {
    const uint32_t idx = dequeue(q.aq, tid, nullptr, nullptr, x ? &x->help_aq : nullptr, x && x->aq_fresh,
                                 x && x->aq_empty);
    if (x) {
        x->aq_fresh = false;
        x->aq_empty = (idx == BOT);
    }
    if (idx == BOT) return false;
    *out = take_and_return(q, idx, tid, x);
    return true;
}
__device__ __forceinline__ bool enqueue_ptr(mpmc* q, uint64_t value, uint32_t tid) {
    return enqueue_ptr(view_of(q), value, tid);
}
__device__ __forceinline__ bool dequeue_ptr(mpmc* q, uint64_t* out, uint32_t tid) {
    return dequeue_ptr(view_of(q), out, tid);
}
// Enqueue for workloads whose consumers poll (the reference has none): fast-path
// attempts only.  With many pollers a request on the wait-free slow path does not
// catch the dequeue front (its tickets come one CAS at a time while pollers take
// Head tickets by the thousand), so this enqueue stays lock-free instead.  false
// when no free index turns up in `tries` attempts (the queue is full); a full item
// ring after GCQ_SPIN_LIMIT attempts sets ERR_SPIN.
__device__ inline bool enqueue_ptr_lockfree(mpmc* q, uint64_t value, uint32_t tid, uint32_t tries) {
    const uint32_t idx = try_dequeue(&q->fq, tid, tries);
    if (idx == BOT) return false;
    st_rlx(&q->data[idx], value);
    const cfg c = load_cfg(&q->aq);
    for (uint32_t k = 0; k < GCQ_SPIN_LIMIT; ++k)
        if (try_enq<true>(&q->aq, c, idx) == 0) return true;
    raise_error(c.err, ERR_SPIN);
    return false;
}

// try_dequeue on the item ring of an MPMC queue.
__device__ __forceinline__ bool try_dequeue_ptr(mpmc* q, uint64_t* out, uint32_t tid, uint32_t tries) {
    const uint32_t idx = try_dequeue(&q->aq, tid, tries);
    if (idx == BOT) return false;
    *out = take_and_return(view_of(q), idx, tid);
    return true;
}

}  // namespace gwf
}  // namespace gcq

// -----------------------------------------------------------------------------
// Reference-named device API (gwf_queue.hpp:351-438).
// -----------------------------------------------------------------------------
#ifdef WF_TID_EXPR
__device__ __forceinline__ uint32_t wf_tid() { return (uint32_t)(WF_TID_EXPR); }
#else
__device__ __forceinline__ uint32_t wf_tid() { return blockIdx.x * blockDim.x + threadIdx.x; }
#endif

// Serial single-thread initialisation, as the reference's <<<1,1>>> init kernels do
// (wf_init, gwf_ring.hpp:229-276; full = the free-index ring of wf_mpmc_init,
// :278-298).  The ring header points at the arrays of the same object.
template <typename Config, uint32_t N_PARAM>
__device__ void wf_init(wf_t<Config, N_PARAM>* q, bool full = false) {
    gcq::gwf::ring* h = &q->hdr;
    h->Entry = q->Entry;
    h->Record = q->Record;
    h->Help = q->Help;
    h->Owner = q->Owner;
    q->err = 0;
    h->err = &q->err;
    h->order = 31 - __clz(N_PARAM);
    h->thr_bits = Config::BITS;
    h->max_threads = Config::MAX_THREADS;
    h->help_delay = WF_HELP_DELAY;
    h->enq_patience = WF_ENQ_PATIENCE;
    h->deq_patience = WF_DEQ_PATIENCE;
#ifdef CACHE_REMAP
    h->remap = 1;
#else
    h->remap = 0;
#endif
    h->deq_wait = 0;
    h->stats = nullptr;
    __threadfence();
    // one thread covers the whole ring (a grid-stride slice of width 1)
    gcq::gwf::init_slice(h, full, 0, 1);
    __threadfence();
}
// wf_mpmc_init, gwf_ring.hpp:278-298: aq empty, fq holding 0..N-1.
template <typename Config, uint32_t N_PARAM>
__device__ void wf_mpmc_init(wf_mpmc_t<Config, N_PARAM>* q) {
    wf_init(&q->aq, false);
    wf_init(&q->fq, true);
    for (uint32_t i = 0; i < N_PARAM; ++i) q->data[i] = 0;
    __threadfence();
}
template <typename Config, uint32_t N_PARAM>
__device__ __forceinline__ void Enqueue_wf(wf_t<Config, N_PARAM>* q, uint32_t index) {
    gcq::gwf::enqueue(&q->hdr, index, wf_tid());
}
template <typename Config, uint32_t N_PARAM>
__device__ __forceinline__ uint32_t Dequeue_wf(wf_t<Config, N_PARAM>* q) {
    return gcq::gwf::dequeue(&q->hdr, wf_tid());
}
template <typename Config, uint32_t N_PARAM>
__device__ __forceinline__ gcq::gwf::mpmc_view wf_view(wf_mpmc_t<Config, N_PARAM>* q) {
    return gcq::gwf::mpmc_view{&q->aq.hdr, &q->fq.hdr, q->data, &q->aq.err};
}
template <typename Config, uint32_t N_PARAM>
__device__ __forceinline__ bool Enqueue_Ptr(wf_mpmc_t<Config, N_PARAM>* q, uint64_t value) {
    return gcq::gwf::enqueue_ptr(wf_view(q), value, wf_tid());
}
template <typename Config, uint32_t N_PARAM>
__device__ __forceinline__ bool Dequeue_Ptr(wf_mpmc_t<Config, N_PARAM>* q, uint64_t* out) {
    return gcq::gwf::dequeue_ptr(wf_view(q), out, wf_tid());
}
