// CPU restatements of gCQ's four queues: test infrastructure (the oracle and the
// timed CPU baseline), never the product path.
//
// Each queue follows the reference algorithm step for step, with std::atomic
// (sequentially consistent) in place of the HIP device atomics the reference
// assumes to be sequentially consistent (gwf_ring.hpp:15-17).  Warp-aggregated
// ticket fetch-and-add becomes one fetch-and-add per thread, which is what the
// reference's batched helper reduces to for a single lane (gwf_ring.hpp:220-222,
// glf_queue.hpp:392-412).  Host threads stand in for GPU threads; the thread
// index passed to each call plays the part of wf_tid() (gwf_ring.hpp:53-63).
//
//   G-WFQ  gwf_queue.hpp:31-345 (types), gwf_ring.hpp:229-298 (init),
//          :309-371 (consume/finalize/catchup), :382-472 (fast path),
//          :486-639 (phase-2 records, cooperative FAA), :650-802 (slow path),
//          :808-861 (helping), :1234-1356 (Enqueue_wf/Dequeue_wf),
//          :1362-1380 (Enqueue_Ptr/Dequeue_Ptr)
//   G-LFQ  glf_queue.hpp:44-138 (layout), :418-440 (init), :447-455 (catchup),
//          :467-582 (enqueue/dequeue/indirection)
//   YMC    wfqueue_hip_opt.hpp:124-189 (layout), :192-237 (find_cell),
//          :248-318 (enqueue), :320-413 (help_enq), :416-524 (dequeue),
//          :527-555 (public API), :571-644 (init)
//   SFQ    sfqueue_hip.hpp:13-66 (layout, ids), sfqueue_hip.cpp:31-128 (ops),
//          :134-144 (u64 wrapper)
//
// Where the reference's slow paths lose or duplicate values, the G-WFQ and YMC
// restatements follow the published algorithms (each departure is marked where it
// is made, and G-WFQ keeps flags that restore the reference's rules).  The G-WFQ
// and G-LFQ cycle tags are 15 and 16 bits wide, as in the device code, instead of
// the reference's 8; WF_CYCLE_BITS / FQ_CYCLE_BITS at compile time restore 8.
//
// Runners at the end drive them like the reference harnesses:
//   history      correctness/history.cpp:188-227 with the logical clock of
//                correctness/wf_linlog.hpp:25-45
//   throughput   throughout_bench.cpp:810-882 (balanced and split kernels)
// and stress them for exactly-once delivery (oracle_gwf_slow_stress,
// oracle_ymc_slow_stress).  gwfmodel, before the runners, restates the device
// MPMC path's additions to the reference algorithm for the same kind of stress
// (oracle_gwf_device_model_stress); it is a model of the device code, not of the
// reference.

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <new>
#include <thread>
#include <vector>

namespace {

using u32 = uint32_t;
using u64 = uint64_t;
using clk = std::chrono::steady_clock;

enum Kind { GWFQ = 0, GLFQ = 1, WFQ = 2, SFQ = 3 };

static inline void cpu_relax() { std::this_thread::yield(); }

// =============================================================================
// G-WFQ
// =============================================================================
namespace gwf {

// Note and Cycle take WF_CYCLE_BITS each at the top of the entry, as in the device
// code; 8 (-DWF_CYCLE_BITS=8) gives gwf_queue.hpp's layout (:110-116, :140-160),
// whose tag wraps when an operation holds a ticket 128 cycles behind the counters.
#ifndef WF_CYCLE_BITS
#define WF_CYCLE_BITS 15
#endif
constexpr u32 CYCLE_MASK = (1u << WF_CYCLE_BITS) - 1, HALF_CYCLE = 1u << (WF_CYCLE_BITS - 1);
constexpr int NOTE_SHIFT = 64 - WF_CYCLE_BITS, CYCLE_SHIFT = 64 - 2 * WF_CYCLE_BITS;
constexpr int SAFE_SHIFT = CYCLE_SHIFT - 1, ENQ_SHIFT = CYCLE_SHIFT - 2;
static_assert(ENQ_SHIFT >= 32, "Note and Cycle must fit above the 32-bit index");
constexpr u64 SAFE_BIT = 1ULL << SAFE_SHIFT, ENQ_BIT = 1ULL << ENQ_SHIFT;
constexpr u32 BOT = 0xFFFFFFFEu, BOT_C = 0xFFFFFFFFu;
constexpr u64 CONSUME_MASK = ENQ_BIT | (u64)BOT_C;
constexpr u64 INIT = ((u64)CYCLE_MASK << NOTE_SHIFT) | SAFE_BIT | ENQ_BIT | BOT;
constexpr u64 FIN = 1, INC = 2, CNT_MASK = ~3ULL;

static inline u32 note(u64 e) { return (u32)((e >> NOTE_SHIFT) & CYCLE_MASK); }
static inline u32 cyc(u64 e) { return (u32)((e >> CYCLE_SHIFT) & CYCLE_MASK); }
static inline bool safe(u64 e) { return (e >> SAFE_SHIFT) & 1; }
static inline bool enq(u64 e) { return (e >> ENQ_SHIFT) & 1; }
static inline u32 idx(u64 e) { return (u32)e; }
static inline u64 pack(u32 n, u32 c, bool s, bool q, u32 i) {
    return ((u64)(n & CYCLE_MASK) << NOTE_SHIFT) | ((u64)(c & CYCLE_MASK) << CYCLE_SHIFT) |
           ((u64)s << SAFE_SHIFT) | ((u64)q << ENQ_SHIFT) | (u64)i;
}
static inline int ccmp(u32 a, u32 b) {
    u32 d = (a - b) & CYCLE_MASK;
    return d == 0 ? 0 : (d < HALF_CYCLE ? 1 : -1);
}

struct Rec {
    // phase-2 record (gwf_queue.hpp:242-247)
    std::atomic<u32> p2_seq1{1};
    std::atomic<u64> p2_local{0};   // address of the victim's localTail/localHead
    std::atomic<u64> p2_cnt{0};
    std::atomic<u32> p2_seq2{0};
    // help request (gwf_queue.hpp:272-286)
    std::atomic<u32> seq1{1}, enqueue{0}, pending{0};
    std::atomic<u64> localTail{0}, initTail{0}, localHead{0}, initHead{0};
    std::atomic<u32> index{0}, seq2{0};
    // private countdown (gwf_queue.hpp:260-261)
    int32_t nextCheck = 64;
    u32 nextTid = 0;
    char pad[8];
};

struct Knobs { int help_delay = 64, enq_patience = 128, deq_patience = 256; };

struct Ring {
    alignas(128) std::atomic<u64> Tail{0};
    alignas(128) std::atomic<u64> Head{0};
    alignas(128) std::atomic<int32_t> Threshold{-1};
    u32 n = 0, slots = 0, max_threads = 0;
    int thr_bits = 0;
    u64 null_tid = 0, cinc = 0;
    Knobs k;
    // true: gwf_ring.hpp:697-704 verbatim (a cycle match counts as produced even
    // when the slot was passed by a dequeuer); false: the corrected rule
    bool reference_produced_rule = false;
    // true: gwf_ring.hpp:548-590 verbatim (a helper that finds a thread index in the
    // counter word clears INC on that thread's phase-2 local whenever the record's
    // seqlock matches); false: the checked form of slow_faa below
    bool reference_phase2_help = false;
    // true: gwf_ring.hpp:729-731, 763-766 verbatim (a slow dequeue attempt reports
    // the request done whatever its FIN CAS found); false: done only once FIN is set
    bool reference_finish_rule = false;
    // true: gwf_ring.hpp:316-326 verbatim (finalize_request stops at the first
    // record whose localTail counter is h, INC or not); false: the holder of h only
    bool reference_finalize_scan = false;
    // true: gwf_ring.hpp:1242-1251 verbatim (with patience 1 the slow path starts
    // at counter 0); false: it starts from a Tail ticket of its own
    bool reference_patience1_start = false;
    std::unique_ptr<std::atomic<u64>[]> Entry;
    std::unique_ptr<Rec[]> Record;

    u64 packg(u64 cnt, u32 t) const { return (cnt << thr_bits) | ((u64)t & null_tid); }
    u64 cnt_of(u64 g) const { return g >> thr_bits; }
    u32 tid_of(u64 g) const { return (u32)(g & null_tid); }
    u32 cycle_of(u64 t) const { return (u32)((t / slots) & CYCLE_MASK); }
    u32 slot_of(u64 t) const { return (u32)(t & (slots - 1)); }
    int32_t thr_max() const { return 3 * (int32_t)n - 1; }

    void init(u32 n_, u32 max_threads_, int thr_bits_, Knobs kn) {
        n = n_; slots = 2 * n_; max_threads = max_threads_; thr_bits = thr_bits_; k = kn;
        null_tid = (1ULL << thr_bits) - 1;
        cinc = 1ULL << thr_bits;
        Entry.reset(new std::atomic<u64>[slots]);
        Record.reset(new Rec[max_threads]);
        reset(false);
    }
    void reset(bool full) {
        Tail = packg(slots, (u32)null_tid);
        Head = packg(slots, (u32)null_tid);
        Threshold = -1;
        for (u32 i = 0; i < slots; ++i) Entry[i].store(INIT);
        for (u32 i = 0; i < max_threads; ++i) {
            Rec& r = Record[i];
            r.nextCheck = k.help_delay; r.nextTid = i;
            r.p2_seq1 = 1; r.p2_local = 0; r.p2_cnt = 0; r.p2_seq2 = 0;
            r.seq1 = 1; r.enqueue = 0; r.pending = 0;
            r.localTail = 0; r.initTail = 0; r.localHead = 0; r.initHead = 0;
            r.index = 0; r.seq2 = 0;
        }
        if (full) {  // gwf_ring.hpp:286-297
            for (u32 i = 0; i < n; ++i) {
                u64 t = (u64)slots + i;
                Entry[slot_of(t)].store(pack(CYCLE_MASK, cycle_of(t), true, true, i));
            }
            Tail = packg((u64)slots + n, (u32)null_tid);
            Threshold = thr_max();
        }
    }

    // ---- consume / finalize / catchup --------------------------------------
    // Sets FIN on the request that holds ticket h.  A localTail whose counter is h
    // with INC set belongs to a request that tried to claim h in the cooperative
    // fetch-and-add and lost (its next attempt moves it on); the holder's localTail
    // is h without INC from before it produced the entry until FIN.  The reference
    // stops at the first counter match: when that is a loser, the holder never gets
    // FIN while its producer is delayed, its helpers take the consumed slot as
    // produced until the slot is reused a cycle later, then move on and produce the
    // index a second time.  So the scan passes over INC matches.
    void finalize_request(u64 h_raw, u32 me) {
        u64 hl = h_raw << 2;
        u32 i = (me + 1) % max_threads;
        while (i != me) {
            u64 lt = Record[i].localTail.load();
            if (reference_finalize_scan ? (lt & CNT_MASK) == hl : (lt & ~FIN) == hl) {
                u64 e = hl;
                Record[i].localTail.compare_exchange_strong(e, hl | FIN);
                return;
            }
            i = (i + 1) % max_threads;
        }
    }
    void consume(u64 h_raw, u32 j, u64 e, u32 me) {
        if (!enq(e)) finalize_request(h_raw, me);
        Entry[j].fetch_or(CONSUME_MASK);
    }
    void catchup(u64 tail_raw, u64 head_raw) {
        for (int i = 0; i < 32; ++i) {
            u64 cur = Tail.load();
            u64 cc = cnt_of(cur);
            if (cc >= head_raw) break;
            if (cc != tail_raw) {
                tail_raw = cc;
                head_raw = cnt_of(Head.load());
                if (tail_raw >= head_raw) break;
                continue;
            }
            u64 want = packg(head_raw, tid_of(cur));
            if (Tail.compare_exchange_strong(cur, want)) break;
            head_raw = cnt_of(Head.load());
            tail_raw = cnt_of(Tail.load());
            if (tail_raw >= head_raw) break;
        }
    }

    // ---- fast path ---------------------------------------------------------
    u64 try_enq(u32 index) {
        u64 T = cnt_of(Tail.fetch_add(cinc));
        u32 tc = cycle_of(T), j = slot_of(T);
        u64 E = Entry[j].load();
        for (;;) {
            u32 ec = cyc(E), ei = idx(E);
            if (ccmp(ec, tc) < 0 && (safe(E) || cnt_of(Head.load()) <= T) &&
                (ei == BOT || ei == BOT_C)) {
                u64 nw = pack(note(E), tc, true, true, index);
                if (!Entry[j].compare_exchange_strong(E, nw)) continue;
                if (Threshold.load() != thr_max()) Threshold.exchange(thr_max());
                return 0;
            }
            return T;
        }
    }
    u64 try_deq(u32* out, u32 me) {
        u64 H = cnt_of(Head.fetch_add(cinc));
        u32 hc = cycle_of(H), j = slot_of(H);
        u64 E = Entry[j].load();
        for (;;) {
            u32 ec = cyc(E), ei = idx(E);
            if (ccmp(ec, hc) == 0 && ei != BOT && ei != BOT_C) {
                consume(H, j, E, me);
                *out = ei;
                return 0;
            }
            u64 nw = (ei == BOT || ei == BOT_C) ? pack(note(E), hc, safe(E), true, BOT)
                                                : pack(note(E), ec, false, enq(E), ei);
            if (ccmp(ec, hc) < 0) {
                if (!Entry[j].compare_exchange_strong(E, nw)) continue;
            }
            break;
        }
        u64 T = cnt_of(Tail.load());
        if (T <= H + 1) {
            catchup(T, H + 1);
            Threshold.fetch_sub(1);
            *out = BOT;
            return 0;
        }
        if (Threshold.fetch_sub(1) <= 0) { *out = BOT; return 0; }
        return H;
    }

    // ---- cooperative fetch-and-add -----------------------------------------
    void prepare_phase2(Rec& me, std::atomic<u64>* local, u64 cnt_local) {
        u32 seq = me.p2_seq1.load() + 1;
        me.p2_seq1.store(seq);
        me.p2_local.store((u64)(uintptr_t)local);
        me.p2_cnt.store(cnt_local);
        me.p2_seq2.store(seq);
    }
    bool slow_faa(std::atomic<u64>* gp_, std::atomic<u64>* local, u64* v,
                  std::atomic<int32_t>* thld, u32 me) {
        Rec& mine = Record[me];
        u64 cnt_local = 0, cnt_raw = 0;
        bool ok = false;
        do {
            u64 lc = local->load();
            if (lc & FIN) { *v = lc; return false; }
            u64 gp = gp_->load();
            u32 gt = tid_of(gp);
            if (gt != (u32)null_tid) {
                Rec& hr = Record[gt];
                u32 seq = hr.p2_seq2.load();
                auto* p2l = (std::atomic<u64>*)(uintptr_t)hr.p2_local.load();
                u64 p2c = hr.p2_cnt.load();
                u32 s1 = hr.p2_seq1.load();
                // A thread has one phase-2 record for both counters, and a counter
                // word keeps a thread index after that thread's own clean-up CAS
                // lost to a fetch-and-add.  So the record read here may describe an
                // increment of the other counter, or a later one of this counter
                // whose CAS has not happened.  Clearing INC for it hands that
                // thread a ticket the counter also gives to a fast-path operation:
                // two enqueuers on one ticket lose a value, two dequeuers duplicate
                // one.  The INC is cleared only when the record's local is fed by
                // this counter and the word, read again after the record, still
                // names the thread past the record's count -- which holds for the
                // phase 2 of that thread's successful CAS until its thread index is
                // cleaned, and the first cleaner clears INC before it cleans.
                bool help_ok = s1 == seq && p2l;
                if (help_ok && !reference_phase2_help) {
                    const u64 g2 = gp_->load();
                    const uintptr_t base = (gp_ == &Tail) ? (uintptr_t)&Record[0].localTail
                                                          : (uintptr_t)&Record[0].localHead;
                    const uintptr_t a = (uintptr_t)p2l;
                    help_ok = a >= base && (a - base) % sizeof(Rec) == 0 && (a - base) / sizeof(Rec) < max_threads &&
                              tid_of(g2) == gt && cnt_of(g2) > (p2c >> 2);
                }
                if (help_ok) {
                    u64 e = p2c | INC;
                    p2l->compare_exchange_strong(e, p2c);
                }
                u64 clean = packg(cnt_of(gp), (u32)null_tid);
                if (!gp_->compare_exchange_strong(gp, clean)) continue;
                gp = clean;
            }
            cnt_raw = cnt_of(gp);
            cnt_local = cnt_raw << 2;
            u64 vc = *v;
            if (!local->compare_exchange_strong(vc, cnt_local | INC)) {
                *v = vc;
                if (vc & FIN) return false;
                if (!(vc & INC)) return true;
                cnt_local = vc & CNT_MASK;
                cnt_raw = cnt_local >> 2;
            } else {
                *v = cnt_local | INC;
            }
            prepare_phase2(mine, local, cnt_local);
            u64 exp = packg(cnt_raw, (u32)null_tid);
            ok = gp_->compare_exchange_strong(exp, packg(cnt_raw + 1, me));
        } while (!ok);
        if (thld) thld->fetch_sub(1);
        u64 e = cnt_local | INC;
        local->compare_exchange_strong(e, cnt_local);
        u64 g = packg(cnt_raw + 1, me);
        gp_->compare_exchange_strong(g, packg(cnt_raw + 1, (u32)null_tid));
        *v = cnt_local;
        return true;
    }

    // ---- slow path ---------------------------------------------------------
    bool try_enq_slow(u64 T, u32 index, Rec& r) {
        u32 tc = cycle_of(T), j = slot_of(T);
        u64 P = Entry[j].load();
        for (;;) {
            u32 ec = cyc(P), en = note(P), ei = idx(P);
            if (ccmp(ec, tc) < 0 && ccmp(en, tc) < 0) {
                if ((!safe(P) && cnt_of(Head.load()) > T) || (ei != BOT && ei != BOT_C)) {
                    u64 nn = pack(tc, ec, safe(P), enq(P), ei);
                    if (!Entry[j].compare_exchange_strong(P, nn)) continue;
                    return false;
                }
                u64 nn = pack(en, tc, true, false, index);
                if (!Entry[j].compare_exchange_strong(P, nn)) continue;
                u64 tl = T << 2;
                if (r.localTail.compare_exchange_strong(tl, (T << 2) | FIN)) {
                    u64 e0 = nn;
                    Entry[j].compare_exchange_strong(e0, pack(en, tc, true, true, index));
                }
                if (Threshold.load() != thr_max()) Threshold.exchange(thr_max());
                return true;
            } else if (ccmp(ec, tc) != 0) {
                return false;
            }
            // at our cycle: produced for this request (our index or consumed, ⊥c),
            // or passed by the dequeuer holding the same ticket (⊥), which the
            // reference also counts as produced
            return reference_produced_rule || ei == index || ei == BOT_C;
        }
    }
    bool try_deq_slow(u64 H, Rec& r) {
        u32 hc = cycle_of(H), j = slot_of(H);
        u64 P = Entry[j].load();
        for (;;) {
            u32 ec = cyc(P), en = note(P), ei = idx(P);
            if (ccmp(ec, hc) == 0 && ei != BOT && ei != BOT_C) {
                u64 hl = H << 2;
                if (r.localHead.compare_exchange_strong(hl, (H << 2) | FIN) || reference_finish_rule) return true;
                return (hl & FIN) != 0;
            }
            u32 nnote = en;
            u64 val = pack(nnote, hc, safe(P), true, BOT);
            if (ei != BOT && ei != BOT_C) {
                if (ccmp(ec, hc) < 0 && ccmp(en, hc) < 0) {
                    u64 nn = pack(hc, ec, safe(P), enq(P), ei);
                    if (!Entry[j].compare_exchange_strong(P, nn)) continue;
                    nnote = hc;
                }
                val = pack(nnote, ec, false, enq(P), ei);
            }
            if (ccmp(ec, hc) < 0) {
                if (!Entry[j].compare_exchange_strong(P, val)) continue;
            }
            break;
        }
        u64 T = cnt_of(Tail.load());
        if (T <= H + 1) catchup(T, H + 1);
        // Done only when the request is finished: at this ticket (this CAS) or
        // already (FIN).  gwf_ring.hpp:763-766 reports done whatever the CAS found;
        // when another helper has moved the request to a later ticket, the owner
        // then stops and gathers at that unfinished ticket (empty), and the helper
        // that finishes the request there later claims an element nobody returns.
        if (Threshold.load() < 0) {
            u64 hl = H << 2;
            if (r.localHead.compare_exchange_strong(hl, (H << 2) | FIN) || reference_finish_rule) return true;
            return (hl & FIN) != 0;
        }
        return false;
    }
    static constexpr u32 NO_SEQ = 0xFFFFFFFFu;
    // a helper (seq != NO_SEQ) stops once the request it read is over
    void enqueue_slow(u64 v, u32 index, Rec& r, u32 me, u32 seq = NO_SEQ) {
        while (slow_faa(&Tail, &r.localTail, &v, nullptr, me)) {
            if (seq != NO_SEQ && r.seq1.load() != seq) break;
            if (try_enq_slow(v >> 2, index, r)) break;
        }
    }
    void dequeue_slow(u64 v, Rec& r, u32 me) {
        while (slow_faa(&Head, &r.localHead, &v, &Threshold, me))
            if (try_deq_slow(v >> 2, r)) break;
    }

    // ---- helping -----------------------------------------------------------
    void help_enqueue(Rec& t, u32 me) {
        u32 seq = t.seq2.load();
        u32 is_enq = t.enqueue.load();
        u32 index = t.index.load();
        u64 it = t.initTail.load();
        if (is_enq && t.seq1.load() == seq) enqueue_slow(it, index, t, me, seq);
    }
    void help_dequeue(Rec& t, u32 me) {
        u32 seq = t.seq2.load();
        u32 is_enq = t.enqueue.load();
        u64 ih = t.initHead.load();
        if (!is_enq && t.seq1.load() == seq) dequeue_slow(ih, t, me);
    }
    void help_threads(u32 me) {
        Rec& r = Record[me];
        if (--r.nextCheck != 0) return;
        Rec& t = Record[r.nextTid];
        if (t.pending.load()) {
            if (t.enqueue.load()) help_enqueue(t, me);
            else help_dequeue(t, me);
        }
        r.nextCheck = k.help_delay;
        r.nextTid = (r.nextTid + 1) % max_threads;
    }

    // ---- top level ---------------------------------------------------------
    void enqueue_wf(u32 index, u32 me) {
        help_threads(me);
        u64 tail = 0;
        int count = k.enq_patience;
        while (--count != 0) {
            tail = try_enq(index);
            if (tail == 0) return;
        }
        // With patience 1 no fast-path attempt leaves a failed ticket, and the
        // reference starts the slow path at counter 0 -- the start of every request
        // of this thread.  A helper of the thread's previous request whose view is
        // still 0 can then CAS the new request's localTail to a count that request
        // already used, and once INC is cleared the new request holds a spent
        // ticket: it takes the consumed slot as produced and its value is lost.  A
        // ticket taken here, and left unused like a failed attempt, makes the start
        // unique.  (The library refuses patience below 2.)
        if (tail == 0 && !reference_patience1_start) tail = cnt_of(Tail.fetch_add(cinc));
        Rec& r = Record[me];
        u32 seq = r.seq1.load();
        r.localTail.store(tail << 2);
        r.initTail.store(tail << 2);
        r.index.store(index);
        r.enqueue.store(1);
        r.seq2.store(seq);
        r.pending.store(1);
        enqueue_slow(tail << 2, index, r, me);
        r.pending.store(0);
        r.seq1.store(seq + 1);
    }
    u32 dequeue_wf(u32 me) {
        if (Threshold.load() < 0) return BOT;
        help_threads(me);
        u32 out = BOT;
        u64 head = 0;
        int count = k.deq_patience;
        while (--count != 0) {
            head = try_deq(&out, me);
            if (head == 0) return out;
        }
        Rec& r = Record[me];
        u32 seq = r.seq1.load();
        r.localHead.store(head << 2);
        r.initHead.store(head << 2);
        r.enqueue.store(0);
        r.seq2.store(seq);
        r.pending.store(1);
        dequeue_slow(head << 2, r, me);
        r.pending.store(0);
        r.seq1.store(seq + 1);
        u64 hr = r.localHead.load() >> 2;
        u32 j = slot_of(hr);
        u64 E = Entry[j].load();
        if (ccmp(cyc(E), cycle_of(hr)) == 0 && idx(E) != BOT && idx(E) != BOT_C) {
            consume(hr, j, E, me);
            return idx(E);
        }
        return BOT;
    }
};

struct Mpmc {
    Ring aq, fq;
    std::unique_ptr<std::atomic<u64>[]> data;
    u32 n = 0;
    void init(u32 n_, u32 max_threads, int thr_bits, Knobs k) {
        n = n_;
        aq.init(n, max_threads, thr_bits, k);
        fq.init(n, max_threads, thr_bits, k);
        fq.reset(true);
        data.reset(new std::atomic<u64>[n]);
        for (u32 i = 0; i < n; ++i) data[i].store(0, std::memory_order_relaxed);
    }
    bool enqueue(u64 v, u32 me) {
        u32 i = fq.dequeue_wf(me);
        if (i == BOT) return false;
        data[i].store(v, std::memory_order_relaxed);
        aq.enqueue_wf(i, me);
        return true;
    }
    bool dequeue(u64* out, u32 me) {
        u32 i = aq.dequeue_wf(me);
        if (i == BOT) return false;
        *out = data[i].load(std::memory_order_relaxed);
        fq.enqueue_wf(i, me);
        return true;
    }
};

}  // namespace gwf

// =============================================================================
// G-LFQ
// =============================================================================
namespace glf {

// The cycle tag takes FQ_CYCLE_BITS above bit 48, as in the device code; 8 gives
// glf_queue.hpp's default (:36-47).
#ifndef FQ_CYCLE_BITS
#define FQ_CYCLE_BITS 16
#endif
constexpr u32 CYCLE_MASK = (1u << FQ_CYCLE_BITS) - 1, HALF = 1u << (FQ_CYCLE_BITS - 1);
static_assert(48 + FQ_CYCLE_BITS <= 64, "the cycle tag must fit above bit 48");
constexpr u32 BOT = 0xFFFFFFFEu, BOT_C = 0xFFFFFFFFu;
constexpr u64 SAFE_BIT = 1ULL << 47;
constexpr u64 INIT = SAFE_BIT | BOT;
constexpr u32 PER_LINE = 8;  // 64-byte lines of 8-byte entries (glf_queue.hpp:50-51)

static inline u32 cyc(u64 e) { return (u32)((e >> 48) & CYCLE_MASK); }
static inline bool safe(u64 e) { return (e >> 47) & 1; }
static inline u32 idx(u64 e) { return (u32)e; }
static inline u64 pack(u32 c, bool s, u32 i) { return ((u64)(c & CYCLE_MASK) << 48) | ((u64)s << 47) | (u64)i; }
static inline int ccmp(u32 a, u32 b) { u32 d = (a - b) & CYCLE_MASK; return d == 0 ? 0 : d < HALF ? 1 : -1; }

struct Ring {
    alignas(128) std::atomic<u64> Tail{0};
    alignas(128) std::atomic<u64> Head{0};
    alignas(128) std::atomic<int32_t> Threshold{-1};
    u32 n = 0, slots = 0;
    std::unique_ptr<std::atomic<u64>[]> Entry;
    u32 cycle_of(u64 t) const { return (u32)((t / slots) & CYCLE_MASK); }
    u32 remap(u64 t) const {
        u32 p = (u32)(t & (slots - 1));
        if (slots <= PER_LINE) return p;  // one line: glf_queue.hpp:116-120 would send every ticket to slot 0
        return (p & (PER_LINE - 1)) * (slots / PER_LINE) + p / PER_LINE;
    }
    int32_t thr_max() const { return 3 * (int32_t)n - 1; }
    void init(u32 n_, bool full) {
        n = n_; slots = 2 * n;
        Entry.reset(new std::atomic<u64>[slots]);
        Tail = slots; Head = slots; Threshold = -1;
        for (u32 i = 0; i < slots; ++i) Entry[i].store(INIT);
        if (full) {
            for (u32 i = 0; i < n; ++i) {
                u64 t = (u64)slots + i;
                Entry[remap(t)].store(pack(cycle_of(t), true, i));
            }
            Tail = (u64)slots + n;
            Threshold = thr_max();
        }
    }
    void catchup(u64 tail, u64 head) {
        for (int i = 0; i < 32; ++i) {
            if (Tail.compare_exchange_strong(tail, head)) break;
            head = Head.load();
            tail = Tail.load();
            if (tail >= head) break;
        }
    }
    void enqueue(u32 index) {
        for (;;) {
            u64 T = Tail.fetch_add(1);
            u32 tc = cycle_of(T), j = remap(T);
            u64 E = Entry[j].load();
            for (;;) {
                u32 ec = cyc(E), ei = idx(E);
                if (ccmp(ec, tc) < 0 && (safe(E) || Head.load() <= T) && (ei == BOT || ei == BOT_C)) {
                    if (!Entry[j].compare_exchange_strong(E, pack(tc, true, index))) continue;
                    if (Threshold.load() != thr_max()) Threshold.exchange(thr_max());
                    return;
                }
                break;
            }
        }
    }
    u32 dequeue() {
        if (Threshold.load() < 0) return BOT;
        for (;;) {
            u64 H = Head.fetch_add(1);
            u32 hc = cycle_of(H), j = remap(H);
            u64 E = Entry[j].load();
            for (;;) {
                u32 ec = cyc(E), ei = idx(E);
                if (ccmp(ec, hc) == 0 && ei != BOT && ei != BOT_C) {
                    Entry[j].fetch_or((u64)BOT_C);
                    return ei;
                }
                u64 nw = (ei == BOT || ei == BOT_C) ? pack(hc, safe(E), BOT) : pack(ec, false, ei);
                if (ccmp(ec, hc) < 0) {
                    if (!Entry[j].compare_exchange_strong(E, nw)) continue;
                }
                break;
            }
            u64 T = Tail.load();
            if (T <= H + 1) {
                catchup(T, H + 1);
                Threshold.fetch_sub(1);
                return BOT;
            }
            if (Threshold.fetch_sub(1) <= 0) return BOT;
        }
    }
};

struct Mpmc {
    Ring aq, fq;
    std::unique_ptr<std::atomic<u64>[]> data;
    void init(u32 n) {
        aq.init(n, false);
        fq.init(n, true);
        data.reset(new std::atomic<u64>[n]);
        for (u32 i = 0; i < n; ++i) data[i].store(0, std::memory_order_relaxed);
    }
    bool enqueue(u64 v) {
        u32 i = fq.dequeue();
        if (i == BOT) return false;
        data[i].store(v, std::memory_order_relaxed);
        aq.enqueue(i);
        return true;
    }
    bool dequeue(u64* out) {
        u32 i = aq.dequeue();
        if (i == BOT) return false;
        *out = data[i].load(std::memory_order_relaxed);
        fq.enqueue(i);
        return true;
    }
};

}  // namespace glf

// =============================================================================
// SFQ (Scogland-Feng ticket queue)
// =============================================================================
namespace sfq {

enum { SUCCESS = 0, BUSY = 1, CLOSED = 2, TIMEDOUT = 3 };

struct Queue {
    alignas(128) std::atomic<u32> head{0};
    alignas(128) std::atomic<u32> tail{0};
    alignas(128) std::atomic<u32> closed{0};
    u32 L = 0, max_id = 0;
    std::unique_ptr<std::atomic<u32>[]> items, ids;
    double timeout_s = 10.0;
    void init(u32 len) {
        L = len;
        max_id = 2u * ((UINT32_MAX / L) + 1u);   // sfqueue_hip.hpp:39
        items.reset(new std::atomic<u32>[L]);
        ids.reset(new std::atomic<u32>[L]);
        for (u32 i = 0; i < L; ++i) { items[i].store(0); ids[i].store(0); }
        head = 0; tail = 0; closed = 0;
    }
    u32 get_id(u32 t) const { return (t / L) * 2u; }   // sfqueue_hip.hpp:35
    u32 next_id(u32 id) const { u32 n = id + 1; return n == max_id ? 0u : n; }
    bool wait_id(u32 target, u32 id, clk::time_point t0) {
        while (ids[target].load() != id) {
            if (closed.load()) return false;
            cpu_relax();
            if (std::chrono::duration<double>(clk::now() - t0).count() > timeout_s) return false;
        }
        return true;
    }
    int enqueue_blocking(u32 item) {
        if (closed.load()) return CLOSED;
        u32 t = tail.fetch_add(1);
        u32 target = t % L, id = get_id(t);
        if (!wait_id(target, id, clk::now())) return closed.load() ? CLOSED : TIMEDOUT;
        items[target].store(item);
        ids[target].store(next_id(id));
        return SUCCESS;
    }
    int dequeue_blocking(u32* out) {
        if (closed.load()) return CLOSED;
        u32 t = head.fetch_add(1);
        u32 target = t % L, id = get_id(t) + 1u;
        if (!wait_id(target, id, clk::now())) return closed.load() ? CLOSED : TIMEDOUT;
        *out = items[target].load();
        ids[target].store(next_id(id));
        return SUCCESS;
    }
    int enqueue_nb(u32 item) {
        if (closed.load()) return CLOSED;
        u32 t = tail.load();
        u32 target = t % L, id = get_id(t);
        if (ids[target].load() != id) return BUSY;
        if (!tail.compare_exchange_strong(t, t + 1)) return BUSY;
        items[target].store(item);
        ids[target].store(next_id(id));
        return SUCCESS;
    }
    int dequeue_nb(u32* out) {
        if (closed.load()) return CLOSED;
        u32 t = head.load();
        u32 target = t % L, id = get_id(t) + 1u;
        if (ids[target].load() != id) return BUSY;
        if (!head.compare_exchange_strong(t, t + 1)) return BUSY;
        *out = items[target].load();
        ids[target].store(next_id(id));
        return SUCCESS;
    }
};

}  // namespace sfq

// =============================================================================
// WFQ-YMC (Yang & Mellor-Crummey, GPU adaptation with a preallocated pool)
// =============================================================================
namespace ymc {

constexpr u64 BOTTOM = 0, TOP = ~0ULL, EMPTY = 0, RETRY = ~0ULL - 1;
constexpr u64 NUL = 0, TOPP = 1;
constexpr int SEG = 1024;

static inline u64 pst(int p, u64 low) { return ((u64)p << 63) | (low & ((1ULL << 63) - 1)); }
static inline int pend(u64 s) { return (int)(s >> 63); }
static inline u64 low(u64 s) { return s & ((1ULL << 63) - 1); }

struct EnqReq { std::atomic<u64> val{0}, state{0}; };
struct DeqReq { std::atomic<u64> id{0}, state{0}; };
struct Cell { std::atomic<u64> val{0}; std::atomic<u64> enq{0}; std::atomic<u64> deq{0}; };

struct Handle {
    Handle* next = nullptr;
    EnqReq enq_req;
    Handle* enq_peer = nullptr;
    u64 enq_id_last = 0;
    DeqReq deq_req;
    Handle* deq_peer = nullptr;
};

struct Queue {
    alignas(128) std::atomic<u64> T{0};
    alignas(128) std::atomic<u64> H{0};
    std::unique_ptr<Cell[]> cells;
    u64 cap_cells = 0;
    int patience = 16;
    std::unique_ptr<Handle[]> handles;
    int nthreads = 0;

    void init(int threads, int ops_per_thread) {
        // wfqueue_hip_opt.hpp:595-599: threads * (3*ops + 128) cells, plus 8 spare segments
        u64 per = (u64)(3 * ops_per_thread + 128);
        u64 total = (u64)threads * per;
        u64 segs = (total + SEG - 1) / SEG + 8;
        if (segs < 2) segs = 2;
        cap_cells = segs * SEG;
        cells.reset(new Cell[cap_cells]);
        nthreads = threads;
        handles.reset(new Handle[threads]);
        for (int i = 0; i < threads; ++i) {
            Handle& h = handles[i];
            h.next = &handles[(i + 1) % threads];
            h.enq_peer = h.next;
            h.deq_peer = h.next;
        }
    }
    Cell* find_cell(u64 id) { return id < cap_cells ? &cells[id] : nullptr; }
    static void advance_end(std::atomic<u64>& E, u64 cid) {
        u64 e = E.load();
        while (e < cid && !E.compare_exchange_strong(e, cid)) {}
    }
    static bool claim(std::atomic<u64>& st, u64 expect_id, u64 cell_id) {
        u64 e = pst(1, expect_id);
        return st.compare_exchange_strong(e, pst(0, cell_id));
    }
    void enq_commit(Cell* c, u64 v, u64 cid) {
        advance_end(T, cid + 1);
        c->val.exchange(v);
    }
    bool enq_fast(u64 v, u64* cid) {
        u64 i = T.fetch_add(1);
        Cell* c = find_cell(i);
        if (!c) { *cid = i; return false; }
        u64 e = BOTTOM;
        if (c->val.compare_exchange_strong(e, v)) return true;
        *cid = i;
        return false;
    }
    bool enq_slow(Handle& h, u64 v, u64 cell_id) {
        EnqReq& r = h.enq_req;
        r.val.store(v);
        r.state.store(pst(1, cell_id));
        for (;;) {
            u64 i = T.fetch_add(1);
            Cell* c = find_cell(i);
            if (!c) break;
            u64 e = NUL;
            if (c->enq.compare_exchange_strong(e, (u64)(uintptr_t)&r)) {
                u64 cur = c->val.load();
                if (cur == BOTTOM || cur == TOP) { claim(r.state, cell_id, i); break; }
            }
            if (!pend(r.state.load())) break;
        }
        u64 fid = low(r.state.load());
        Cell* d = find_cell(fid);
        if (d) {
            // The value goes into the claimed cell before the enqueue returns, as in
            // Yang & Mellor-Crummey's enq_slow.  wfqueue_hip_opt.hpp:313-314 commits
            // only when the cell already reads TOP; a cell still at BOTTOM then waits
            // for a dequeuer to commit the request's val, which this handle's next
            // slow enqueue overwrites.
            enq_commit(d, v, fid);
            return true;
        }
        return false;
    }
    u64 help_enq(Handle& h, Cell* c, u64 i) {
        u64 old = BOTTOM;
        if (!c->val.compare_exchange_strong(old, TOP)) {
            if (old != TOP) return old;
        }
        u64 ce = c->enq.load();
        if (ce == NUL) {
            Handle* p = h.enq_peer ? h.enq_peer : &h;
            EnqReq* r = &p->enq_req;
            u64 s = r->state.load();
            u64 rid = low(s);
            int pd = pend(s);
            if (h.enq_id_last != 0 && h.enq_id_last != rid) {
                h.enq_id_last = 0;
                p = p->next;
                h.enq_peer = p;
                r = &p->enq_req;
                s = r->state.load();
                rid = low(s);
                pd = pend(s);
            }
            if (pd && rid > 0 && rid <= i) {
                u64 prev = NUL;
                c->enq.compare_exchange_strong(prev, (u64)(uintptr_t)r);
                if (prev != NUL && prev != (u64)(uintptr_t)r) {
                    ce = prev;
                    h.enq_id_last = rid;
                } else {
                    ce = (u64)(uintptr_t)r;
                    h.enq_id_last = 0;
                    h.enq_peer = p->next;
                }
            } else {
                h.enq_id_last = 0;
                h.enq_peer = p->next;
            }
            if (ce == NUL) {
                u64 prev = NUL;
                ce = c->enq.compare_exchange_strong(prev, TOPP) ? TOPP : prev;
            }
        }
        if (ce == TOPP) return T.load() <= i ? EMPTY : RETRY;
        EnqReq* r = (EnqReq*)(uintptr_t)ce;
        u64 s = r->state.load();
        int pd = pend(s);
        u64 rid = low(s);
        u64 v = r->val.load();
        if (!pd) {
            if (rid == i) {
                if (c->val.load() == TOP) enq_commit(c, v, i);
                return c->val.load();
            }
            // bound to a request that took another cell: the cell is dead (TOP), not
            // evidence of an empty queue, as in Yang & Mellor-Crummey's help_enq;
            // wfqueue_hip_opt.hpp:394-395 returns EMPTY here when T <= i
            return c->val.load();
        }
        if (rid > i) return T.load() <= i ? EMPTY : RETRY;
        if (claim(r->state, rid, i) || r->state.load() == pst(0, i)) {
            if (c->val.load() == TOP) enq_commit(c, v, i);
        }
        return c->val.load();
    }
    u64 deq_fast(Handle& h, u64* id) {
        u64 i = H.fetch_add(1);
        Cell* c = find_cell(i);
        if (!c) { *id = i; return EMPTY; }
        u64 v = help_enq(h, c, i);
        if (v == EMPTY) return EMPTY;
        if (v != TOP && v != RETRY) {
            u64 e = NUL;
            if (c->deq.compare_exchange_strong(e, TOPP)) return v;
        }
        *id = i;
        return RETRY;
    }
    void help_deq(Handle& h, Handle& helpee) {
        DeqReq& r = helpee.deq_req;
        u64 s = r.state.load();
        u64 id = r.id.load();
        if (!pend(s) || low(s) < id) return;
        u64 prior = id, i = id, cand = 0;
        for (;;) {
            s = r.state.load();
            if (!pend(s) || r.id.load() != id) return;
            while (!cand && pend(s) && low(s) == prior) {
                Cell* c = find_cell(++i);
                if (!c) break;
                advance_end(H, i + 1);
                u64 v = help_enq(h, c, i);
                if (v == EMPTY || (v != TOP && v != RETRY && c->deq.load() == NUL)) { cand = i; break; }
                s = r.state.load();
                if (!pend(s) || r.id.load() != id) return;
            }
            if (cand) {
                // The candidate is kept when a smaller cell is announced instead: that
                // cell is tried first, and if its claim fails this one is announced
                // next (Yang & Mellor-Crummey's "if (idx >= new) new = 0").  Dropping
                // it, as wfqueue_hip_opt.hpp:474-479 does, resumes the scan past it,
                // and its value is left behind the request's cell.
                u64 e = pst(1, prior);
                if (r.state.compare_exchange_strong(e, pst(1, cand)) || !pend(e) || low(e) >= cand) cand = 0;
            }
            s = r.state.load();
            if (!pend(s) || r.id.load() != id) return;
            u64 a = low(s);
            Cell* c = find_cell(a);
            if (!c) return;
            // Claimed for this request by this helper or by another one: the value
            // the CAS found is compared, as Yang & Mellor-Crummey's help_deq does.
            // wfqueue_hip_opt.hpp:489-492 compares a value loaded before the CAS, so
            // a helper that loses the claim to another helper of the same request
            // moves on, announces a later cell, and the claimed cell is orphaned.
            u64 e = NUL;
            if (c->val.load() == TOP || c->deq.compare_exchange_strong(e, (u64)(uintptr_t)&r) ||
                e == (u64)(uintptr_t)&r) {
                u64 se = s;
                r.state.compare_exchange_strong(se, pst(0, a));
                return;
            }
            prior = a;
            if (a >= i) i = a;
        }
    }
    u64 deq_slow(Handle& h, u64 cid) {
        DeqReq& r = h.deq_req;
        r.id.store(cid);
        r.state.store(pst(1, cid));
        help_deq(h, h);
        u64 ix = low(r.state.load());
        Cell* c = find_cell(ix);
        if (!c) { advance_end(H, ix + 1); return EMPTY; }
        u64 v = c->val.load();
        advance_end(H, ix + 1);
        return v == TOP ? EMPTY : v;
    }
    bool enqueue(u64 v, int tid) {
        Handle& h = handles[tid];
        for (int p = patience; p >= 0; --p) {
            u64 cid = 0;
            if (enq_fast(v, &cid)) return true;
            if (p == 0) return enq_slow(h, v, cid);
        }
        return false;
    }
    u64 dequeue(int tid) {
        Handle& h = handles[tid];
        u64 v = RETRY, cid = 0;
        for (int p = patience; p >= 0; --p) {
            v = deq_fast(h, &cid);
            if (v != RETRY) break;
        }
        if (v == RETRY) v = deq_slow(h, cid);
        if (v != EMPTY) {
            help_deq(h, *h.deq_peer);
            h.deq_peer = h.deq_peer->next;
        }
        return v;
    }
};

}  // namespace ymc

// =============================================================================
// Uniform front end
// =============================================================================

struct AnyQueue {
    int kind = 0;
    gwf::Mpmc* g = nullptr;
    glf::Mpmc* l = nullptr;
    ymc::Queue* y = nullptr;
    sfq::Queue* s = nullptr;
    ~AnyQueue() { delete g; delete l; delete y; delete s; }
};

static int bits_for(u32 max_threads) {
    int b = 5;
    while (((1ULL << b) - 1) < (u64)max_threads + 1) ++b;   // NULL_TID must stay free
    return b;
}

static AnyQueue* make_queue(int kind, u32 order, u32 threads, int ops_hint) {
    AnyQueue* q = new AnyQueue;
    q->kind = kind;
    u32 n = 1u << order;
    switch (kind) {
        case GWFQ: {
            q->g = new gwf::Mpmc;
            q->g->init(n, std::max<u32>(threads, 32), bits_for(std::max<u32>(threads, 32)), gwf::Knobs{});
            break;
        }
        case GLFQ: q->l = new glf::Mpmc; q->l->init(n); break;
        case WFQ: q->y = new ymc::Queue; q->y->init((int)threads, ops_hint); break;
        case SFQ: q->s = new sfq::Queue; q->s->init(n); break;
        default: delete q; return nullptr;
    }
    return q;
}

// The harness shims of throughout_bench.cpp:134-285 / history.cpp:56-140.
static inline bool q_enqueue(AnyQueue* q, u64 v, u32 tid, bool split) {
    switch (q->kind) {
        case GWFQ: return q->g->enqueue(v, tid);
        case GLFQ: return q->l->enqueue(v);
        case WFQ: return q->y->enqueue(v, (int)tid);
        default: {
            u32 x = (u32)(v ^ (v >> 32));       // throughout_bench.cpp:246-249
            if (x == 0) x = 1;
            return (split ? q->s->enqueue_nb(x) : q->s->enqueue_blocking(x)) == sfq::SUCCESS;
        }
    }
}
static inline bool q_dequeue(AnyQueue* q, u64* out, u32 tid, bool split) {
    switch (q->kind) {
        case GWFQ: return q->g->dequeue(out, tid);
        case GLFQ: return q->l->dequeue(out);
        case WFQ: { u64 v = q->y->dequeue((int)tid); if (v == ymc::EMPTY) return false; *out = v; return true; }
        default: {
            u32 item = 0;
            int rc = split ? q->s->dequeue_nb(&item) : q->s->dequeue_blocking(&item);
            if (rc != sfq::SUCCESS) return false;
            *out = item;
            return true;
        }
    }
}


// -----------------------------------------------------------------------------
// Model of the device G-WFQ MPMC path (test infrastructure).  The device
// Enqueue_Ptr / Dequeue_Ptr add to the reference's algorithm: the second ring's
// ticket taken beside the first ring's access (an aq ticket that an Enqueue_Ptr
// finding the queue full abandons), the empty exit before a ticket (with catchup),
// and a per-thread context that skips the Threshold pre-check after the thread's
// own enqueue and tries the empty exit first after its own empty dequeue.  This
// restates those additions over the rings above so that a stress on the CPU can
// check them for exactly-once delivery.  prefetch: 0 none, 1 an aq ticket on every
// Enqueue_Ptr, 2 only while the thread's last free-ring dequeue succeeded, with a
// Threshold reset when a ticket is abandoned (the device's rule).
namespace gwfmodel {
using namespace gwf;
struct Ctx { bool aq_fresh = false, fq_fresh = false, aq_empty = false, fq_empty = false; };
static bool seen_empty(Ring& q) {
    const u64 h = q.cnt_of(q.Head.load());
    const u64 t = q.cnt_of(q.Tail.load());
    if (t > h) return false;
    if (t < h) q.catchup(t, h);
    return true;
}
static u64 try_enq_at(Ring& q, u32 index, u64 T) {
    const u32 tc = q.cycle_of(T), j = q.slot_of(T);
    u64 E = q.Entry[j].load();
    for (;;) {
        const u32 ec = cyc(E), ei = idx(E);
        if (ccmp(ec, tc) < 0 && (safe(E) || q.cnt_of(q.Head.load()) <= T) && (ei == BOT || ei == BOT_C)) {
            if (!q.Entry[j].compare_exchange_strong(E, pack(note(E), tc, true, true, index))) continue;
            if (q.Threshold.load() != q.thr_max()) q.Threshold.exchange(q.thr_max());
            return 0;
        }
        return T;
    }
}
static u64 try_deq_pf(Ring& q, u32* out, u32 me, std::atomic<u64>* pf, u64* pf_raw) {
    const u64 H = q.cnt_of(q.Head.fetch_add(q.cinc));
    if (pf) *pf_raw = pf->fetch_add(q.cinc);
    const u32 hc = q.cycle_of(H), j = q.slot_of(H);
    u64 E = q.Entry[j].load();
    for (;;) {
        const u32 ec = cyc(E), ei = idx(E);
        if (ccmp(ec, hc) == 0 && ei != BOT && ei != BOT_C) { q.consume(H, j, E, me); *out = ei; return 0; }
        if (ccmp(ec, hc) >= 0) break;
        const u64 nw = (ei == BOT || ei == BOT_C) ? pack(note(E), hc, safe(E), true, BOT)
                                                  : pack(note(E), ec, false, enq(E), ei);
        if (q.Entry[j].compare_exchange_strong(E, nw)) break;
    }
    const u64 T = q.cnt_of(q.Tail.load());
    if (T <= H + 1) { q.catchup(T, H + 1); q.Threshold.fetch_sub(1); *out = BOT; return 0; }
    if (q.Threshold.fetch_sub(1) <= 0) { *out = BOT; return 0; }
    return H;
}
static u32 dequeue(Ring& q, u32 me, std::atomic<u64>* pf, u64* pf_raw, bool skip_check, bool first_check) {
    if (!skip_check && q.Threshold.load() < 0) return BOT;
    if (first_check && seen_empty(q)) return BOT;
    q.help_threads(me);
    u32 out = BOT;
    u64 head = 0;
    if (pf) {
        head = try_deq_pf(q, &out, me, pf, pf_raw);
        if (head == 0) return out;
        if (seen_empty(q)) return BOT;
    }
    for (int count = q.k.deq_patience - (pf ? 1 : 0); --count > 0;) {
        head = try_deq_pf(q, &out, me, nullptr, nullptr);
        if (head == 0) return out;
        if (seen_empty(q)) return BOT;
    }
    Rec& r = q.Record[me];
    const u32 seq = r.seq1.load();
    r.localHead.store(head << 2); r.initHead.store(head << 2); r.enqueue.store(0);
    r.seq2.store(seq); r.pending.store(1);
    q.dequeue_slow(head << 2, r, me);
    r.pending.store(0); r.seq1.store(seq + 1);
    const u64 hr = r.localHead.load() >> 2;
    const u32 j = q.slot_of(hr);
    const u64 E = q.Entry[j].load();
    if (ccmp(cyc(E), q.cycle_of(hr)) == 0 && idx(E) != BOT && idx(E) != BOT_C) { q.consume(hr, j, E, me); return idx(E); }
    return BOT;
}
static void enqueue(Ring& q, u32 index, u32 me, u64 first_raw) {
    q.help_threads(me);
    u64 tail = 0;
    for (int count = q.k.enq_patience; --count > 0;) {
        const u64 T = first_raw ? q.cnt_of(first_raw) : q.cnt_of(q.Tail.fetch_add(q.cinc));
        first_raw = 0;
        tail = try_enq_at(q, index, T);
        if (tail == 0) return;
    }
    if (first_raw) tail = q.cnt_of(first_raw);
    Rec& r = q.Record[me];
    const u32 seq = r.seq1.load();
    r.localTail.store(tail << 2); r.initTail.store(tail << 2); r.index.store(index); r.enqueue.store(1);
    r.seq2.store(seq); r.pending.store(1);
    q.enqueue_slow(tail << 2, index, r, me);
    r.pending.store(0); r.seq1.store(seq + 1);
}
static void abandon(Ring& q, u64 T_raw, bool reset) {
    const u64 T = q.cnt_of(T_raw);
    const u32 tc = q.cycle_of(T), j = q.slot_of(T);
    u64 E = q.Entry[j].load();
    if (ccmp(cyc(E), tc) < 0 && (idx(E) == BOT || idx(E) == BOT_C))
        q.Entry[j].compare_exchange_strong(E, pack(note(E), tc, safe(E), true, BOT));
    if (reset && q.Threshold.load() != q.thr_max()) q.Threshold.exchange(q.thr_max());
}
struct Queue {
    Mpmc m;
    int prefetch = 2;
    bool enqueue_ptr(u64 v, u32 me, Ctx& x) {
        u64 aq_raw = 0;
        const bool pf = prefetch == 1 || (prefetch == 2 && !x.fq_empty);
        const u32 i = dequeue(m.fq, me, pf ? &m.aq.Tail : nullptr, &aq_raw, x.fq_fresh, x.fq_empty);
        x.fq_fresh = false;
        x.fq_empty = (i == BOT);
        if (i == BOT) {
            if (aq_raw) abandon(m.aq, aq_raw, prefetch == 2);
            return false;
        }
        m.data[i].store(v);
        enqueue(m.aq, i, me, aq_raw);
        x.aq_fresh = true;
        return true;
    }
    bool dequeue_ptr(u64* out, u32 me, Ctx& x) {
        const u32 i = dequeue(m.aq, me, nullptr, nullptr, x.aq_fresh, x.aq_empty);
        x.aq_fresh = false;
        x.aq_empty = (i == BOT);
        if (i == BOT) return false;
        const u64 fq_raw = m.fq.Tail.fetch_add(m.fq.cinc);
        *out = m.data[i].load();
        enqueue(m.fq, i, me, fq_raw);
        x.fq_fresh = true;
        return true;
    }
};
}  // namespace gwfmodel

// The device G-LFQ ring operations (a model of the device code, not of the
// reference): slots in ticket order (the device's default; the reference spreads
// them over lines), the enqueue CAS tried first against the steady-state free
// slot, a bounded wait for the enqueuer holding the dequeuer's ticket before the
// slot is marked (deq_wait), and the empty exit before a retry ticket.
namespace glfmodel {
using namespace glf;
struct Ring {
    alignas(128) std::atomic<u64> Tail{0};
    alignas(128) std::atomic<u64> Head{0};
    alignas(128) std::atomic<int32_t> Threshold{-1};
    u32 n = 0, slots = 0, deq_wait = 0;
    std::unique_ptr<std::atomic<u64>[]> Entry;
    u32 cycle_of(u64 t) const { return (u32)((t / slots) & CYCLE_MASK); }
    u32 slot_of(u64 t) const { return (u32)(t & (slots - 1)); }
    int32_t thr_max() const { return 3 * (int32_t)n - 1; }
    void init(u32 n_, bool full, u32 wait) {
        n = n_; slots = 2 * n; deq_wait = wait;
        Entry.reset(new std::atomic<u64>[slots]);
        for (u32 i = 0; i < slots; ++i) Entry[i].store(INIT);
        Head = slots;
        Tail = full ? (u64)slots + n : (u64)slots;
        Threshold = full ? thr_max() : -1;
        if (full)
            for (u32 i = 0; i < n; ++i) Entry[slot_of((u64)slots + i)].store(pack(cycle_of((u64)slots + i), true, i));
    }
    void catchup(u64 tail, u64 head) {
        for (int i = 0; i < 32; ++i) {
            if (Tail.compare_exchange_strong(tail, head)) break;
            head = Head.load();
            tail = Tail.load();
            if (tail >= head) break;
        }
    }
    void enqueue(u32 index) {
        for (;;) {
            const u64 T = Tail.fetch_add(1);
            const u32 tc = cycle_of(T), j = slot_of(T);
            u64 E = pack(tc - 1, true, BOT_C);
            if (Entry[j].compare_exchange_strong(E, pack(tc, true, index))) {
                if (Threshold.load() != thr_max()) Threshold.exchange(thr_max());
                return;
            }
            for (;;) {
                const u32 ec = cyc(E), ei = idx(E);
                if (ccmp(ec, tc) >= 0 || ei < BOT) break;
                if (!safe(E) && Head.load() > T) break;
                if (!Entry[j].compare_exchange_strong(E, pack(tc, true, index))) continue;
                if (Threshold.load() != thr_max()) Threshold.exchange(thr_max());
                return;
            }
        }
    }
    u32 dequeue() {
        if (Threshold.load() < 0) return BOT;
        for (;;) {
            const u64 H = Head.fetch_add(1);
            const u32 hc = cycle_of(H), j = slot_of(H);
            u64 E = Entry[j].load();
            for (u32 w = 0; w < deq_wait && ccmp(cyc(E), hc) < 0 && idx(E) >= BOT; ++w) {
                cpu_relax();
                E = Entry[j].load();
            }
            for (;;) {
                const u32 ec = cyc(E), ei = idx(E);
                if (ccmp(ec, hc) == 0 && ei < BOT) {
                    Entry[j].fetch_or((u64)BOT_C);
                    return ei;
                }
                if (ccmp(ec, hc) >= 0) break;
                const u64 nw = ei >= BOT ? pack(hc, safe(E), BOT) : pack(ec, false, ei);
                if (Entry[j].compare_exchange_strong(E, nw)) break;
            }
            const u64 T = Tail.load();
            if (T <= H + 1) {
                catchup(T, H + 1);
                Threshold.fetch_sub(1);
                return BOT;
            }
            if (Threshold.fetch_sub(1) <= 0) return BOT;
            const u64 h = Head.load(), t = Tail.load();
            if (t <= h) {
                if (t < h) catchup(t, h);
                return BOT;
            }
        }
    }
};
struct Queue {
    Ring aq, fq;
    std::unique_ptr<std::atomic<u64>[]> data;
    void init(u32 n, u32 deq_wait) {
        aq.init(n, false, deq_wait);
        fq.init(n, true, deq_wait);
        data.reset(new std::atomic<u64>[n]);
        for (u32 i = 0; i < n; ++i) data[i].store(0, std::memory_order_relaxed);
    }
    bool enqueue_ptr(u64 v) {
        const u32 i = fq.dequeue();
        if (i == BOT) return false;
        data[i].store(v, std::memory_order_relaxed);
        aq.enqueue(i);
        return true;
    }
    bool dequeue_ptr(u64* out) {
        const u32 i = aq.dequeue();
        if (i == BOT) return false;
        *out = data[i].load(std::memory_order_relaxed);
        fq.enqueue(i);
        return true;
    }
};
}  // namespace glfmodel

}  // namespace

extern "C" {

typedef struct {
    uint64_t proc;
    uint32_t op;
    uint32_t _pad;
    uint64_t arg;
    uint64_t ret;
    int64_t call;
    int64_t end;
} oracle_hist_rec;

typedef struct {
    uint64_t enq_success, enq_fail, deq_success, deq_empty;
    double elapsed_ms;
    uint32_t threads;
    uint32_t _pad;
} oracle_tb_stats;

// History of `threads` host threads each doing `ops` operations (mode 0:
// enqueue then dequeue; mode 1: the first producer_percent% of threads only
// enqueue, the rest only dequeue), bracketed by a shared logical clock.
// value_mode 0: (tid<<32)|(seq+1) (history.cpp:184); 1: 32-bit (tid<<16)|(seq+1).
// SFQ uses the non-blocking operations and the 15+16-bit encoding of
// history.cpp:121-140 whatever value_mode says; its BUSY dequeues are written as
// op 2 (dequeue without effect).  Returns records written.
int64_t oracle_history(int kind, uint32_t order, uint32_t threads, uint32_t ops, int mode,
                       int producer_percent, int value_mode, oracle_hist_rec* out, uint64_t cap) {
    uint64_t need = (uint64_t)threads * ops * (mode == 0 ? 2 : 1);
    if (need > cap) return -1;
    std::unique_ptr<AnyQueue> q(make_queue(kind, order, threads, (int)ops * 2 + 8));
    if (!q) return -2;
    std::atomic<uint64_t> clock{1};
    std::atomic<int> ready{0};
    std::vector<std::thread> ths;
    std::vector<uint64_t> counts(threads, 0);
    const uint64_t stride = (uint64_t)ops * (mode == 0 ? 2 : 1);
    for (uint32_t t = 0; t < threads; ++t) {
        ths.emplace_back([&, t]() {
            ready.fetch_add(1);
            while (ready.load() < (int)threads) cpu_relax();
            oracle_hist_rec* rec = out + (uint64_t)t * stride;
            uint64_t k = 0;
            bool producer = ((uint64_t)t * 100 / threads) < (uint64_t)producer_percent;
            for (uint32_t i = 0; i < ops; ++i) {
                u64 v;
                if (kind == SFQ) v = (((u64)t & 0x7FFF) << 16) | ((i + 1) & 0xFFFF);
                else if (value_mode == 1) v = (((u64)t & 0xFFFF) << 16) | ((i + 1) & 0xFFFF);
                else v = ((u64)t << 32) | (u64)(i + 1);
                if (mode == 0 || producer) {
                    oracle_hist_rec& r = rec[k++];
                    r.proc = t; r.op = 0; r._pad = 0; r.arg = v;
                    r.call = (int64_t)clock.fetch_add(1);
                    bool ok = q_enqueue(q.get(), v, t, true);
                    r.ret = ok ? 1 : 0;
                    r.end = (int64_t)clock.fetch_add(1);
                }
                if (mode == 0 || !producer) {
                    oracle_hist_rec& r = rec[k++];
                    r.proc = t; r.op = 1; r._pad = 0; r.arg = 0;
                    r.call = (int64_t)clock.fetch_add(1);
                    u64 o = 0;
                    bool ok = q_dequeue(q.get(), &o, t, true);
                    r.ret = ok ? o : 0;
                    r.end = (int64_t)clock.fetch_add(1);
                    // SFQ's non-blocking dequeue fails with BUSY, not "empty": record the
                    // no-op dequeue (op 2) that the checker models for it.
                    if (!ok && kind == SFQ) r.op = 2;
                }
            }
            counts[t] = k;
        });
    }
    for (auto& th : ths) th.join();
    // compact per-thread blocks (split mode writes `ops` records per thread)
    uint64_t n = 0;
    for (uint32_t t = 0; t < threads; ++t) {
        oracle_hist_rec* rec = out + (uint64_t)t * stride;
        for (uint64_t i = 0; i < counts[t]; ++i) out[n++] = rec[i];
    }
    return (int64_t)n;
}

// Fixed-duration throughput run (throughout_bench.cpp:959-1051) with host threads.
// mode 0 balanced (enqueue then dequeue per iteration), 1 split.
int oracle_tb_run(int kind, uint32_t order, uint32_t threads, int mode, int producer_percent,
                  double warmup_ms, double run_ms, oracle_tb_stats* out) {
    std::unique_ptr<AnyQueue> q(make_queue(kind, order, threads, 512));
    if (!q) return -2;
    std::atomic<int> phase{0};   // 0 warmup, 1 timed, 2 stop
    std::atomic<int> ready{0};
    struct alignas(128) Ctr { uint64_t eo = 0, ef = 0, dok = 0, de = 0; };
    std::vector<Ctr> ctr(threads);
    std::vector<std::thread> ths;
    for (uint32_t t = 0; t < threads; ++t) {
        ths.emplace_back([&, t]() {
            ready.fetch_add(1);
            bool producer = ((uint64_t)t * 100 / threads) < (uint64_t)producer_percent;
            Ctr local;
            uint32_t i = 0;
            bool counting = false;
            for (;;) {
                int ph = phase.load(std::memory_order_relaxed);
                if (ph == 2) break;
                if (ph == 1 && !counting) { counting = true; local = Ctr{}; }
                for (int c = 0; c < 64; ++c, ++i) {
                    if (mode == 0) {
                        u64 v = ((u64)t << 32) ^ (u64)(i + 1) ^ 0x9e3779b97f4a7c15ULL;
                        if (q_enqueue(q.get(), v, t, false)) local.eo++; else local.ef++;
                        u64 o;
                        if (q_dequeue(q.get(), &o, t, false)) local.dok++; else local.de++;
                    } else if (producer) {
                        u64 v = ((u64)t << 32) ^ (u64)(i + 1) ^ 0x517cc1b727220a95ULL;
                        if (q_enqueue(q.get(), v, t, true)) local.eo++; else local.ef++;
                    } else {
                        u64 o;
                        if (q_dequeue(q.get(), &o, t, true)) local.dok++; else local.de++;
                    }
                }
            }
            ctr[t] = local;
        });
    }
    while (ready.load() < (int)threads) std::this_thread::yield();
    std::this_thread::sleep_for(std::chrono::duration<double, std::milli>(warmup_ms));
    auto t0 = clk::now();
    phase.store(1);
    std::this_thread::sleep_for(std::chrono::duration<double, std::milli>(run_ms));
    phase.store(2);
    auto t1 = clk::now();
    for (auto& th : ths) th.join();
    std::memset(out, 0, sizeof(*out));
    for (auto& c : ctr) {
        out->enq_success += c.eo; out->enq_fail += c.ef;
        out->deq_success += c.dok; out->deq_empty += c.de;
    }
    // Operations finish their current 64-op batch after the stop flag; count the
    // elapsed time to the last join so that the rate is not overstated.
    auto t2 = clk::now();
    (void)t1;
    out->elapsed_ms = std::chrono::duration<double, std::milli>(t2 - t0).count();
    out->threads = threads;
    return 0;
}

// Produce-then-drain FIFO check (throughout_bench.cpp:531-603) on host threads.
// Exactly-once is checked as in the reference (counts per token).  The reference's
// per-producer order check (an atomicMax over last_seq, :585-588) starts from
// 0xFFFFFFFF (:691) and so never fires; here every dequeue is bracketed by a shared
// logical clock instead, and an order error is a pair of tokens from one producer,
// seq a < seq b, whose dequeue of b returned before the dequeue of a was called.
// out_counts = [in, out, dup, order_err, missing+oob].  Returns 0 when clean.
int oracle_fifo_check(int kind, uint32_t order, uint32_t threads, uint32_t ops_per_thread,
                      uint64_t* out_counts) {
    std::unique_ptr<AnyQueue> q(make_queue(kind, order, threads, (int)ops_per_thread * 2 + 8));
    if (!q) return -2;
    std::vector<std::thread> ths;
    for (uint32_t t = 0; t < threads; ++t)
        ths.emplace_back([&, t]() {
            for (uint32_t i = 0; i < ops_per_thread; ++i) {
                u64 tok = kind == SFQ ? ((((u64)t & 0x7FFF) << 16) | ((i + 1) & 0xFFFF))
                                      : (((u64)t << 32) | (u64)(i + 1));
                auto t0 = clk::now();
                while (!q_enqueue(q.get(), tok, t, true)) {
                    cpu_relax();
                    if (std::chrono::duration<double>(clk::now() - t0).count() > 10.0) return;
                }
            }
        });
    for (auto& th : ths) th.join();
    ths.clear();
    const uint64_t total = (uint64_t)threads * ops_per_thread;
    std::vector<std::atomic<uint32_t>> cnt(total);
    std::vector<int64_t> call(total, 0), end(total, 0);
    for (auto& c : cnt) c.store(0);
    std::atomic<uint64_t> consumed{0}, dup{0}, oob{0}, clock{1};
    for (uint32_t t = 0; t < threads; ++t)
        ths.emplace_back([&, t]() {
            auto t0 = clk::now();
            while (consumed.load() < total) {
                u64 v = 0;
                int64_t c0 = (int64_t)clock.fetch_add(1);
                bool ok = q_dequeue(q.get(), &v, t, true);
                int64_t c1 = (int64_t)clock.fetch_add(1);
                if (!ok) {
                    cpu_relax();
                    if (std::chrono::duration<double>(clk::now() - t0).count() > 10.0) return;
                    continue;
                }
                if (consumed.fetch_add(1) >= total) continue;
                u32 ptid, seq;
                if (kind == SFQ) { ptid = (u32)(v >> 16) & 0x7FFF; seq = (u32)(v & 0xFFFF) - 1; }
                else { ptid = (u32)(v >> 32); seq = (u32)v - 1; }
                if (ptid >= threads || seq >= ops_per_thread) { oob++; continue; }
                u64 slot = (u64)ptid * ops_per_thread + seq;
                if (cnt[slot].fetch_add(1) >= 1) { dup++; continue; }
                call[slot] = c0;
                end[slot] = c1;
            }
        });
    for (auto& th : ths) th.join();
    uint64_t missing = 0, ord = 0;
    for (uint32_t p = 0; p < threads; ++p) {
        int64_t max_call = -1;
        for (uint32_t s = 0; s < ops_per_thread; ++s) {
            u64 slot = (u64)p * ops_per_thread + s;
            if (cnt[slot].load() == 0) { missing++; continue; }
            if (end[slot] < max_call) ord++;
            max_call = std::max(max_call, call[slot]);
        }
    }
    if (out_counts) {
        out_counts[0] = total; out_counts[1] = std::min<uint64_t>(consumed.load(), total);
        out_counts[2] = dup.load(); out_counts[3] = ord; out_counts[4] = missing + oob.load();
    }
    return (consumed.load() >= total && !dup && !missing && !oob && !ord) ? 0 : 1;
}


// Known-answer case for the slow-path "already produced" rule, one thread, no
// timing: an enqueuer takes Tail ticket T; the dequeuer that takes Head ticket T
// finds the slot empty and marks it (cycle(T), ⊥); the enqueuer's slow path then
// tries ticket T.  Returns what try_enq_slow reports for ticket T (1 = "done") and,
// in *deq_out, what a dequeue returns after the slow path has run to completion
// (the index, or ⊥ = 0xFFFFFFFE if the element was lost).
// reference_rule = 1 runs the rule of gwf_ring.hpp:697-704.
int oracle_gwf_slow_passed_slot(int reference_rule, uint32_t* deq_out) {
    gwf::Ring q;
    q.init(8, 4, 2, gwf::Knobs());
    q.reference_produced_rule = reference_rule != 0;
    const u64 T = q.cnt_of(q.Tail.fetch_add(q.cinc));   // enqueuer (thread 0) takes T
    u32 out = 0;
    const u64 H = q.try_deq(&out, 1);                   // dequeuer (thread 1) takes T too
    if (H != 0 || out != gwf::BOT) return -1;
    const u32 index = 5;
    gwf::Rec& r = q.Record[0];
    const u32 seq = r.seq1.load();
    r.localTail.store(T << 2);
    r.initTail.store(T << 2);
    r.index.store(index);
    r.enqueue.store(1);
    r.seq2.store(seq);
    r.pending.store(1);
    const bool done_at_T = q.try_enq_slow(T, index, r);
    if (!done_at_T) q.enqueue_slow(T << 2, index, r, 0);
    r.pending.store(0);
    r.seq1.store(seq + 1);
    if (deq_out) *deq_out = q.dequeue_wf(2);
    return done_at_T ? 1 : 0;
}

// finalize_request with a losing claimant, deterministically: thread 2's request
// holds Tail ticket T and its producer has written index 5 there with Enq = 0 but
// not yet set FIN (it is delayed); thread 1's request tried to claim T in the
// cooperative fetch-and-add and lost, so its localTail reads T | INC.  Thread 0
// dequeues ticket T and finalizes.  out[0] and out[1] receive the two localTails
// afterwards; returns the dequeued index.  reference_scan = 1 runs the scan of
// gwf_ring.hpp:316-326.
int oracle_gwf_finalize_loser(int reference_scan, uint64_t* out) {
    gwf::Ring q;
    q.init(8, 4, 2, gwf::Knobs());
    q.reference_finalize_scan = reference_scan != 0;
    const u64 T = q.cnt_of(q.Tail.fetch_add(q.cinc));
    q.Record[1].localTail.store((T << 2) | gwf::INC);
    q.Record[2].localTail.store(T << 2);
    const u32 j = q.slot_of(T);
    const u64 E = q.Entry[j].load();
    q.Entry[j].store(gwf::pack(gwf::note(E), q.cycle_of(T), true, false, 5));
    u32 got = gwf::BOT;
    if (q.try_deq(&got, 0) != 0) return -1;
    out[0] = q.Record[1].localTail.load();
    out[1] = q.Record[2].localTail.load();
    return (int)got;
}

// Host fault injection for the wait-free helping of G-WFQ (gwf_ring.hpp:808-861,
// restated above): thread 0 takes a Tail ticket, publishes a slow-path enqueue
// request for index `stalled_index` and then stalls -- it makes no further step --
// while `threads - 1` workers each run `ops` enqueue/dequeue pairs of their own
// values with patience 1, so every operation takes the slow path, checking one peer
// every `help_delay` operations (1: every operation; a delay longer than the run
// disables helping, the control case).  The stalled request must be completed by the helpers: its
// index is in the queue while thread 0 is still stalled -- dequeued by a worker, or
// left in the queue and drained after the workers finish, before thread 0 resumes.
// Thread 0 then resumes its own slow path, which must find the request done and not
// insert the index again; a final drain must find every value exactly once.
// Returns 1 when all of that holds, 0 when it does not, negative for bad arguments.
// stats[0]: dequeues of the stalled index while thread 0 was stalled (workers and
// the drain before the resume), stats[1]: dequeues of it in total, stats[2]: worker
// values dequeued exactly once, stats[3]: worker values enqueued.
int oracle_gwf_stalled_helping(uint32_t threads, uint32_t ops, uint32_t help_delay, uint64_t* stats) {
    if (threads < 2 || threads > 64 || ops == 0 || ops > 4096 || help_delay == 0 || !stats) return -1;
    gwf::Ring q;
    gwf::Knobs kn;
    kn.help_delay = (int)help_delay;
    kn.enq_patience = 1;
    kn.deq_patience = 1;
    q.init(1024, threads, bits_for(threads), kn);
    const u32 stalled_index = 7;   // workers use values from 1000 up
    // thread 0: a failed fast-path ticket, then the published request, then nothing
    const u64 T = q.cnt_of(q.Tail.fetch_add(q.cinc));
    gwf::Rec& r = q.Record[0];
    const u32 seq = r.seq1.load();
    r.localTail.store(T << 2);
    r.initTail.store(T << 2);
    r.index.store(stalled_index);
    r.enqueue.store(1);
    r.seq2.store(seq);
    r.pending.store(1);
    std::vector<std::vector<u32>> got(threads);
    std::vector<std::thread> ths;
    std::atomic<int> ready{0};
    for (u32 w = 1; w < threads; ++w) {
        ths.emplace_back([&, w]() {
            ready.fetch_add(1);
            while (ready.load() < (int)threads - 1) cpu_relax();
            for (u32 i = 0; i < ops; ++i) {
                q.enqueue_wf(1000 + w * ops + i, w);
                const u32 v = q.dequeue_wf(w);
                if (v != gwf::BOT) got[w].push_back(v);
            }
        });
    }
    for (auto& th : ths) th.join();
    // What the workers left in the queue, drained (as worker 1, whose operations
    // are over) before thread 0 resumes: with the workers' own dequeues it is
    // everything inserted while thread 0 was stalled.
    std::vector<u32> left;
    for (int k = 0; k < (int)(threads * ops + 16); ++k) {
        const u32 v = q.dequeue_wf(1);
        if (v == gwf::BOT) break;
        left.push_back(v);
    }
    uint64_t seen_while_stalled = 0;
    for (u32 w = 1; w < threads; ++w)
        for (u32 v : got[w]) seen_while_stalled += (v == stalled_index);
    for (u32 v : left) seen_while_stalled += (v == stalled_index);
    // thread 0 resumes: its own slow path must find the request finished
    q.enqueue_slow(T << 2, stalled_index, r, 0);
    r.pending.store(0);
    r.seq1.store(seq + 1);
    std::vector<u32> all(left);
    for (u32 w = 1; w < threads; ++w) all.insert(all.end(), got[w].begin(), got[w].end());
    for (int k = 0; k < (int)(threads * ops + 16); ++k) {
        const u32 v = q.dequeue_wf(0);
        if (v == gwf::BOT) break;
        all.push_back(v);
    }
    uint64_t stalled_total = 0, worker_once = 0;
    std::vector<u32> counts((size_t)threads * ops + 1000, 0);
    bool ok = true;
    for (u32 v : all) {
        if (v == stalled_index) { ++stalled_total; continue; }
        if (v < 1000 || v - 1000 >= threads * ops) { ok = false; continue; }
        ++counts[v - 1000];
    }
    const uint64_t enqueued = (uint64_t)(threads - 1) * ops;
    for (u32 w = 1; w < threads; ++w)
        for (u32 i = 0; i < ops; ++i) worker_once += counts[w * ops + i] == 1;
    stats[0] = seen_while_stalled;
    stats[1] = stalled_total;
    stats[2] = worker_once;
    stats[3] = enqueued;
    return (ok && seen_while_stalled == 1 && stalled_total == 1 && worker_once == enqueued) ? 1 : 0;
}

// Exactly-once stress of G-WFQ's slow paths (the CPU port): `threads` threads each
// run `ops` enqueue/dequeue pairs of their own values with the given patiences
// (1: every operation starts on the slow path; 2: after one failed fast-path
// attempt) and help delay, then the queue is drained.  Returns how many of `runs`
// runs lost or duplicated a value.  reference_rules bit 0 runs the phase-2 help of
// gwf_ring.hpp:548-590 verbatim, bit 1 the finalize_request scan of :316-326, bit 2
// the patience-1 slow-path start of :1242-1251.
int oracle_gwf_slow_stress(uint32_t threads, uint32_t ops, uint32_t enq_patience, uint32_t deq_patience,
                           uint32_t help_delay, uint32_t runs, int reference_rules) {
    if (threads < 1 || threads > 64 || ops == 0 || ops > 4096 || help_delay == 0 || runs == 0) return -1;
    int failed = 0;
    for (uint32_t run = 0; run < runs; ++run) {
        gwf::Ring q;
        gwf::Knobs kn;
        kn.help_delay = (int)help_delay;
        kn.enq_patience = (int)enq_patience;
        kn.deq_patience = (int)deq_patience;
        q.init(1024, threads, bits_for(threads), kn);
        q.reference_phase2_help = (reference_rules & 1) != 0;
        q.reference_finalize_scan = (reference_rules & 2) != 0;
        q.reference_patience1_start = (reference_rules & 4) != 0;
        std::vector<std::vector<u32>> got(threads);
        std::vector<std::thread> ths;
        std::atomic<int> ready{0};
        for (u32 w = 0; w < threads; ++w) {
            ths.emplace_back([&, w]() {
                ready.fetch_add(1);
                while (ready.load() < (int)threads) cpu_relax();
                for (u32 i = 0; i < ops; ++i) {
                    q.enqueue_wf(1000 + w * ops + i, w);
                    const u32 v = q.dequeue_wf(w);
                    if (v != gwf::BOT) got[w].push_back(v);
                }
            });
        }
        for (auto& th : ths) th.join();
        std::vector<u32> counts((size_t)threads * ops, 0);
        bool ok = true;
        auto take = [&](u32 v) {
            if (v < 1000 || v - 1000 >= threads * ops) ok = false;
            else ++counts[v - 1000];
        };
        for (auto& g : got)
            for (u32 v : g) take(v);
        for (u32 k = 0; k < threads * ops + 16; ++k) {
            const u32 v = q.dequeue_wf(0);
            if (v == gwf::BOT) break;
            take(v);
        }
        for (u32 c : counts) ok = ok && c == 1;
        failed += ok ? 0 : 1;
    }
    return failed;
}

// Split-role stress of the G-WFQ port's single ring: P producer threads enqueue K
// values each (P * K <= n, so the ring never overfills), C consumer threads dequeue
// until every value came out or a 2 s bound passes; then the ring is drained.
// Returns how many of `runs` runs lost, duplicated or invented a value.
// reference_finish = 1 runs the slow dequeue's completion rule of
// gwf_ring.hpp:729-731, 763-766 verbatim.
int oracle_gwf_split_stress(uint32_t P, uint32_t Cn, uint32_t K, uint32_t n, uint32_t enq_patience,
                            uint32_t deq_patience, uint32_t help_delay, uint32_t runs, int reference_finish) {
    const uint32_t threads = P + Cn;
    if (P == 0 || Cn == 0 || threads > 64 || K == 0 || (uint64_t)P * K > n || n < threads || (n & (n - 1)) ||
        help_delay == 0 || runs == 0)
        return -1;
    int failed = 0;
    for (uint32_t run = 0; run < runs; ++run) {
        gwf::Ring q;
        gwf::Knobs kn;
        kn.help_delay = (int)help_delay;
        kn.enq_patience = (int)enq_patience;
        kn.deq_patience = (int)deq_patience;
        q.init(n, threads, bits_for(threads), kn);
        q.reference_finish_rule = reference_finish != 0;
        const u32 total = P * K;
        std::vector<std::vector<u32>> got(threads);
        std::atomic<u32> taken{0};
        std::vector<std::thread> ths;
        std::atomic<int> ready{0};
        const auto deadline = std::chrono::steady_clock::now() + std::chrono::seconds(2);
        for (u32 w = 0; w < threads; ++w) {
            ths.emplace_back([&, w]() {
                ready.fetch_add(1);
                while (ready.load() < (int)threads) cpu_relax();
                if (w < P) {
                    for (u32 i = 0; i < K; ++i) q.enqueue_wf(1000 + w * K + i, w);
                    return;
                }
                while (taken.load() < total && std::chrono::steady_clock::now() < deadline) {
                    const u32 v = q.dequeue_wf(w);
                    if (v != gwf::BOT) {
                        got[w].push_back(v);
                        taken.fetch_add(1);
                    }
                }
            });
        }
        for (auto& th : ths) th.join();
        std::vector<u32> counts(total, 0);
        bool ok = true;
        auto take = [&](u32 v) {
            if (v < 1000 || v - 1000 >= total) ok = false;
            else ++counts[v - 1000];
        };
        for (auto& g : got)
            for (u32 v : g) take(v);
        for (u32 misses = 0, k = 0; k < total + 64 && misses < 64; ++k) {
            const u32 v = q.dequeue_wf(0);
            if (v == gwf::BOT) ++misses;
            else take(v);
        }
        for (u32 c : counts) ok = ok && c == 1;
        failed += ok ? 0 : 1;
    }
    return failed;
}

// Exactly-once stress of the YMC port: `threads` threads each run `ops`
// enqueue/dequeue pairs of their own values with the given patience (0: one
// fast-path attempt, then the slow path), then the queue is drained.  Returns how
// many of `runs` runs lost or duplicated a value.
int oracle_ymc_slow_stress(uint32_t threads, uint32_t ops, int patience, uint32_t runs) {
    if (threads < 1 || threads > 64 || ops == 0 || ops > 4096 || patience < 0 || runs == 0) return -1;
    int failed = 0;
    for (uint32_t run = 0; run < runs; ++run) {
        ymc::Queue q;
        q.init((int)threads, (int)ops);
        q.patience = patience;
        std::vector<std::vector<u64>> got(threads);
        std::vector<std::thread> ths;
        std::atomic<int> ready{0};
        for (u32 w = 0; w < threads; ++w) {
            ths.emplace_back([&, w]() {
                ready.fetch_add(1);
                while (ready.load() < (int)threads) cpu_relax();
                for (u32 i = 0; i < ops; ++i) {
                    q.enqueue(1000 + (u64)w * ops + i, (int)w);
                    const u64 v = q.dequeue((int)w);
                    if (v != ymc::EMPTY) got[w].push_back(v);
                }
            });
        }
        for (auto& th : ths) th.join();
        std::vector<u32> counts((size_t)threads * ops, 0);
        bool ok = true;
        auto take = [&](u64 v) {
            if (v < 1000 || v - 1000 >= (u64)threads * ops) ok = false;
            else ++counts[v - 1000];
        };
        for (auto& g : got)
            for (u64 v : g) take(v);
        for (u32 k = 0; k < threads * ops + 16; ++k) {
            const u64 v = q.dequeue(0);
            if (v == ymc::EMPTY) break;
            take(v);
        }
        for (u32 c : counts) ok = ok && c == 1;
        failed += ok ? 0 : 1;
    }
    return failed;
}

// Exactly-once stress of the device-path model (gwfmodel above): `threads` threads
// run `ops` iterations in balanced mode (mode 0: enqueue then dequeue) or split
// mode (mode 1: the first producer_percent % of threads enqueue, the rest
// dequeue) on a ring of n entries, then the queue is drained.  Returns how many of
// `runs` runs lost, duplicated or invented a value.
int oracle_gwf_device_model_stress(uint32_t threads, uint32_t ops, uint32_t n, uint32_t enq_patience,
                                   uint32_t deq_patience, uint32_t help_delay, int mode, int producer_percent,
                                   int prefetch, uint32_t runs) {
    if (threads < 1 || threads > 64 || ops == 0 || ops > 4096 || n < 2 || (n & (n - 1)) || n < threads ||
        help_delay == 0 || runs == 0 || prefetch < 0 || prefetch > 2)
        return -1;
    int failed = 0;
    for (uint32_t run = 0; run < runs; ++run) {
        gwfmodel::Queue d;
        d.prefetch = prefetch;
        gwf::Knobs k;
        k.enq_patience = (int)enq_patience;
        k.deq_patience = (int)deq_patience;
        k.help_delay = (int)help_delay;
        d.m.init(n, threads, bits_for(threads), k);
        std::vector<std::vector<u64>> got(threads), put(threads);
        std::vector<std::thread> ths;
        std::atomic<int> ready{0};
        for (u32 w = 0; w < threads; ++w) {
            ths.emplace_back([&, w]() {
                gwfmodel::Ctx x;
                ready.fetch_add(1);
                while (ready.load() < (int)threads) cpu_relax();
                const bool producer = (u64)w * 100 / threads < (u64)producer_percent;
                for (u32 i = 0; i < ops; ++i) {
                    const u64 v = 1000 + (u64)w * ops + i;
                    u64 o;
                    if (mode == 0 || producer)
                        if (d.enqueue_ptr(v, w, x)) put[w].push_back(v);
                    if (mode == 0 || !producer)
                        if (d.dequeue_ptr(&o, w, x)) got[w].push_back(o);
                }
            });
        }
        for (auto& th : ths) th.join();
        std::vector<u32> counts((size_t)threads * ops, 0), in((size_t)threads * ops, 0);
        for (auto& p : put)
            for (u64 v : p) in[v - 1000] = 1;
        bool ok = true;
        auto take = [&](u64 v) {
            if (v < 1000 || v - 1000 >= (u64)threads * ops || !in[v - 1000]) ok = false;
            else ++counts[v - 1000];
        };
        for (auto& g : got)
            for (u64 v : g) take(v);
        gwfmodel::Ctx x;
        u64 o;
        for (u32 misses = 0, k2 = 0; k2 < threads * ops + 64 && misses < 64; ++k2) {
            if (d.dequeue_ptr(&o, 0, x)) take(o);
            else ++misses;
        }
        for (size_t i = 0; i < counts.size(); ++i) ok = ok && counts[i] == in[i];
        failed += ok ? 0 : 1;
    }
    return failed;
}

// Exactly-once stress of the ports' MPMC queues as the reference composes them
// (gwf_ring.hpp:1362-1380, glf_queue.hpp:566-582): kind 0 G-WFQ with the given
// patiences and help delay, kind 1 G-LFQ (which has none); `threads` threads each
// run `ops` enqueue-then-dequeue pairs on an n-entry queue, which is then drained.
// Returns how many of `runs` runs lost, duplicated or invented a value.
int oracle_port_mpmc_stress(int kind, uint32_t threads, uint32_t ops, uint32_t n, uint32_t enq_patience,
                            uint32_t deq_patience, uint32_t help_delay, uint32_t runs) {
    if ((kind != 0 && kind != 1) || threads < 1 || threads > 64 || ops == 0 || ops > 4096 || n < 2 ||
        (n & (n - 1)) || n < threads || help_delay == 0 || runs == 0)
        return -1;
    int failed = 0;
    for (uint32_t run = 0; run < runs; ++run) {
        gwf::Mpmc wq;
        glf::Mpmc lq;
        if (kind == 0) {
            gwf::Knobs k;
            k.enq_patience = (int)enq_patience;
            k.deq_patience = (int)deq_patience;
            k.help_delay = (int)help_delay;
            wq.init(n, threads, bits_for(threads), k);
        } else {
            lq.init(n);
        }
        auto enqueue = [&](u64 v, u32 w) { return kind == 0 ? wq.enqueue(v, w) : lq.enqueue(v); };
        auto dequeue = [&](u64* o, u32 w) { return kind == 0 ? wq.dequeue(o, w) : lq.dequeue(o); };
        std::vector<std::vector<u64>> got(threads), put(threads);
        std::vector<std::thread> ths;
        std::atomic<int> ready{0};
        for (u32 w = 0; w < threads; ++w) {
            ths.emplace_back([&, w]() {
                ready.fetch_add(1);
                while (ready.load() < (int)threads) cpu_relax();
                for (u32 i = 0; i < ops; ++i) {
                    const u64 v = 1000 + (u64)w * ops + i;
                    u64 o;
                    if (enqueue(v, w)) put[w].push_back(v);
                    if (dequeue(&o, w)) got[w].push_back(o);
                }
            });
        }
        for (auto& th : ths) th.join();
        std::vector<u32> counts((size_t)threads * ops, 0), in((size_t)threads * ops, 0);
        for (auto& p : put)
            for (u64 v : p) in[v - 1000] = 1;
        bool ok = true;
        auto take = [&](u64 v) {
            if (v < 1000 || v - 1000 >= (u64)threads * ops || !in[v - 1000]) ok = false;
            else ++counts[v - 1000];
        };
        for (auto& g : got)
            for (u64 v : g) take(v);
        u64 o;
        for (u32 misses = 0, k2 = 0; k2 < threads * ops + 64 && misses < 64; ++k2) {
            if (dequeue(&o, 0)) take(o);
            else ++misses;
        }
        for (size_t i = 0; i < counts.size(); ++i) ok = ok && counts[i] == in[i];
        failed += ok ? 0 : 1;
    }
    return failed;
}

// Exactly-once stress of the G-LFQ device-path model (glfmodel above), driven as
// oracle_gwf_device_model_stress drives G-WFQ's: balanced (mode 0) or split
// (mode 1, the first producer_percent % of threads enqueue) on an n-entry queue,
// then drained; deq_wait is the dequeuer's bounded wait.  Returns how many of
// `runs` runs lost, duplicated or invented a value.
int oracle_glf_device_model_stress(uint32_t threads, uint32_t ops, uint32_t n, int mode, int producer_percent,
                                   uint32_t deq_wait, uint32_t runs) {
    if (threads < 1 || threads > 64 || ops == 0 || ops > 4096 || n < 2 || (n & (n - 1)) || runs == 0)
        return -1;
    int failed = 0;
    for (uint32_t run = 0; run < runs; ++run) {
        glfmodel::Queue d;
        d.init(n, deq_wait);
        std::vector<std::vector<u64>> got(threads), put(threads);
        std::vector<std::thread> ths;
        std::atomic<int> ready{0};
        for (u32 w = 0; w < threads; ++w) {
            ths.emplace_back([&, w]() {
                ready.fetch_add(1);
                while (ready.load() < (int)threads) cpu_relax();
                const bool producer = (u64)w * 100 / threads < (u64)producer_percent;
                for (u32 i = 0; i < ops; ++i) {
                    const u64 v = 1000 + (u64)w * ops + i;
                    u64 o;
                    if (mode == 0 || producer)
                        if (d.enqueue_ptr(v)) put[w].push_back(v);
                    if (mode == 0 || !producer)
                        if (d.dequeue_ptr(&o)) got[w].push_back(o);
                }
            });
        }
        for (auto& th : ths) th.join();
        std::vector<u32> counts((size_t)threads * ops, 0), in((size_t)threads * ops, 0);
        for (auto& p : put)
            for (u64 v : p) in[v - 1000] = 1;
        bool ok = true;
        auto take = [&](u64 v) {
            if (v < 1000 || v - 1000 >= (u64)threads * ops || !in[v - 1000]) ok = false;
            else ++counts[v - 1000];
        };
        for (auto& g : got)
            for (u64 v : g) take(v);
        u64 o;
        for (u32 misses = 0, k2 = 0; k2 < threads * ops + 64 && misses < 64; ++k2) {
            if (d.dequeue_ptr(&o)) take(o);
            else ++misses;
        }
        for (size_t i = 0; i < counts.size(); ++i) ok = ok && counts[i] == in[i];
        failed += ok ? 0 : 1;
    }
    return failed;
}

}  // extern "C"
