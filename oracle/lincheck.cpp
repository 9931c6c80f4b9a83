// FIFO linearizability checker: test infrastructure (the oracle), not product code.
//
// Restates, in C++, the checker the reference runs on its recorded histories:
//   correctness/lincheck/main.go:14-21   record fields {proc, op, arg, ret, call, end}
//   correctness/lincheck/main.go:63-75   op 0 = enqueue(arg), ret != 0 means it succeeded;
//                                        op 1 = dequeue, ret == 0 means "empty"
//   correctness/lincheck/main.go:90-136  sequential FIFO model: a failed enqueue is a
//                                        legal no-op; a dequeue of an empty queue is legal
//                                        only if it reported empty; a valued dequeue must
//                                        return the head
//   correctness/lincheck/main.go:138-159 10 s budget; "Linearizable (FIFO)" exits 0,
//                                        "Not linearizable (FIFO)" / "Unknown (timeout)" exit 1
//
// The reference delegates the search to github.com/anishathalye/porcupine v1.0.3
// (correctness/lincheck/go.mod:5), which is not vendored and cannot run here (no Go
// toolchain).  Its published method is the Wing & Gong search (J. Parallel Distrib.
// Comput. 1993) with Lowe's memoisation of (linearised-set, state) pairs ("Testing
// for linearizability", CCPE 2017).  `wgl_check` below is a fresh implementation of
// that method.
//
// `pattern_check` is a second, independent decision procedure for queue histories
// whose enqueued values are distinct (true of every history the harnesses emit: the
// value is (thread, sequence)).  It looks for the violation patterns of Henzinger,
// Sezgin and Vafeiadis ("Aspect-oriented linearizability proofs", CONCUR 2013):
// VFresh, VRepet, VOrd, and for "empty" dequeues an interval-cover test.  It runs in O(n log n)
// and so scales to the large histories that the exponential search cannot finish.
// For histories without empty dequeues the three value patterns are complete; for
// empty dequeues it only reports definite violations (see gcq_lincheck_patterns).
// Every pattern it reports is a definite violation, so gcq_lincheck_records runs it
// first and answers "Not linearizable" at once when it finds one; the exhaustive
// search then only has to confirm histories that are linearizable, which it does
// quickly, instead of exhausting every interleaving of a broken one.
//
// Extension: op code 2 is a dequeue that failed without effect (the BUSY result of
// SFQ's non-blocking dequeue, sfqueue_hip.cpp:109-128).  The reference's harness
// writes BUSY as an "empty" dequeue (correctness/history.cpp:134-140), which the
// FIFO model rejects whenever a later-ticket enqueue had already completed; modelled
// as a no-op, like a failed enqueue (main.go:100-103), it is always legal.

#include <algorithm>
#include <chrono>
#include <cinttypes>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <limits>
#include <string>
#include <unordered_map>
#include <vector>

extern "C" {

// One history record, same fields as a line of the JSONL history.
typedef struct {
    uint64_t proc;
    uint32_t op;   // 0 = enqueue, 1 = dequeue, 2 = dequeue that failed without effect
    uint32_t _pad;
    uint64_t arg;  // enqueue value
    uint64_t ret;  // enqueue: 1 ok / 0 failed; dequeue: value or 0 for empty
    int64_t call;  // logical call time
    int64_t end;   // logical return time
} gcq_hist_rec;

// Result of pattern_check: number of violating operations found per pattern.
typedef struct {
    uint64_t fresh;    // dequeue of a value never enqueued, or before its enqueue began
    uint64_t repeat;   // value dequeued more than once
    uint64_t order;    // FIFO order inverted between two values
    uint64_t empty;    // "empty" while some value was certainly in the queue
} gcq_pattern_report;

int gcq_lincheck_records(const gcq_hist_rec* recs, size_t n, double timeout_s);
int gcq_lincheck_search(const gcq_hist_rec* recs, size_t n, double timeout_s);
int gcq_lincheck_patterns(const gcq_hist_rec* recs, size_t n, gcq_pattern_report* out);
int gcq_lincheck_parse_jsonl(const char* path, gcq_hist_rec* out, size_t cap, size_t* n_out);
}

namespace {

// ------------------------------------------------------------------------------
// Wing-Gong / Lowe search
// ------------------------------------------------------------------------------

struct Event {
    int op;          // operation id
    bool is_call;
    int64_t time;
    Event* prev = nullptr;
    Event* next = nullptr;
    Event* match = nullptr;  // call -> its return
};

struct Op {
    bool is_enq;
    bool ok;        // enqueue succeeded / dequeue returned a value
    bool noop;      // failed without effect (BUSY dequeue)
    uint64_t val;   // enqueue argument or dequeued value
};

// The FIFO model of main.go:93-121, applied in place with an undo record.
// Returns false if the step is illegal.  kind: 0 no-op, 1 pushed, 2 popped.
static bool model_step(std::deque<uint64_t>& q, const Op& o, int* kind) {
    if (o.noop) { *kind = 0; return true; }
    if (o.is_enq) {
        if (!o.ok) { *kind = 0; return true; }   // failed enqueue: legal no-op
        q.push_back(o.val);
        *kind = 1;
        return true;
    }
    if (q.empty()) { *kind = 0; return !o.ok; }  // empty queue: only "empty" is legal
    if (!o.ok) return false;                     // non-empty queue reported empty
    if (q.front() != o.val) return false;        // must return the head
    q.pop_front();
    *kind = 2;
    return true;
}

static inline uint64_t mix64(uint64_t x) {
    x ^= x >> 30; x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27; x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}

struct CacheKey {
    std::vector<uint64_t> bits;
    std::vector<uint64_t> state;
};

class Wgl {
public:
    Wgl(std::vector<Op> ops, const std::vector<int64_t>& call, const std::vector<int64_t>& ret)
        : ops_(std::move(ops)) {
        const int n = (int)ops_.size();
        prepare_order(call, ret);
        events_.resize(2 * n);
        for (int i = 0; i < n; ++i) {
            Event* c = &events_[2 * i];
            Event* r = &events_[2 * i + 1];
            c->op = r->op = i;
            c->is_call = true;  c->time = call[i];
            r->is_call = false; r->time = ret[i];
            c->match = r;
        }
        std::vector<Event*> order;
        order.reserve(2 * n);
        for (auto& e : events_) order.push_back(&e);
        // Time order; at equal times calls come before returns so that touching
        // intervals count as overlapping.
        std::stable_sort(order.begin(), order.end(), [](const Event* a, const Event* b) {
            if (a->time != b->time) return a->time < b->time;
            return a->is_call && !b->is_call;
        });
        head_.next = nullptr;
        Event* prev = &head_;
        for (Event* e : order) { prev->next = e; e->prev = prev; prev = e; }
        prev->next = nullptr;
        words_ = (n + 63) / 64;
        zob_.resize(n);
        for (int i = 0; i < n; ++i) zob_[i] = mix64(0x9e3779b97f4a7c15ULL * (uint64_t)(i + 1));
    }

    // 0 linearizable, 1 not linearizable, 2 out of time
    //
    // Pruning beyond the published method: only enqueues are branch points.
    //  * An operation that is legal now and leaves the state unchanged (failed
    //    enqueue, failed-without-effect dequeue, "empty" on an empty queue) is
    //    linearised at once: the state is the same either way and taking it only
    //    relaxes the real-time constraint of its return event.
    //  * A dequeue whose value is at the head is also taken at once: in any
    //    successful order from here, everything before it is an enqueue or a no-op
    //    (no other dequeue can return the head, no "empty" can see a non-empty
    //    queue), so moving it first stays legal, and its call is already due.
    // At every node these dominant operations are taken first, before any enqueue is
    // tried; when every continuation after one fails, skipping it would fail too, so
    // the search backtracks past it to the last enqueue choice.  With distinct values
    // the operation whose return is next decides what can help: if it is a dequeue
    // that is not dominant, only its own value's enqueue into an empty queue can
    // (anything else, including more enqueues, only delays the failure).
    int run(double timeout_s) {
        const auto t0 = std::chrono::steady_clock::now();
        std::vector<uint64_t> bits(words_, 0);
        uint64_t bits_hash = 0;
        std::deque<uint64_t> state;
        struct Frame { Event* call; int kind; uint64_t val; int cand; };
        std::vector<Frame> stack;
        uint64_t iters = 0;
        bool backtrack = false, fresh = true;
        int next_cand = 0;          // first enqueue candidate to try at this node
        std::vector<Event*> cands;
        // apply op of call event x; false if illegal; on success pushes a frame or,
        // when the configuration was seen before, undoes it and requests a backtrack
        auto take = [&](Event* x, int* kind_out) -> int {
            const Op& o = ops_[x->op];
            int kind = 0;
            const uint64_t popped = state.empty() ? 0 : state.front();
            if (o.is_enq && o.ok && !o.noop && !order_ok(x->op)) return 0;
            if (!model_step(state, o, &kind)) return 0;
            if (kind == 1 && pos_[x->op] >= 0) fen_add(pos_[x->op], 1);
            bits[x->op >> 6] |= (1ULL << (x->op & 63));
            const uint64_t nh = bits_hash ^ zob_[x->op];
            *kind_out = kind;
            if (!remember(bits, nh, state)) {
                bits[x->op >> 6] &= ~(1ULL << (x->op & 63));
                undo(state, kind, popped);
                if (kind == 1 && pos_[x->op] >= 0) fen_add(pos_[x->op], -1);
                return 2;
            }
            stack.push_back({x, kind, popped, -1});
            bits_hash = nh;
            lift(x);
            return 1;
        };
        auto dominant = [&](Event* x) {
            const Op& o = ops_[x->op];
            if (o.noop || (o.is_enq && !o.ok)) return true;
            if (o.is_enq) return false;
            if (!o.ok) return state.empty();
            return !state.empty() && state.front() == o.val;
        };
        while (head_.next != nullptr) {
            if ((++iters & 0xFFF) == 0) {
                double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
                if (el > timeout_s) return 2;
            }
            if (backtrack) {
                backtrack = false;
                for (;;) {
                    if (stack.empty()) return 1;
                    Frame f = stack.back();
                    stack.pop_back();
                    undo(state, f.kind, f.val);
                    if (f.kind == 1 && pos_[f.call->op] >= 0) fen_add(pos_[f.call->op], -1);
                    bits[f.call->op >> 6] &= ~(1ULL << (f.call->op & 63));
                    bits_hash ^= zob_[f.call->op];
                    unlift(f.call);
                    if (f.kind == 1) { next_cand = f.cand + 1; fresh = false; break; }
                }
                continue;
            }
            if (fresh) {
                // dominant operations among those already called
                bool took = false;
                for (Event* x = head_.next; x && x->is_call; x = x->next) {
                    if (!dominant(x)) continue;
                    int kind = 0;
                    const int r = take(x, &kind);
                    if (r == 1) { took = true; break; }
                    if (r == 2) { backtrack = true; break; }
                }
                if (backtrack || took) continue;
                fresh = false;
                next_cand = 0;
            }
            // Branch on an enqueue among those already called, earliest deadline
            // first: the queue order must follow the dequeue order, so the value
            // whose dequeue returns first is the most likely next one.  The order is
            // a heuristic only; backtracking still tries every candidate.
            cands.clear();
            Event* first_ret = head_.next;
            while (first_ret && first_ret->is_call) first_ret = first_ret->next;
            const Op* due = first_ret ? &ops_[first_ret->op] : nullptr;
            if (distinct_ && due && !due->is_enq && !due->noop) {
                // The operation whose return comes next is a dequeue that is not
                // dominant now.  An "empty" needs an empty queue and a valued
                // dequeue needs its value at the head; adding enqueues helps only
                // if the queue is empty and the dequeue's own value goes in next.
                if (!due->ok || !state.empty()) { backtrack = true; continue; }
                for (Event* x = head_.next; x && x->is_call; x = x->next) {
                    const Op& o = ops_[x->op];
                    if (o.is_enq && o.ok && !o.noop && o.val == due->val) cands.push_back(x);
                }
            } else {
                for (Event* x = head_.next; x && x->is_call; x = x->next) {
                    const Op& o = ops_[x->op];
                    if (o.is_enq && o.ok && !o.noop) cands.push_back(x);
                }
            }
            std::stable_sort(cands.begin(), cands.end(),
                             [&](const Event* a, const Event* b) { return deadline_[a->op] < deadline_[b->op]; });
            bool took = false;
            for (int ci = next_cand; ci < (int)cands.size(); ++ci) {
                int kind = 0;
                const int r = take(cands[ci], &kind);
                if (r == 1) { stack.back().cand = ci; took = true; break; }
            }
            if (took) { fresh = true; continue; }
            backtrack = true;   // no enqueue can go next: undo the last choice
        }
        return 0;
    }

private:
    // FIFO order constraints for histories whose values are distinct.  Dequeued
    // values are ranked by the return time of their dequeue; an enqueue of v may be
    // linearised only once every value whose dequeue returned before deq(v) was
    // called has been enqueued (otherwise that value would sit behind v yet leave
    // first).  A value never dequeued needs every dequeued value enqueued before it.
    // need_[op] is that prefix length, pos_[op] the op's own rank (-1 if none).
    void prepare_order(const std::vector<int64_t>& call, const std::vector<int64_t>& ret) {
        const int n = (int)ops_.size();
        need_.assign(n, 0);
        pos_.assign(n, -1);
        deadline_.assign(n, std::numeric_limits<int64_t>::max());
        std::unordered_map<uint64_t, int> enq_of, deq_of;
        distinct_ = true;
        for (int i = 0; i < n; ++i) {
            const Op& o = ops_[i];
            if (o.noop || !o.ok) continue;
            auto& m = o.is_enq ? enq_of : deq_of;
            if (!m.emplace(o.val, i).second) distinct_ = false;
        }
        if (!distinct_) return;
        std::vector<std::pair<int64_t, uint64_t>> ends;   // (deq return, value)
        for (auto& kv : deq_of) {
            if (!enq_of.count(kv.first)) { distinct_ = false; return; }
            ends.emplace_back(ret[kv.second], kv.first);
        }
        std::sort(ends.begin(), ends.end());
        ndeq_ = (int)ends.size();
        std::vector<int64_t> end_times(ndeq_);
        for (int k = 0; k < ndeq_; ++k) {
            end_times[k] = ends[k].first;
            pos_[enq_of[ends[k].second]] = k;
        }
        for (auto& kv : enq_of) {
            const int e = kv.second;
            auto d = deq_of.find(kv.first);
            if (d == deq_of.end()) { need_[e] = ndeq_; continue; }
            deadline_[e] = ret[d->second];
            need_[e] = (int)(std::lower_bound(end_times.begin(), end_times.end(), call[d->second]) - end_times.begin());
        }
        fen_.assign(ndeq_ + 1, 0);
    }
    void fen_add(int i, int v) { for (++i; i <= ndeq_; i += i & -i) fen_[i] += v; }
    int fen_sum(int k) const { int s = 0; for (; k > 0; k -= k & -k) s += fen_[k]; return s; }
    bool order_ok(int op) const { return !distinct_ || fen_sum(need_[op]) == need_[op]; }

    static void undo(std::deque<uint64_t>& q, int kind, uint64_t popped) {
        if (kind == 1) q.pop_back();
        else if (kind == 2) q.push_front(popped);
    }
    void lift(Event* c) {
        c->prev->next = c->next;
        if (c->next) c->next->prev = c->prev;
        Event* r = c->match;
        r->prev->next = r->next;
        if (r->next) r->next->prev = r->prev;
    }
    void unlift(Event* c) {
        Event* r = c->match;
        r->prev->next = r;
        if (r->next) r->next->prev = r;
        c->prev->next = c;
        if (c->next) c->next->prev = c;
    }
    // Insert (bits, state) into the memo table; false if it was already there.
    bool remember(const std::vector<uint64_t>& bits, uint64_t bits_hash,
                  const std::deque<uint64_t>& state) {
        uint64_t h = bits_hash;
        for (uint64_t v : state) h = mix64(h ^ v) + 0x632be59bd9b4e019ULL;
        auto& bucket = cache_[h];
        for (const CacheKey& k : bucket) {
            if (k.state.size() != state.size()) continue;
            if (k.bits != bits) continue;
            if (std::equal(k.state.begin(), k.state.end(), state.begin())) return false;
        }
        bucket.push_back(CacheKey{bits, std::vector<uint64_t>(state.begin(), state.end())});
        return true;
    }

    std::vector<Op> ops_;
    std::vector<Event> events_;
    Event head_{};
    int words_ = 0;
    std::vector<uint64_t> zob_;
    std::unordered_map<uint64_t, std::vector<CacheKey>> cache_;
    bool distinct_ = false;
    int ndeq_ = 0;
    std::vector<int> need_, pos_, fen_;
    std::vector<int64_t> deadline_;
};

// ------------------------------------------------------------------------------
// Violation patterns for queues with distinct values
// ------------------------------------------------------------------------------

struct ValInfo {
    bool enq = false;
    int64_t enq_call = 0, enq_end = 0;
    int deqs = 0;
    int64_t deq_call = 0, deq_end = 0;
};

}  // namespace

// The exact search alone (no pattern pre-check); exported so the tests can
// cross-check it against brute-force enumeration on small histories.
extern "C" int gcq_lincheck_search(const gcq_hist_rec* recs, size_t n, double timeout_s) {
    if (n > (size_t)std::numeric_limits<int>::max() / 2) return -1;
    std::vector<Op> ops(n);
    std::vector<int64_t> call(n), ret(n);
    for (size_t i = 0; i < n; ++i) {
        const gcq_hist_rec& r = recs[i];
        if (r.op > 2) return -1;
        ops[i].is_enq = (r.op == 0);
        ops[i].noop = (r.op == 2);
        ops[i].ok = (r.ret != 0);
        ops[i].val = ops[i].is_enq ? r.arg : r.ret;
        call[i] = r.call;
        ret[i] = r.end;
        if (r.end < r.call) return -1;
    }
    Wgl w(std::move(ops), call, ret);
    return w.run(timeout_s);
}

// The verdict: a pattern found is a definite violation; a history with distinct
// values and no "empty" dequeue and no pattern is linearizable (Henzinger et al.,
// Theorem on queues: VFresh, VRepet and VOrd are the only violations when no
// dequeue reports empty); anything else goes to the exact search.
extern "C" int gcq_lincheck_records(const gcq_hist_rec* recs, size_t n, double timeout_s) {
    gcq_pattern_report rep;
    int prc = gcq_lincheck_patterns(recs, n, &rep);
    if (prc == 1) return 1;          // a definite violation
    if (prc == -1) return -1;        // malformed
    if (prc == 0) {
        bool any_empty = false;
        for (size_t i = 0; i < n && !any_empty; ++i) any_empty = (recs[i].op == 1 && recs[i].ret == 0);
        if (!any_empty) return 0;
    }
    return gcq_lincheck_search(recs, n, timeout_s);
}

// Note on emptiness: an "empty" dequeue d is flagged when, at every instant of its
// interval, some value was certainly queued (its enqueue had returned and its
// dequeue, if any, had not been called).  That is a definite violation.  Other ways
// an "empty" can be illegal (through the order in which concurrent operations must
// be placed) are left to the exact search.
extern "C" int gcq_lincheck_patterns(const gcq_hist_rec* recs, size_t n, gcq_pattern_report* out) {
    std::memset(out, 0, sizeof(*out));
    std::unordered_map<uint64_t, ValInfo> vals;
    vals.reserve(n);
    std::vector<size_t> empties;
    for (size_t i = 0; i < n; ++i) {
        const gcq_hist_rec& r = recs[i];
        if (r.op > 2 || r.end < r.call) return -1;
        if (r.op == 2) continue;       // no-op dequeue
        if (r.op == 0) {
            if (r.ret == 0) continue;  // failed enqueue: no effect
            ValInfo& v = vals[r.arg];
            if (v.enq) return -2;       // values are not distinct: procedure not applicable
            v.enq = true; v.enq_call = r.call; v.enq_end = r.end;
        } else if (r.ret == 0) {
            empties.push_back(i);
        }
    }
    for (size_t i = 0; i < n; ++i) {
        const gcq_hist_rec& r = recs[i];
        if (r.op != 1 || r.ret == 0) continue;
        auto it = vals.find(r.ret);
        if (it == vals.end() || !it->second.enq) { out->fresh++; continue; }
        ValInfo& v = it->second;
        if (r.end < v.enq_call) out->fresh++;
        if (++v.deqs > 1) { out->repeat++; continue; }
        v.deq_call = r.call; v.deq_end = r.end;
    }
    const int64_t INF = std::numeric_limits<int64_t>::max();
    // Values sorted by the end of their enqueue.
    std::vector<const ValInfo*> by_end;
    by_end.reserve(vals.size());
    for (auto& kv : vals) by_end.push_back(&kv.second);
    std::sort(by_end.begin(), by_end.end(),
              [](const ValInfo* a, const ValInfo* b) { return a->enq_end < b->enq_end; });
    // VOrd: enq(a) before enq(b) in real time, b dequeued, and a dequeued only after
    // deq(b) returned (or never).  Sweep b by enqueue call time with a running maximum
    // of deq_call(a) over the values whose enqueue already returned.
    {
        std::vector<const ValInfo*> by_call(by_end);
        std::sort(by_call.begin(), by_call.end(),
                  [](const ValInfo* a, const ValInfo* b) { return a->enq_call < b->enq_call; });
        size_t k = 0;
        int64_t max_deq_call = std::numeric_limits<int64_t>::min();
        for (const ValInfo* b : by_call) {
            while (k < by_end.size() && by_end[k]->enq_end < b->enq_call) {
                const ValInfo* a = by_end[k++];
                int64_t dc = a->deqs ? a->deq_call : INF;
                max_deq_call = std::max(max_deq_call, dc);
            }
            if (b->deqs && max_deq_call > b->deq_end) out->order++;
        }
    }
    // Empty dequeues: value v is certainly queued strictly between the return of
    // enq(v) and the call of deq(v) (or forever if never dequeued).  An "empty" d
    // has no legal linearisation point if those open intervals cover all of d's
    // interval.  Greedy cover with a prefix maximum over intervals sorted by start.
    {
        std::vector<std::pair<int64_t, int64_t>> iv;   // (enq_end, deq_call or INF)
        iv.reserve(by_end.size());
        for (const ValInfo* a : by_end) iv.emplace_back(a->enq_end, a->deqs ? a->deq_call : INF);
        std::vector<int64_t> pmax(iv.size() + 1, std::numeric_limits<int64_t>::min());
        for (size_t k = 0; k < iv.size(); ++k) pmax[k + 1] = std::max(pmax[k], iv[k].second);
        for (size_t i : empties) {
            int64_t reach = recs[i].call;
            const int64_t goal = recs[i].end;
            for (;;) {
                // intervals starting before `reach`
                size_t k = std::lower_bound(iv.begin(), iv.end(), std::make_pair(reach, std::numeric_limits<int64_t>::min())) - iv.begin();
                int64_t best = pmax[k];
                if (best <= reach) break;
                reach = best;
                if (reach >= goal) break;
            }
            if (reach >= goal) out->empty++;
        }
    }
    return (out->fresh | out->repeat | out->order | out->empty) ? 1 : 0;
}

// ------------------------------------------------------------------------------
// JSONL reader (the record format written by correctness/history.cpp:271-280)
// ------------------------------------------------------------------------------

static bool json_field(const char* line, const char* key, uint64_t* v) {
    const char* p = std::strstr(line, key);
    if (!p) return false;
    p += std::strlen(key);
    while (*p == ' ' || *p == ':' || *p == '"') ++p;
    char* endp = nullptr;
    unsigned long long x = std::strtoull(p, &endp, 10);
    if (endp == p) return false;
    *v = (uint64_t)x;
    return true;
}

extern "C" int gcq_lincheck_parse_jsonl(const char* path, gcq_hist_rec* out, size_t cap, size_t* n_out) {
    FILE* f = std::fopen(path, "rb");
    if (!f) return -1;
    size_t n = 0;
    char buf[1024];
    int rc = 0;
    while (std::fgets(buf, sizeof buf, f)) {
        if (buf[0] == '\n' || buf[0] == 0) continue;
        uint64_t proc, op, arg, ret, call, end;
        if (!json_field(buf, "\"proc\"", &proc) || !json_field(buf, "\"op\"", &op) ||
            !json_field(buf, "\"arg\"", &arg) || !json_field(buf, "\"ret\"", &ret) ||
            !json_field(buf, "\"call\"", &call) || !json_field(buf, "\"end\"", &end)) {
            rc = -2;
            break;
        }
        if (out && n < cap) {
            out[n].proc = proc; out[n].op = (uint32_t)op; out[n]._pad = 0;
            out[n].arg = arg; out[n].ret = ret;
            out[n].call = (int64_t)call; out[n].end = (int64_t)end;
        }
        ++n;
    }
    std::fclose(f);
    *n_out = n;
    if (rc) return rc;
    return (out && n > cap) ? -3 : 0;
}

#ifdef GCQ_LINCHECK_MAIN
// Command line, same contract as correctness/lincheck/main.go:34-159:
//   lincheck <history.jsonl>  prints one of the three verdicts, exits 0 only if linearizable.
//   --patterns                also runs the pattern procedure and prints its counts.
//   --timeout S               search budget in seconds (default 10, main.go:138).
int main(int argc, char** argv) {
    const char* path = nullptr;
    double timeout = 10.0;
    bool patterns = false;
    for (int i = 1; i < argc; ++i) {
        if (!std::strcmp(argv[i], "--patterns")) patterns = true;
        else if (!std::strcmp(argv[i], "--timeout") && i + 1 < argc) timeout = std::atof(argv[++i]);
        else path = argv[i];
    }
    if (!path) {
        std::fprintf(stderr, "usage: %s <history.jsonl> [--timeout S] [--patterns]\n", argv[0]);
        return 2;
    }
    size_t n = 0;
    if (gcq_lincheck_parse_jsonl(path, nullptr, 0, &n) != 0 && n == 0) {
        std::fprintf(stderr, "cannot read %s\n", path);
        return 2;
    }
    std::vector<gcq_hist_rec> recs(n);
    if (gcq_lincheck_parse_jsonl(path, recs.data(), n, &n) != 0) {
        std::fprintf(stderr, "malformed history %s\n", path);
        return 2;
    }
    if (patterns) {
        gcq_pattern_report rep;
        int prc = gcq_lincheck_patterns(recs.data(), n, &rep);
        std::printf("patterns: fresh=%" PRIu64 " repeat=%" PRIu64 " order=%" PRIu64 " empty=%" PRIu64 " (%s)\n",
                    rep.fresh, rep.repeat, rep.order, rep.empty,
                    prc == 0 ? "none" : prc == 1 ? "violations" : "values not distinct");
    }
    int rc = gcq_lincheck_records(recs.data(), n, timeout);
    if (rc == 0) std::printf("Linearizable (FIFO)\n");
    else if (rc == 1) std::printf("Not linearizable (FIFO)\n");
    else if (rc == 2) std::printf("Unknown (timeout)\n");
    else { std::printf("malformed history\n"); return 2; }
    return rc == 0 ? 0 : 1;
}
#endif
