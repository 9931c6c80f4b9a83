// history: the history generator (correctness/history.cpp), over libgcq.so.
//
// Command line as the reference (history.cpp:294-299):
//   history [out.jsonl] [threads] [ops] [mode] [producer_percent]
// mode 0 alternates enqueue/dequeue per thread, mode 1 splits threads into
// producers and consumers.  Output: one JSON object per completed operation,
// sorted by (call, end, proc, op), in the reference's line format
// (history.cpp:271-280).  Values are (tid << 32) | (seq + 1) (history.cpp:184); SFQ
// uses its 15+16-bit encoding and caps threads and ops as the reference does
// (history.cpp:285-292).
//
// SFQ's "busy" dequeue (failed without effect) is written as the reference writes
// it, op 1 with ret 0; HIST_KEEP_BUSY=1 in the environment writes it as op 2, which
// the checker in oracle/ reads as a no-op.
//
// Knobs (compile-time): HIST_THREADS, HIST_OPS, HIST_MODE, HIST_PRODUCER_PERCENT,
// HIST_BLOCK_SIZE.  Exit codes as the reference: 2 bad arguments, 3 nothing to do.
#include <vector>

#include "harness_common.h"

#ifndef HIST_THREADS
#define HIST_THREADS 64
#endif
#ifndef HIST_OPS
#define HIST_OPS 16
#endif
#ifndef HIST_MODE
#define HIST_MODE 0
#endif
#ifndef HIST_PRODUCER_PERCENT
#define HIST_PRODUCER_PERCENT 50
#endif
#ifndef HIST_BLOCK_SIZE
#define HIST_BLOCK_SIZE 256
#endif

int main(int argc, char** argv) {
    const char* out_path = (argc > 1) ? argv[1] : "correctness/histories/history.jsonl";
    const int threads = (argc > 2) ? std::atoi(argv[2]) : HIST_THREADS;
    int ops = (argc > 3) ? std::atoi(argv[3]) : HIST_OPS;
    const int mode = (argc > 4) ? std::atoi(argv[4]) : HIST_MODE;
    const int producer_percent = (argc > 5) ? std::atoi(argv[5]) : HIST_PRODUCER_PERCENT;
    if (threads <= 0 || ops <= 0) return 2;
    const int kind = harness::queue_kind();
    if (kind == GCQ_SFQ) {   // 15-bit thread id, 16-bit sequence
        if (threads > (1 << 15)) return 3;
        if (ops > 0xFFFF) ops = 0xFFFF;
    }
    const char* keep = std::getenv("HIST_KEEP_BUSY");
    const bool keep_busy = keep && std::atoi(keep) != 0;

    gcq_queue* q = nullptr;
    harness::check(gcq_create(kind, harness::default_capacity_log2(kind), (uint32_t)threads, nullptr, &q),
                   "gcq_create");
    const size_t cap = (size_t)threads * (size_t)ops * 2 + 16;
    std::vector<gcq_log_entry> recs(cap);
    size_t n = 0;
    harness::check(gcq_run_history(q, (uint32_t)threads, HIST_BLOCK_SIZE, (uint32_t)ops, mode, producer_percent, 0,
                                   recs.data(), cap, &n, nullptr),
                   "gcq_run_history");
    gcq_destroy(q);

    FILE* f = std::fopen(out_path, "wb");
    if (!f) return 1;
    for (size_t i = 0; i < n; ++i) {
        const gcq_log_entry& e = recs[i];
        unsigned op = e.op;
        unsigned long long ret = e.ret;
        if (op == 2 && !keep_busy) { op = 1; ret = 0; }
        std::fprintf(f, "{\"proc\":%llu,\"op\":%u,\"arg\":%llu,\"ret\":%llu,\"call\":%llu,\"end\":%llu}\n",
                     (unsigned long long)e.proc, op, (unsigned long long)e.arg, ret, (unsigned long long)e.call,
                     (unsigned long long)e.end);
    }
    std::fclose(f);
    return 0;
}
