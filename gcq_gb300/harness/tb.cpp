// tb: the fixed-duration throughput harness (throughout_bench.cpp), over libgcq.so.
//
// Same sweep, knobs, console lines and CSV columns as the reference main
// (throughout_bench.cpp:1057-1160): balanced mode, then split mode at 25/50/75 %
// producers, over 512..32768 threads; one queue per (mode, threads) point.  The
// chunks run through gcq_tb_run, which replays a CUDA graph of chunk launches
// instead of launching and synchronising each chunk from the host.
//
// Knobs (compile-time, as the reference's -D flags): RUN_MS, WARMUP_MS, CHUNK_OPS,
// BLOCK_SIZE, ONLY_BALANCED, ONLY_SPLIT, CSV_FILE, MODE_FIFO, FIFO_OPS_PER_THREAD,
// FIFO_BLOCK_SIZE.  Extension: TB_THREADS="512,1024" in the environment replaces
// the thread sweep.
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <vector>

#include "harness_common.h"

#ifndef RUN_MS
#define RUN_MS 500
#endif
#ifndef WARMUP_MS
#define WARMUP_MS 100
#endif
#ifndef CHUNK_OPS
#define CHUNK_OPS 64
#endif
#ifndef BLOCK_SIZE
#define BLOCK_SIZE 256
#endif
#ifndef ONLY_BALANCED
#define ONLY_BALANCED 0
#endif
#ifndef ONLY_SPLIT
#define ONLY_SPLIT 0
#endif
#ifndef CSV_FILE
#define CSV_FILE "benchmark_results.csv"
#endif
#ifndef MODE_FIFO
#define MODE_FIFO 0
#endif
#ifndef FIFO_OPS_PER_THREAD
#define FIFO_OPS_PER_THREAD 64
#endif
#ifndef FIFO_BLOCK_SIZE
#define FIFO_BLOCK_SIZE BLOCK_SIZE
#endif
#ifndef GRAPH_CHUNKS
#define GRAPH_CHUNKS 16
#endif

namespace {

struct Stats { uint64_t enq_success, enq_fail, deq_success, deq_empty; };

void print_result_line(const std::string& label, int threads, double ms, const Stats& s) {
    const double sec = ms / 1000.0;
    const double enq = (double)s.enq_success / sec / 1e6, deq = (double)s.deq_success / sec / 1e6;
    const double empty = (double)s.deq_empty / sec / 1e6, fail = (double)s.enq_fail / sec / 1e6;
    const double succ = (double)(s.enq_success + s.deq_success) / sec / 1e6;
    std::cout << std::setw(12) << label << " | threads=" << std::setw(6) << threads << " | time=" << std::fixed
              << std::setprecision(1) << std::setw(7) << ms << " ms"
              << " | succ=" << std::setprecision(2) << std::setw(9) << succ << " Mops/s"
              << " | enq=" << std::setw(9) << enq << " | deq=" << std::setw(9) << deq << " | empty=" << std::setw(9)
              << empty << " | fail=" << std::setw(9) << fail << "\n";
}

void append_csv(std::ofstream& csv, const std::string& gpu, const char* qname, const std::string& mode, int pp,
                int threads, double ms, const Stats& s) {
    const double sec = ms / 1000.0;
    csv << harness::csv_escape(gpu) << "," << qname << "," << mode << "," << pp << "," << threads << "," << RUN_MS
        << "," << WARMUP_MS << "," << CHUNK_OPS << "," << BLOCK_SIZE << "," << std::fixed << std::setprecision(3)
        << ms << "," << s.enq_success << "," << s.enq_fail << "," << s.deq_success << "," << s.deq_empty << ","
        << std::setprecision(6) << (double)(s.enq_success + s.deq_success) / sec / 1e6 << ","
        << (double)s.enq_success / sec / 1e6 << "," << (double)s.deq_success / sec / 1e6 << ","
        << (double)s.deq_empty / sec / 1e6 << "," << (double)s.enq_fail / sec / 1e6 << "\n";
}

void print_fifo(const gcq_fifo_result& r) {
    if (r.verified < 0) {
        std::cout << "FIFO check skipped (capacity / threads leaves 0 ops per thread)\n";
        return;
    }
    std::cout << "FIFO in: " << r.in_count << "\n";
    std::cout << "FIFO out: " << r.out_count << "\n";
    std::cout << "FIFO verified: " << (r.verified ? "YES" : "NO");
    if (!r.verified)
        std::cout << " (oob=" << r.err_oob << ", dup=" << r.err_dup << ", order=" << r.err_order
                  << ", missing=" << r.err_missing << ", gt1=" << r.err_gt1 << ")";
    std::cout << "\n";
}

std::vector<int> thread_counts() {
    std::vector<int> t = {512, 1024, 2048, 4096, 8192, 16384, 32768};
    const char* env = std::getenv("TB_THREADS");
    if (env && *env) {
        t.clear();
        std::stringstream ss(env);
        std::string item;
        while (std::getline(ss, item, ',')) t.push_back(std::atoi(item.c_str()));
    }
    return t;
}

Stats run_point(int kind, int mode, int pp, int threads, double* ms, gcq_queue** keep) {
    gcq_queue* q = nullptr;
    harness::check(gcq_create(kind, harness::default_capacity_log2(kind), (uint32_t)threads, nullptr, &q),
                   "gcq_create");
    gcq_tb_result r;
    harness::check(gcq_tb_run(q, mode, pp, (uint32_t)threads, BLOCK_SIZE, CHUNK_OPS, WARMUP_MS, RUN_MS,
                              GRAPH_CHUNKS, &r),
                   "gcq_tb_run");
    *ms = r.gpu_ms;
    *keep = q;
    return Stats{r.counters.enq_success, r.counters.enq_fail, r.counters.deq_success, r.counters.deq_empty};
}

}  // namespace

int main() {
    const int kind = harness::queue_kind();
    const std::string gpu = harness::gpu_name();
    const char* qname = harness::queue_name(kind);
    const std::string csv_path = CSV_FILE;
    const bool csv_exists = std::ifstream(csv_path).good();
    std::ofstream csv(csv_path, std::ios::app);
    if (!csv) {
        std::cerr << "Failed to open CSV file: " << csv_path << "\n";
        return 1;
    }
    if (!csv_exists)
        csv << "gpu_name,queue,mode,producer_percent,threads,run_ms,warmup_ms,chunk_ops,block_size,elapsed_ms,"
               "enq_success,enq_fail,deq_success,deq_empty,succ_mops,enq_mops,deq_mops,empty_mops,fail_mops\n";

    std::cout << "GPU: " << gpu << "\n";
    std::cout << "Queue: " << qname << "\n";
    std::cout << "Method: fixed-duration timed throughput harness\n";
    std::cout << "RUN_MS=" << RUN_MS << " WARMUP_MS=" << WARMUP_MS << " CHUNK_OPS=" << CHUNK_OPS
              << " BLOCK_SIZE=" << BLOCK_SIZE << " MODE_FIFO=" << MODE_FIFO << "\n";
    std::cout << "Backend: libgcq.so (sm_103a), capacity 2^" << harness::default_capacity_log2(kind)
              << ", chunks replayed as a CUDA graph of " << GRAPH_CHUNKS << " launches\n";

    const std::vector<int> counts = thread_counts();
    const int producer_percents[] = {25, 50, 75};
    if (!ONLY_SPLIT) {
        std::cout << "=== Balanced Pairwise Timed Benchmark ===\n";
        std::cout << "Each active thread repeatedly performs enqueue then dequeue.\n\n";
        for (int threads : counts) {
            double ms = 0;
            gcq_queue* q = nullptr;
            const Stats s = run_point(kind, 0, 50, threads, &ms, &q);
            print_result_line("balanced", threads, ms, s);
            if (MODE_FIFO) {
                gcq_fifo_result fr;
                harness::check(gcq_fifo_check(q, (uint32_t)threads, FIFO_BLOCK_SIZE, FIFO_OPS_PER_THREAD, &fr),
                               "gcq_fifo_check");
                print_fifo(fr);
            }
            append_csv(csv, gpu, qname, "balanced", -1, threads, ms, s);
            gcq_destroy(q);
        }
        std::cout << "\n";
    }
    if (!ONLY_BALANCED) {
        std::cout << "=== Split Producer/Consumer Timed Benchmark ===\n";
        std::cout << "Producer percentage sweeps offered load by role population.\n";
        std::cout << "25% producers matches the classic 1P/3C imbalance pattern.\n\n";
        for (int p : producer_percents) {
            std::cout << "--- producer_percent=" << p << " (" << p << "% producers / " << (100 - p)
                      << "% consumers) ---\n";
            for (int threads : counts) {
                double ms = 0;
                gcq_queue* q = nullptr;
                const Stats s = run_point(kind, 1, p, threads, &ms, &q);
                print_result_line("split-" + std::to_string(p), threads, ms, s);
                if (MODE_FIFO) {
                    gcq_fifo_result fr;
                    harness::check(gcq_fifo_check(q, (uint32_t)threads, FIFO_BLOCK_SIZE, FIFO_OPS_PER_THREAD, &fr),
                                   "gcq_fifo_check");
                    print_fifo(fr);
                }
                append_csv(csv, gpu, qname, "split", p, threads, ms, s);
                gcq_destroy(q);
            }
            std::cout << "\n";
        }
    }
    csv.flush();
    std::cout << "Done.\n";
    return 0;
}
