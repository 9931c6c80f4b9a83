// bfs: the BFS harness (concurrent_bfs/bfs_bench.cpp), over libgcq.so.
//
// Command line as the reference (bfs_bench.cpp:656-676):
//   bfs --graph <file.mtx | SNAP edge list> | --grid R C
//       [--src S] [--threads T] [--block B] [--warmup W] [--iters N] [--verbose 0|1]
// plus graphs generated in place of the datasets, and the persistent traversal:
//   --grid R C --keep P --diag P --seed S   edges kept with probability P, diagonal
//                                           shortcuts with probability P (defaults 1, 0:
//                                           the reference's full grid)
//   --rmat SCALE [--ef F] [--seed S]        seeded R-MAT, a,b,c = 0.57, 0.19, 0.19
//   --persistent 1                          one cooperative launch per traversal
// Output lines and the CSV row (CSV_NAME, default bfs_bench_final2.csv) follow
// bfs_bench.cpp:681-795; TEPS = edges scanned / kernel time.
#include <algorithm>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

#include "harness_common.h"

namespace {

struct Stats { double med = 0, q1 = 0, q3 = 0, iqr = 0; };

// median and inter-quartile range with linear interpolation
Stats stats(std::vector<double> v) {
    Stats s;
    if (v.empty()) return s;
    std::sort(v.begin(), v.end());
    auto pct = [&](double p) {
        const double i = p * (double)(v.size() - 1);
        const size_t a = (size_t)i, b = std::min(a + 1, v.size() - 1);
        const double f = i - (double)a;
        return v[a] * (1 - f) + v[b] * f;
    };
    s.q1 = pct(0.25);
    s.med = pct(0.5);
    s.q3 = pct(0.75);
    s.iqr = s.q3 - s.q1;
    return s;
}

std::string base_name(const std::string& path) { return path.substr(path.find_last_of("/\\") + 1); }

}  // namespace

int main(int argc, char** argv) {
    std::string graph_path;
    int src = 0, threads = 8192, block = 256, warmup = 3, iters = 10, grid_r = 0, grid_c = 0, rmat = 0, ef = 16;
    int persistent = 0;
    double keep = 1.0, diag = 0.0;
    unsigned long long seed = 1;
    bool verbose = false;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&] { return (i + 1 < argc) ? argv[++i] : (char*)""; };
        if (a == "--graph") graph_path = next();
        else if (a == "--grid") { grid_r = std::atoi(next()); grid_c = std::atoi(next()); }
        else if (a == "--src") src = std::atoi(next());
        else if (a == "--threads") threads = std::atoi(next());
        else if (a == "--block") block = std::atoi(next());
        else if (a == "--warmup") warmup = std::atoi(next());
        else if (a == "--iters") iters = std::atoi(next());
        else if (a == "--verbose") verbose = std::atoi(next()) != 0;
        else if (a == "--keep") keep = std::atof(next());
        else if (a == "--diag") diag = std::atof(next());
        else if (a == "--seed") seed = std::strtoull(next(), nullptr, 10);
        else if (a == "--rmat") rmat = std::atoi(next());
        else if (a == "--ef") ef = std::atoi(next());
        else if (a == "--persistent") persistent = std::atoi(next());
        else { std::cout << "Unknown: " << a << "\n"; return 1; }
    }
    const int kind = harness::queue_kind();
    const std::string gpu = harness::gpu_name();
    std::cout << "GPU: " << gpu << "  CUs=" << harness::gpu_sms() << "\n";
    std::cout << "Queue: " << harness::queue_name(kind) << "\n";

    int32_t *off = nullptr, *idx = nullptr, V = 0;
    int64_t E = 0;
    std::string gname;
    if (grid_r > 0 && grid_c > 0) {
        harness::check(gcq_graph_grid((uint32_t)grid_r, (uint32_t)grid_c, keep, diag, seed, &off, &idx, &V, &E),
                       "gcq_graph_grid");
        std::cout << "Graph: grid " << grid_r << "x" << grid_c << "\n";
        gname = "grid" + std::to_string(grid_r) + "x" + std::to_string(grid_c);
    } else if (rmat > 0) {
        harness::check(gcq_graph_rmat((uint32_t)rmat, (uint32_t)ef, 0.57, 0.19, 0.19, seed, &off, &idx, &V, &E),
                       "gcq_graph_rmat");
        std::cout << "Graph: rmat scale " << rmat << " ef " << ef << "\n";
        gname = "rmat" + std::to_string(rmat);
    } else if (!graph_path.empty()) {
        const bool mtx = graph_path.size() >= 4 && graph_path.substr(graph_path.size() - 4) == ".mtx";
        const int rc = mtx ? gcq_graph_load_mtx(graph_path.c_str(), &off, &idx, &V, &E)
                           : gcq_graph_load_snap(graph_path.c_str(), &off, &idx, &V, &E);
        if (rc != GCQ_OK) { std::cerr << "Empty graph\n"; return 1; }
        std::cout << "Graph: " << graph_path << "\n";
        gname = base_name(graph_path);
    } else {
        std::cout << "Usage: --graph <path> | --grid R C | --rmat SCALE\n";
        return 1;
    }
    if (V <= 0) { std::cerr << "Empty graph\n"; return 1; }
    std::cout << "V=" << V << " E=" << E << " threads=" << threads << " block=" << block << "\n";

    gcq_bfs_ctx* ctx = nullptr;
    harness::check(gcq_bfs_create(kind, off, idx, V, E, (uint32_t)threads, 0, nullptr, &ctx), "gcq_bfs_create");
    std::vector<double> v_total, v_kernel, v_init, v_teps;
    uint32_t last_reached = 0;
    int last_levels = 0;
    for (int r = 0; r < warmup + iters; ++r) {
        gcq_bfs_result rr;
        harness::check(gcq_bfs_run(ctx, src, (uint32_t)block, persistent, nullptr, &rr), "gcq_bfs_run");
        if (r >= warmup) {
            v_total.push_back(rr.total_ms);
            v_kernel.push_back(rr.kernel_ms);
            v_init.push_back(rr.init_ms);
            const double ks = rr.kernel_ms / 1000.0;
            v_teps.push_back(ks > 0 ? (double)rr.edges_scanned / ks : 0);
        }
        last_reached = rr.reached;
        last_levels = rr.levels;
        if (verbose)
            std::cout << (r < warmup ? "[warm] " : "[run]  ") << "total=" << rr.total_ms << " ms"
                      << " kernel=" << rr.kernel_ms << " ms"
                      << " edges=" << rr.edges_scanned << " reached=" << rr.reached << " levels=" << rr.levels
                      << "\n";
    }
    gcq_bfs_destroy(ctx);

    const Stats st = stats(v_total), sk = stats(v_kernel), si = stats(v_init), se = stats(v_teps);
    std::cout << "\n== Summary (" << iters << " runs, " << warmup << " warmup) ==\n";
    std::cout << "Reached: " << last_reached << "/" << V << " Levels: " << last_levels << "\n";
    std::cout << std::fixed << std::setprecision(3);
    std::cout << "  total:  med=" << st.med << " ms  IQR=" << st.iqr << "\n";
    std::cout << "  kernel: med=" << sk.med << " ms  IQR=" << sk.iqr << "\n";
    std::cout << "  init:   med=" << si.med << " ms  IQR=" << si.iqr << "\n";
    std::cout << "  TEPS:   med=" << std::setprecision(4) << (se.med / 1e9) << " Gedges/s  IQR=" << (se.iqr / 1e9)
              << "\n";
    {
        const char* env = std::getenv("CSV_NAME");
        const char* csv = (env && *env) ? env : "bfs_bench_final2.csv";
        std::ofstream ofs(csv, std::ios::app);
        ofs << gpu << "," << harness::queue_name(kind) << "," << gname << "," << V << "," << E << "," << threads
            << "," << block << "," << st.med << "," << st.iqr << "," << (se.med / 1e9) << "," << (se.iqr / 1e9)
            << "\n";
    }
    gcq_free(off);
    gcq_free(idx);
    return 0;
}
