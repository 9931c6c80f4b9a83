// Graph file loaders for the BFS harness: MatrixMarket coordinate files and SNAP
// edge lists, read into the undirected CSR the reference builds
// (load_mtx / load_snap / csr_from_edges, bfs_bench.cpp:186-243):
//   * every edge (u, v) with u != v is stored in both directions;
//   * duplicates are removed and each adjacency list is sorted (the reference sorts
//     and uniques its edge list before building the CSR);
//   * MatrixMarket: 1-based indices, entries outside the declared size are dropped,
//     V = max(rows, cols);
//   * SNAP: '#' and '%' lines are comments, ids are shifted down by one when the
//     smallest id is 1, V = largest id + 1.
// Host code only.  The file is read in one piece and parsed in place; the CSR is
// built by counting, scattering and a per-vertex sort.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "gcq.h"

namespace {

bool read_file(const char* path, std::vector<char>* buf) {
    FILE* f = fopen(path, "rb");
    if (!f) return false;
    std::vector<char>& b = *buf;
    b.clear();
    char tmp[1 << 16];
    size_t n;
    while ((n = fread(tmp, 1, sizeof tmp, f)) > 0) b.insert(b.end(), tmp, tmp + n);
    fclose(f);
    b.push_back('\n');
    b.push_back('\0');
    return true;
}

// Signed decimal integer at *p (skips blanks, not newlines); false if none.
bool next_int(const char*& p, long long* out) {
    while (*p == ' ' || *p == '\t' || *p == '\r') ++p;
    bool neg = false;
    if (*p == '-' || *p == '+') neg = (*p++ == '-');
    if (*p < '0' || *p > '9') return false;
    long long v = 0;
    while (*p >= '0' && *p <= '9') {
        v = v * 10 + (*p - '0');
        if (v > (1ll << 40)) return false;
        ++p;
    }
    *out = neg ? -v : v;
    return true;
}

void skip_line(const char*& p) {
    while (*p && *p != '\n') ++p;
    if (*p == '\n') ++p;
}

template <typename F>
void parallel_for(uint64_t n, F&& body) {
    const unsigned nth = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (n < (1u << 16) || nth == 1) {
        for (uint64_t i = 0; i < n; ++i) body(i);
        return;
    }
    std::vector<std::thread> ts;
    for (unsigned t = 0; t < nth; ++t)
        ts.emplace_back([&, t]() { for (uint64_t i = n * t / nth; i < n * (t + 1) / nth; ++i) body(i); });
    for (auto& th : ts) th.join();
}

// Undirected, deduplicated, sorted CSR from the directed pairs (eu[i], ev[i]);
// self loops must already be gone.
int build_csr(uint64_t V, const std::vector<uint32_t>& eu, const std::vector<uint32_t>& ev, int32_t** offsets,
              int32_t** indices, int32_t* V_out, int64_t* E_out) {
    const uint64_t M = eu.size();
    std::vector<int64_t> start(V + 1, 0);
    for (uint64_t e = 0; e < M; ++e) {
        ++start[eu[e] + 1];
        ++start[ev[e] + 1];
    }
    for (uint64_t v = 0; v < V; ++v) start[v + 1] += start[v];
    std::vector<int32_t> adj((size_t)std::max<int64_t>(start[V], 1));
    std::vector<int64_t> cur(start.begin(), start.end() - 1);
    for (uint64_t e = 0; e < M; ++e) {
        adj[cur[eu[e]]++] = (int32_t)ev[e];
        adj[cur[ev[e]]++] = (int32_t)eu[e];
    }
    std::vector<int32_t> ndeg(V);
    parallel_for(V, [&](uint64_t v) {
        int32_t* b = adj.data() + start[v];
        int32_t* e = adj.data() + start[v + 1];
        std::sort(b, e);
        ndeg[v] = (int32_t)(std::unique(b, e) - b);
    });
    int32_t* off = (int32_t*)malloc((V + 1) * sizeof(int32_t));
    if (!off) return GCQ_ENOMEM;
    off[0] = 0;
    int64_t total = 0;
    for (uint64_t v = 0; v < V; ++v) {
        total += ndeg[v];
        if (total > INT32_MAX) { free(off); return GCQ_ECAPACITY; }
        off[v + 1] = (int32_t)total;
    }
    int32_t* idx = (int32_t*)malloc((size_t)std::max<int64_t>(total, 1) * sizeof(int32_t));
    if (!idx) { free(off); return GCQ_ENOMEM; }
    parallel_for(V, [&](uint64_t v) { std::copy(adj.data() + start[v], adj.data() + start[v] + ndeg[v], idx + off[v]); });
    *offsets = off;
    *indices = idx;
    *V_out = (int32_t)V;
    *E_out = total;
    return GCQ_OK;
}

}  // namespace

extern "C" {

int gcq_graph_load_mtx(const char* path, int32_t** offsets, int32_t** indices, int32_t* V, int64_t* E) {
    if (!path || !offsets || !indices || !V || !E) return GCQ_EINVAL;
    std::vector<char> buf;
    if (!read_file(path, &buf)) return GCQ_EINVAL;
    const char* p = buf.data();
    if (strncmp(p, "%%MatrixMarket", 14) != 0) return GCQ_EINVAL;
    skip_line(p);
    long long nr = 0, nc = 0, nz = 0;
    for (;;) {   // size line: first line that is neither empty nor a comment
        if (!*p) return GCQ_EINVAL;
        if (*p == '%' || *p == '\n' || *p == '\r') { skip_line(p); continue; }
        if (!next_int(p, &nr) || !next_int(p, &nc) || !next_int(p, &nz)) return GCQ_EINVAL;
        skip_line(p);
        break;
    }
    if (nr <= 0 || nc <= 0 || nz < 0 || std::max(nr, nc) >= INT32_MAX) return GCQ_EINVAL;
    std::vector<uint32_t> eu, ev;
    eu.reserve((size_t)nz);
    ev.reserve((size_t)nz);
    long long cnt = 0;
    while (cnt < nz && *p) {
        if (*p == '%' || *p == '\n' || *p == '\r') { skip_line(p); continue; }
        long long i = 0, j = 0;
        const bool ok = next_int(p, &i) && next_int(p, &j);
        skip_line(p);
        if (!ok) continue;
        ++cnt;
        --i;
        --j;
        if (i == j || i < 0 || j < 0 || i >= nr || j >= nc) continue;
        eu.push_back((uint32_t)i);
        ev.push_back((uint32_t)j);
    }
    return build_csr((uint64_t)std::max(nr, nc), eu, ev, offsets, indices, V, E);
}

int gcq_graph_load_snap(const char* path, int32_t** offsets, int32_t** indices, int32_t* V, int64_t* E) {
    if (!path || !offsets || !indices || !V || !E) return GCQ_EINVAL;
    std::vector<char> buf;
    if (!read_file(path, &buf)) return GCQ_EINVAL;
    const char* p = buf.data();
    std::vector<uint32_t> eu, ev;
    long long mn = (1ll << 60), mx = -1;
    while (*p) {
        if (*p == '#' || *p == '%' || *p == '\n' || *p == '\r') { skip_line(p); continue; }
        long long u = 0, v = 0;
        const bool ok = next_int(p, &u) && next_int(p, &v);
        skip_line(p);
        if (!ok || u == v) continue;
        if (u < 0 || v < 0 || u >= INT32_MAX || v >= INT32_MAX) return GCQ_EINVAL;
        mn = std::min(mn, std::min(u, v));
        mx = std::max(mx, std::max(u, v));
        eu.push_back((uint32_t)u);
        ev.push_back((uint32_t)v);
    }
    if (mx < 0) return GCQ_EINVAL;   // no edge
    if (mn == 1) {
        for (size_t e = 0; e < eu.size(); ++e) { --eu[e]; --ev[e]; }
        --mx;
    }
    return build_csr((uint64_t)mx + 1, eu, ev, offsets, indices, V, E);
}

}  // extern "C"
