// Serial BFS over a CSR graph: test infrastructure (the oracle for BFS depths).
//
// The reference prints only "Reached: r/V Levels: L" (concurrent_bfs/bfs_bench.cpp:
// 779-780) and has no depth check; its CSR is built by csr_from_edges
// (bfs_bench.cpp:186-200).  Depths from the GPU traversal must equal these bit for
// bit: level[v] = hop distance from src, -1 where unreachable.
#include <cstdint>
#include <vector>

extern "C" int32_t oracle_bfs(int32_t V, const int32_t* offsets, const int32_t* indices, int32_t src,
                              int32_t* level) {
    if (V <= 0 || src < 0 || src >= V) return -1;
    for (int32_t v = 0; v < V; ++v) level[v] = -1;
    std::vector<int32_t> q;
    q.reserve((size_t)V);
    level[src] = 0;
    q.push_back(src);
    size_t head = 0;
    int32_t maxl = 0;
    while (head < q.size()) {
        const int32_t u = q[head++];
        const int32_t lu = level[u];
        for (int32_t e = offsets[u]; e < offsets[u + 1]; ++e) {
            const int32_t w = indices[e];
            if (level[w] < 0) {
                level[w] = lu + 1;
                if (lu + 1 > maxl) maxl = lu + 1;
                q.push_back(w);
            }
        }
    }
    return maxl;   // eccentricity of src within its component
}

// Checksum of a level array as the served traversals report it: the sum (mod 2^64)
// over v of splitmix64(v << 32 | level), level 0xFFFFFFFF where unreached (-1).
// splitmix64 is Steele, Lea and Flood's SplitMix64 finaliser (OOPSLA 2014).
static uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}

extern "C" uint64_t oracle_levels_checksum(int32_t V, const int32_t* level) {
    uint64_t s = 0;
    for (int32_t v = 0; v < V; ++v) {
        const uint32_t l = level[v] < 0 ? 0xFFFFFFFFu : (uint32_t)level[v];
        s += splitmix64(((uint64_t)(uint32_t)v << 32) | l);
    }
    return s;
}
