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
