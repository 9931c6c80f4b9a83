// rt_bench: the ray-tracing benchmark configuration over libgcq.so.  The reference's
// tracer (rt, concurrent_rt/rt_final.cpp) renders its own two scenes at 1280x720;
// this one renders the benchmark scenes with gcq_rt_bounce_render and reports in
// the same form.
//
//   rt_bench [scene] [max_bounces] [threads_per_tile] [seed]
// scene 0 = 512 random spheres over a ground quad, 1 = box room with a ceiling
// light; one sample per pixel; RT_IMG x RT_IMG pixels in RT_TILE x RT_TILE tiles,
// one ring of RT_QUEUE_N entries per tile.  Console lines as rt; the image is
// written to rtb_<queue>_<spheres|room>.ppm (P6, clamped to [0,255]) and a CSV row
// appended to rt_bench_perf.csv.
//
// Knobs (compile-time): RT_QUEUE_N, RT_IMG, RT_TILE.
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "harness_common.h"

#ifndef RT_QUEUE_N
#define RT_QUEUE_N 32768
#endif
#ifndef RT_IMG
#define RT_IMG 1024
#endif
#ifndef RT_TILE
#define RT_TILE 32
#endif

int main(int argc, char** argv) {
    const int scene = (argc > 1) ? std::atoi(argv[1]) : 0;
    const int max_bounces = (argc > 2) ? std::atoi(argv[2]) : 4;
    const int threads_per_tile = (argc > 3) ? std::atoi(argv[3]) : 1024;
    const unsigned long long seed = (argc > 4) ? std::strtoull(argv[4], nullptr, 10) : 1ull;
    const int kind = harness::queue_kind();
    const std::string gpu = harness::gpu_name();
    const uint32_t qlog2 = (uint32_t)__builtin_ctz((unsigned)RT_QUEUE_N);
    const int tiles_side = (RT_IMG + RT_TILE - 1) / RT_TILE;
    const std::string scene_str = scene == 0 ? "spheres" : "room";
    std::cout << "=== Ray-bounce queue raytracer, benchmark scenes (" << harness::queue_name(kind) << ") ===\n"
              << "GPU:              " << gpu << "\n"
              << "Scene:            " << scene << " (" << (scene == 0 ? "512 random spheres" : "Box room") << ")\n"
              << "Image:            " << RT_IMG << "x" << RT_IMG << ", 1 sample per pixel, seed " << seed << "\n"
              << "Max bounces:      " << max_bounces << "\n"
              << "Threads/tile:     " << threads_per_tile << "\n"
              << "Tiles:            " << tiles_side << "x" << tiles_side << " = " << tiles_side * tiles_side
              << " of " << RT_TILE << "x" << RT_TILE << " px\n"
              << "Queue capacity:   " << RT_QUEUE_N << "\n\n";

    std::vector<float> img((size_t)RT_IMG * RT_IMG * 3);
    gcq_rt_result r;
    const int rc = gcq_rt_bounce_render(kind, scene, RT_IMG, RT_IMG, RT_TILE, threads_per_tile, max_bounces, qlog2,
                                        seed, img.data(), &r);
    if (rc == GCQ_ECAPACITY || rc == GCQ_EINVAL || rc == GCQ_EUNSUPPORTED) {
        std::fprintf(stderr, "ERROR: %s (scene %d, threads/tile %d, tile pixels %d, queue %d)\n", gcq_strerror(rc),
                     scene, threads_per_tile, RT_TILE * RT_TILE, RT_QUEUE_N);
        return 1;
    }
    harness::check(rc, "gcq_rt_bounce_render");
    const double total_ms = r.gen_ms + r.trace_ms;
    const double mrays_total = total_ms > 0 ? ((double)r.total_rays / 1e6) / (total_ms / 1e3) : 0.0;
    const double mrays_trace = r.trace_ms > 0 ? ((double)r.total_rays / 1e6) / (r.trace_ms / 1e3) : 0.0;
    std::cout << "=== RESULTS ===\n"
              << "Primary rays:       " << r.primary_rays << "\n"
              << "Total rays traced:  " << r.total_rays << "\n"
              << "Secondary rays:     " << (r.total_rays - r.primary_rays) << "\n"
              << "Generate time:      " << r.gen_ms << " ms\n"
              << "Trace time:         " << r.trace_ms << " ms\n"
              << "Total time:         " << total_ms << " ms\n"
              << "Throughput (total): " << mrays_total << " MRays/s\n"
              << "Throughput (trace): " << mrays_trace << " MRays/s\n"
              << "Kernel launches:    2\n";

    const std::string filename = std::string("rtb_") + harness::queue_tag(kind) + "_" + scene_str + ".ppm";
    if (FILE* f = std::fopen(filename.c_str(), "wb")) {
        std::fprintf(f, "P6\n%d %d\n255\n", RT_IMG, RT_IMG);
        std::vector<unsigned char> row((size_t)RT_IMG * 3);
        for (int y = 0; y < RT_IMG; ++y) {
            for (int i = 0; i < RT_IMG * 3; ++i)
                row[i] = (unsigned char)std::fmin(255.f, std::fmax(0.f, img[(size_t)y * RT_IMG * 3 + i] * 255.f));
            std::fwrite(row.data(), 1, row.size(), f);
        }
        std::fclose(f);
        std::cout << "Image saved: " << filename << "\n";
    }
    const char* csv = "rt_bench_perf.csv";
    const bool exists = std::ifstream(csv).good();
    std::ofstream ofs(csv, std::ios::app);
    if (ofs) {
        if (!exists) ofs << "GPU,QUEUE,SCENE,THREADS,BOUNCES,PRIMARY,TOTAL,GEN_MS,TRACE_MS,TOTAL_MS,MRAYS\n";
        static const char* csv_names[] = {"GWFQ", "GLFQ", "WFQ", "SFQ"};
        ofs << "\"" << gpu << "\"," << csv_names[kind] << "," << scene_str << "," << threads_per_tile << ","
            << max_bounces << "," << r.primary_rays << "," << r.total_rays << "," << r.gen_ms << "," << r.trace_ms
            << "," << total_ms << "," << mrays_trace << "\n";
    }
    return 0;
}
