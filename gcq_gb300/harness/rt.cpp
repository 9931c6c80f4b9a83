// rt: the persistent wavefront ray tracer (concurrent_rt/rt_final.cpp), over libgcq.so.
//
// Command line as the reference (rt_final.cpp:713-715):
//   rt [scene] [max_bounces] [threads_per_tile]
// scene 0 = complex spheres, 1 = Cornell box; 1280x720 image in 8x8 tiles
// (rt_final.cpp:313-320), one ring of RT_QUEUE_N entries per tile.  Console lines,
// the image file rt_<queue>_<complex|cornell>.ppm (P6, clamped to [0,255]) and the
// CSV row of rt_queue_perf.csv follow rt_final.cpp:743-1000; the CSV row carries
// all eleven columns its header names (the reference writes eight of them).
//
// Knobs (compile-time): RT_QUEUE_N, RT_IMG_W, RT_IMG_H, RT_TILES_X, RT_TILES_Y.
#include <cmath>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "harness_common.h"

#ifndef RT_QUEUE_N
#define RT_QUEUE_N 32768
#endif
#ifndef RT_IMG_W
#define RT_IMG_W 1280
#endif
#ifndef RT_IMG_H
#define RT_IMG_H 720
#endif
#ifndef RT_TILES_X
#define RT_TILES_X 8
#endif
#ifndef RT_TILES_Y
#define RT_TILES_Y 8
#endif

int main(int argc, char** argv) {
    const int scene = (argc > 1) ? std::atoi(argv[1]) : 0;
    const int max_bounces = (argc > 2) ? std::atoi(argv[2]) : 4;
    const int threads_per_tile = (argc > 3) ? std::atoi(argv[3]) : 1024;
    const int kind = harness::queue_kind();
    const std::string gpu = harness::gpu_name();
    const uint32_t qlog2 = (uint32_t)__builtin_ctz((unsigned)RT_QUEUE_N);
    const int tpb = 256;
    std::cout << "=== Persistent Wavefront Raytracer (" << harness::queue_name(kind) << ") ===\n"
              << "GPU:              " << gpu << "\n"
              << "Scene:            " << scene << " (" << (scene == 0 ? "Complex Spheres" : "Cornell Box") << ")\n"
              << "Max bounces:      " << max_bounces << "\n"
              << "Threads/tile:     " << threads_per_tile << "\n"
              << "Tiles:            " << RT_TILES_X << "x" << RT_TILES_Y << " = " << RT_TILES_X * RT_TILES_Y << "\n"
              << "Blocks/tile:      " << (threads_per_tile + tpb - 1) / tpb << "\n"
              << "Queue capacity:   " << RT_QUEUE_N << "\n\n";

    std::vector<float> img((size_t)RT_IMG_W * RT_IMG_H * 3);
    gcq_rt_result r;
    const int rc = gcq_rt_render(kind, scene, RT_IMG_W, RT_IMG_H, RT_TILES_X, RT_TILES_Y, threads_per_tile,
                                 max_bounces, qlog2, img.data(), &r);
    if (rc == GCQ_ECAPACITY || rc == GCQ_EINVAL || rc == GCQ_EUNSUPPORTED) {
        std::fprintf(stderr, "ERROR: %s (threads/tile %d, tile pixels %d, queue %d)\n", gcq_strerror(rc),
                     threads_per_tile,
                     ((RT_IMG_W + RT_TILES_X - 1) / RT_TILES_X) * ((RT_IMG_H + RT_TILES_Y - 1) / RT_TILES_Y),
                     RT_QUEUE_N);
        return 1;
    }
    harness::check(rc, "gcq_rt_render");
    std::cout << "Generating primary rays...\n";
    std::cout << "  " << r.primary_rays << " primary rays in " << r.gen_ms << " ms\n";
    std::cout << "Persistent trace (max " << max_bounces << " bounces)...\n";
    const double total_ms = r.gen_ms + r.trace_ms;
    const double mrays_total = total_ms > 0 ? ((double)r.total_rays / 1e6) / (total_ms / 1e3) : 0.0;
    const double mrays_trace = r.trace_ms > 0 ? ((double)r.total_rays / 1e6) / (r.trace_ms / 1e3) : 0.0;
    std::cout << "\n=== RESULTS ===\n"
              << "Primary rays:       " << r.primary_rays << "\n"
              << "Total rays traced:  " << r.total_rays << "\n"
              << "Secondary rays:     " << (r.total_rays - r.primary_rays) << "\n"
              << "Generate time:      " << r.gen_ms << " ms\n"
              << "Trace time:         " << r.trace_ms << " ms\n"
              << "Total time:         " << total_ms << " ms\n"
              << "Throughput (total): " << mrays_total << " MRays/s\n"
              << "Throughput (trace): " << mrays_trace << " MRays/s\n"
              << "Kernel launches:    2\n";
    if (r.leftover != 0) std::cerr << "WARNING: " << r.leftover << " rays still alive after trace!\n";

    const std::string scene_str = scene == 0 ? "complex" : "cornell";
    const std::string filename = std::string("rt_") + harness::queue_tag(kind) + "_" + scene_str + ".ppm";
    if (FILE* f = std::fopen(filename.c_str(), "wb")) {
        std::fprintf(f, "P6\n%d %d\n255\n", RT_IMG_W, RT_IMG_H);
        std::vector<unsigned char> row((size_t)RT_IMG_W * 3);
        for (int y = 0; y < RT_IMG_H; ++y) {
            for (int i = 0; i < RT_IMG_W * 3; ++i)
                row[i] = (unsigned char)std::fmin(255.f, std::fmax(0.f, img[(size_t)y * RT_IMG_W * 3 + i] * 255.f));
            std::fwrite(row.data(), 1, row.size(), f);
        }
        std::fclose(f);
        std::cout << "Image saved: " << filename << "\n";
    }
    const char* csv = "rt_queue_perf.csv";
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
