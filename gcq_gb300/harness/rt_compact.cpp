// rt_compact: the double-buffer + stream-compaction ray tracer
// (concurrent_rt/baselines/rt_compaction.cpp), over libgcq.so.
//
// Command line as the reference (:593-601):  rt_compact [scene] [max_bounces]
// scene 0 = complex spheres, 1 = Cornell box, 2 = mirror tunnel; 1280x720.
// Console lines, the image rt_COMPACT_<complex|cornell|mirror_tunnel>.ppm and the CSV
// row of rt_performance.csv (DEVICE,QUEUE,THREADS,TOTAL_RAYS,TOTAL_TIME_MS,TOTAL_MRAYS)
// follow :845-897.  THREADS is the block size, as the reference writes it.
#include <cmath>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "harness_common.h"

int main(int argc, char** argv) {
    const int scene = (argc > 1) ? std::atoi(argv[1]) : 0;
    const int max_bounces = (argc > 2) ? std::atoi(argv[2]) : 4;
    const int W = 1280, H = 720;
    const std::string gpu = harness::gpu_name();
    std::cout << "Wavefront Raytracer (Double-Buffer + Stream Compaction) on " << gpu << "\n";
    std::cout << "Scene " << scene << " ("
              << (scene == 0 ? "Complex Spheres" : scene == 1 ? "Cornell Box" : "Mirror Tunnel") << ")\n";
    std::cout << "Max bounces: " << max_bounces << "\n";
    std::cout << "Resolution: " << W << "x" << H << " = " << W * H << " pixels\n";
    std::vector<float> img((size_t)W * H * 3);
    gcq_rt_result r;
    harness::check(gcq_rt_compact_render(scene, W, H, max_bounces, img.data(), &r), "gcq_rt_compact_render");
    const double mrays = (r.total_rays / 1.0e6) / (r.total_ms / 1.0e3);
    std::cout << "\n========================================\n";
    std::cout << "RESULTS (Double-Buffer + Stream Compaction)\n";
    std::cout << "========================================\n";
    std::cout << "Total rays traced: " << r.total_rays << "\n";
    std::cout << "Total time: " << r.total_ms << " ms\n";
    std::cout << "Throughput: " << mrays << " MRays/s\n";
    {
        const char* csv = "rt_performance.csv";
        const bool exists = std::ifstream(csv).good();
        std::ofstream ofs(csv, std::ios::app);
        if (ofs) {
            if (!exists) ofs << "DEVICE,QUEUE,THREADS,TOTAL_RAYS,TOTAL_TIME_MS,TOTAL_MRAYS\n";
            const std::string dev = gpu.substr(gpu.find_last_of(' ') + 1);
            ofs << dev << ",COMPACT,256," << r.total_rays << "," << r.total_ms << "," << mrays << "\n";
        }
    }
    const std::string scene_str = scene == 0 ? "complex" : scene == 1 ? "cornell" : "mirror_tunnel";
    const std::string filename = "rt_COMPACT_" + scene_str + ".ppm";
    if (FILE* f = std::fopen(filename.c_str(), "wb")) {
        std::fprintf(f, "P6\n%d %d\n255\n", W, H);
        std::vector<unsigned char> row((size_t)W * 3);
        for (int y = 0; y < H; ++y) {
            for (int i = 0; i < W * 3; ++i)
                row[i] = (unsigned char)std::fmin(255.f, std::fmax(0.f, img[(size_t)y * W * 3 + i] * 255.f));
            std::fwrite(row.data(), 1, row.size(), f);
        }
        std::fclose(f);
        std::cout << "\nImage saved: " << filename << "\n";
    }
    return 0;
}
