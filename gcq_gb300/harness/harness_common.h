// Shared pieces of the harness executables (tb, history, bfs, rt): queue selection,
// GPU name, status checks.  The executables are host C++ over the C ABI of gcq.h;
// they reproduce the reference harnesses' command lines, compile-time knobs and
// output lines.
//
// Queue selection follows the reference Makefile (Makefile:66-80): -DUSE_GWFQ,
// -DUSE_GLFQ, -DUSE_WFQ or -DUSE_SFQ at compile time.  A build without one of them
// reads the QUEUE environment variable (gwfq, glfq, wfq, sfq; default gwfq).
#pragma once

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "gcq.h"

namespace harness {

inline int queue_kind() {
#if defined(USE_GWFQ)
    return GCQ_GWFQ;
#elif defined(USE_GLFQ)
    return GCQ_GLFQ;
#elif defined(USE_WFQ)
    return GCQ_WFQ;
#elif defined(USE_SFQ)
    return GCQ_SFQ;
#else
    const char* q = std::getenv("QUEUE");
    const std::string s = (q && *q) ? q : "gwfq";
    if (s == "gwfq") return GCQ_GWFQ;
    if (s == "glfq") return GCQ_GLFQ;
    if (s == "wfq") return GCQ_WFQ;
    if (s == "sfq") return GCQ_SFQ;
    std::fprintf(stderr, "Unsupported QUEUE='%s'. Use one of: gwfq glfq wfq sfq\n", s.c_str());
    std::exit(2);
#endif
}

// Lower-case tag used in file names (rt_gwfq_complex.ppm, ...).
inline const char* queue_tag(int kind) {
    static const char* tags[] = {"gwfq", "glfq", "wfq", "sfq"};
    return tags[kind];
}

// Display names printed by the reference harnesses (throughout_bench.cpp:128,
// rt_final.cpp:60,108).
inline const char* queue_name(int kind) {
    static const char* names[] = {"gWFQ", "gLFQ", "WFQ", "SFQ"};
    return names[kind];
}

// Queue capacity (log2) each reference harness uses: GWF_N = 65536 (gwf_64k),
// FQ_N = 32768, SFQ_QUEUE_LENGTH = 65536 (throughout_bench.cpp:118-120,
// glf_queue.hpp:32-34, sfqueue_hip.hpp:13-15); YMC's pool is sized per thread.
inline uint32_t default_capacity_log2(int kind) {
#ifdef GWF_N
    if (kind == GCQ_GWFQ) return (uint32_t)__builtin_ctz((unsigned)GWF_N);
#endif
#ifdef FQ_N
    if (kind == GCQ_GLFQ) return (uint32_t)__builtin_ctz((unsigned)FQ_N);
#endif
#ifdef SFQ_QUEUE_LENGTH
    if (kind == GCQ_SFQ) return (uint32_t)__builtin_ctz((unsigned)SFQ_QUEUE_LENGTH);
#endif
    return kind == GCQ_GLFQ ? 15u : 16u;
}

inline std::string gpu_name() {
    const char* env = std::getenv("GPU_NAME");
    if (env && *env) return env;
    char name[256] = {0};
    int sms = 0;
    if (gcq_device_info(name, sizeof name, &sms) != GCQ_OK) return "unknown";
    return name;
}

inline int gpu_sms() {
    int sms = 0;
    gcq_device_info(nullptr, 0, &sms);
    return sms;
}

// The reference exits on any HIP error (HIP_CHECK, throughout_bench.cpp:79-86);
// these exit on any gcq error, with its text.
inline void check(int rc, const char* what) {
    if (rc != GCQ_OK) {
        std::fprintf(stderr, "%s failed: %s", what, gcq_strerror(rc));
        if (rc == GCQ_ECUDA) std::fprintf(stderr, " (%s)", gcq_last_cuda_error());
        std::fprintf(stderr, "\n");
        std::exit(1);
    }
}

inline std::string csv_escape(const std::string& s) {
    if (s.find_first_of(",\"\n") == std::string::npos) return s;
    std::string o = "\"";
    for (char c : s) {
        if (c == '"') o += '"';
        o += c;
    }
    return o + "\"";
}

}  // namespace harness
