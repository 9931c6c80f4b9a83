// Atomic roofline microbenchmark: the denominators the queue throughput is
// reported against, measured on the same GPU in the same process.
//   R1   single-address 64-bit atomicAdd, every thread on one word
//   R1w  single-address, warp-aggregated (one atomic per warp, 32 tickets)
//   Rs   spread 64-bit fetch-add, each lane on its own 128-byte line, L2-resident
//   Rsc  spread 64-bit fetch-add, a warp on 32 consecutive words (the layout of
//        consecutive ring tickets with identity slots)
//   Rc   spread 64-bit CAS, each lane on its own line
//   Rc128 spread 128-bit CAS (atom.cas.b128, sm_90+), each lane on its own line
//   HBM  device-to-device copy bandwidth (read + write bytes)
// All RMWs are acq_rel at gpu scope, the ordering the queues use.
#include <algorithm>
#include <cstring>

#include "gcq_internal.cuh"

namespace {

__global__ void k_single(gcq::u64a* p, uint32_t iters) {
    for (uint32_t i = 0; i < iters; ++i) gcq::fetch_add(p, 1ull);
}
__global__ void k_single_warp(gcq::u64a* p, uint32_t iters) {
    for (uint32_t i = 0; i < iters; ++i) gcq::warp_fetch_add(p, 1ull);
}
// each thread owns one 128-byte line of a buffer of `lines` lines
__global__ void k_spread(gcq::u64a* buf, uint64_t lines, uint32_t iters) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    gcq::u64a* p = buf + (gid % lines) * 16;
    for (uint32_t i = 0; i < iters; ++i) gcq::fetch_add(p, 1ull);
}
// a warp's lanes hit consecutive 8-byte words; warps spread over the buffer
__global__ void k_spread_contig(gcq::u64a* buf, uint64_t words, uint32_t iters) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    gcq::u64a* p = buf + (gid % words);
    for (uint32_t i = 0; i < iters; ++i) gcq::fetch_add(p, 1ull);
}
__global__ void k_spread_cas(gcq::u64a* buf, uint64_t lines, uint32_t iters, gcq::u64a* sink) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    gcq::u64a* p = buf + (gid % lines) * 16;
    uint64_t v = 0, acc = 0;
    for (uint32_t i = 0; i < iters; ++i) {
        const uint64_t old = gcq::cas(p, v, v + 1);
        acc += (old == v);
        v = (old == v) ? v + 1 : old;
    }
    if (acc == 0xFFFFFFFFFFFFFFFFull) *sink = acc;
}
__global__ void k_spread_cas128(gcq::u64a* buf, uint64_t lines, uint32_t iters, gcq::u64a* sink) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    gcq::u64a* p = buf + (gid % lines) * 16;   // 16-byte aligned (128-byte lines)
    uint64_t lo = 0, hi = 0, acc = 0;
    for (uint32_t i = 0; i < iters; ++i) {
        uint64_t olo, ohi;
        asm volatile(
            "{\n\t.reg .b128 cmp, val, old;\n\t"
            "mov.b128 cmp, {%2, %3};\n\t"
            "mov.b128 val, {%4, %5};\n\t"
            "atom.acq_rel.gpu.global.cas.b128 old, [%6], cmp, val;\n\t"
            "mov.b128 {%0, %1}, old;\n\t}"
            : "=l"(olo), "=l"(ohi)
            : "l"(lo), "l"(hi), "l"(lo + 1), "l"(hi), "l"(p)
            : "memory");
        const bool ok = (olo == lo && ohi == hi);
        acc += ok;
        lo = ok ? lo + 1 : olo;
        hi = ok ? hi : ohi;
    }
    if (acc == 0xFFFFFFFFFFFFFFFFull) *sink = acc;
}
__global__ void k_copy(const uint4* __restrict__ a, uint4* __restrict__ b, uint64_t n) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        b[i] = a[i];
}

// Unfused fp32 multiply and add (the ray tracer is built without contraction):
// eight independent chains per thread, each step one rounded multiply and one
// rounded add, so the count is 2 operations per step per chain.
__global__ void k_fp32(float a, float b, uint32_t iters, float* sink) {
    float x[8];
    for (int k = 0; k < 8; ++k) x[k] = (float)(threadIdx.x + k);
    for (uint32_t i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) x[k] = __fadd_rn(__fmul_rn(x[k], a), b);
    }
    float s = 0.f;
    for (int k = 0; k < 8; ++k) s += x[k];
    if (s == 1234.5f) *sink = s;   // keeps the chains live
}

struct timer {
    cudaEvent_t a, b;
    timer() { cudaEventCreate(&a); cudaEventCreate(&b); }
    ~timer() { cudaEventDestroy(a); cudaEventDestroy(b); }
    void start() { cudaEventRecord(a); }
    double stop_ms() {
        cudaEventRecord(b);
        cudaEventSynchronize(b);
        float ms = 0;
        cudaEventElapsedTime(&ms, a, b);
        return ms;
    }
};

}  // namespace

extern "C" {

int gcq_roofline_measure(gcq_roofline* out, int reps) {
    if (!out) return GCQ_EINVAL;
    if (reps < 1) reps = 1;
    memset(out, 0, sizeof(*out));
    int dev = 0, sms = 0;
    GCQ_CUDA(cudaGetDevice(&dev));
    GCQ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    out->sms = sms;
    const unsigned block = 256, grid = (unsigned)sms * 8;
    const uint64_t threads = (uint64_t)grid * block;
    // 32 MB atomic buffer: L2-resident (129 MB L2), one 128-B line per thread
    const uint64_t lines = threads;
    gcq::u64a* buf = nullptr;
    GCQ_CUDA(cudaMalloc(&buf, lines * 128 + 256));
    GCQ_CUDA(cudaMemset(buf, 0, lines * 128 + 256));
    gcq::u64a* sink = buf + lines * 16;
    timer t;
    auto best = [&](auto launch, double ops) {
        double b = 0;
        launch();   // warm-up
        cudaDeviceSynchronize();
        for (int r = 0; r < reps; ++r) {
            t.start();
            launch();
            const double ms = t.stop_ms();
            if (ms > 0) b = std::max(b, ops / (ms * 1e-3));
        }
        return b;
    };
    const uint32_t it_single = 64, it_spread = 256;
    out->r1_single = best([&] { k_single<<<grid, block>>>(buf, it_single); }, (double)threads * it_single);
    out->r1_warp = best([&] { k_single_warp<<<grid, block>>>(buf, it_single); }, (double)threads * it_single);
    out->rs_lines = best([&] { k_spread<<<grid, block>>>(buf, lines, it_spread); }, (double)threads * it_spread);
    out->rs_contig = best([&] { k_spread_contig<<<grid, block>>>(buf, lines * 16, it_spread); },
                          (double)threads * it_spread);
    out->rc_lines = best([&] { k_spread_cas<<<grid, block>>>(buf, lines, it_spread, sink); },
                         (double)threads * it_spread);
    out->rc128_lines = best([&] { k_spread_cas128<<<grid, block>>>(buf, lines, it_spread, sink); },
                            (double)threads * it_spread);
    const uint32_t it_fp = 4096;
    out->fp32_gops = best([&] { k_fp32<<<grid, block>>>(0.999f, 1e-3f, it_fp, (float*)sink); },
                          (double)threads * it_fp * 16.0) / 1e9;
    GCQ_CUDA(cudaGetLastError());
    GCQ_CUDA(cudaFree(buf));
    // HBM: 2 GiB copy (well above L2)
    const uint64_t bytes = 2ull << 30;
    void *a = nullptr, *b = nullptr;
    GCQ_CUDA(cudaMalloc(&a, bytes));
    GCQ_CUDA(cudaMalloc(&b, bytes));
    GCQ_CUDA(cudaMemset(a, 1, bytes));
    const uint64_t n16 = bytes / 16;
    out->hbm_gbs = best([&] { k_copy<<<(unsigned)sms * 16, 512>>>((const uint4*)a, (uint4*)b, n16); },
                        2.0 * (double)bytes) / 1e9;
    GCQ_CUDA(cudaGetLastError());
    cudaFree(a);
    cudaFree(b);
    GCQ_CUDA(cudaDeviceSynchronize());
    return GCQ_OK;
}

}  // extern "C"
