// Internal definitions shared by the libgcq.so translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>

#include "gcq.h"
#include "gcq/gcq_atomics.cuh"
#include "gcq/gwf_ring.cuh"
#include "gcq/glf_queue.cuh"
#include "gcq/sfqueue.cuh"
#include "gcq/wfqueue.cuh"

// Host-side handle behind gcq_queue*.
struct gcq_queue {
    int kind;
    uint32_t order;          // log2 capacity (SFQ: log2 length)
    uint32_t max_threads;
    gcq_knobs knobs;
    void* base;              // the single device allocation
    uint64_t bytes;
    void* obj;               // device address of the queue object
    gcq::u32a* err;          // device address of the error word
    uint64_t ymc_cells;      // YMC pool size in cells
    gcq::u64a* stats;        // G-WFQ operation counters (2 rings x 8), device address
};

namespace gcqi {

// Record the failing CUDA call for gcq_last_cuda_error and map it to GCQ_ECUDA.
int cuda_fail(cudaError_t e, const char* what, const char* file, int line);

#define GCQ_CUDA(call)                                                       \
    do {                                                                     \
        cudaError_t _e = (call);                                             \
        if (_e != cudaSuccess) return gcqi::cuda_fail(_e, #call, __FILE__, __LINE__); \
    } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Thread counts the device can keep resident at once for `kernel` with `block`.
int resident_threads(const void* kernel, int block, size_t smem, uint64_t* out);

// Grid size for a grid-stride kernel over `n` items.
inline unsigned grid_for(uint64_t n, unsigned block, unsigned cap = 152u * 16u) {
    uint64_t g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > cap) g = cap;
    return (unsigned)g;
}

__host__ __device__ inline uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}

// Per-kind adapters used by the harness kernels: the backend shims of
// throughout_bench.cpp:112-292 and history.cpp:44-144.
//   enq: true on success (false = full, or a failed non-blocking attempt)
//   deq: 1 value, 0 empty, 2 failed without effect (SFQ BUSY / timeout)
template <int K> struct qops;

template <> struct qops<GCQ_GWFQ> {
    using Q = gcq::gwf::mpmc;
    __device__ static bool enq(Q* q, uint64_t v, uint32_t tid, bool /*nonblocking*/) {
        return gcq::gwf::enqueue_ptr(q, v, tid);
    }
    __device__ static int deq(Q* q, uint64_t* out, uint32_t tid, bool /*nonblocking*/) {
        return gcq::gwf::dequeue_ptr(q, out, tid) ? 1 : 0;
    }
    __device__ static uint64_t tb_value(uint32_t p) { return p; }
};

template <> struct qops<GCQ_GLFQ> {
    using Q = gcq::glf::mpmc;
    __device__ static bool enq(Q* q, uint64_t v, uint32_t, bool) { return gcq::glf::enqueue_ptr(q, v); }
    __device__ static int deq(Q* q, uint64_t* out, uint32_t, bool) { return gcq::glf::dequeue_ptr(q, out) ? 1 : 0; }
    __device__ static uint64_t tb_value(uint32_t p) { return p; }
};

template <> struct qops<GCQ_WFQ> {
    using Q = gcq::ymc::queue;
    __device__ static bool enq(Q* q, uint64_t v, uint32_t tid, bool) { return gcq::ymc::enqueue(q, tid, v); }
    __device__ static int deq(Q* q, uint64_t* out, uint32_t tid, bool) {
        const uint64_t v = gcq::ymc::dequeue(q, tid);
        if (v == gcq::ymc::EMPTY) return 0;
        *out = v;
        return 1;
    }
    // YMC reserves 0 (empty), ~0 and ~0-1: shift the payload into [1, 2^32].
    __device__ static uint64_t tb_value(uint32_t p) { return (uint64_t)p + 1; }
};

template <> struct qops<GCQ_SFQ> {
    using Q = gcq::sfq::queue;
    // sfq_pack_value, throughout_bench.cpp:246-249: fold to 32 bits, 0 -> 1
    __device__ static uint32_t pack(uint64_t v) {
        const uint32_t x = (uint32_t)(v ^ (v >> 32));
        return x == 0 ? 1u : x;
    }
    __device__ static bool enq(Q* q, uint64_t v, uint32_t, bool nonblocking) {
        const uint32_t x = pack(v);
        return (nonblocking ? gcq::sfq::enqueue_nb(q, x) : gcq::sfq::enqueue_blocking(q, x)) == SFQ_SUCCESS;
    }
    __device__ static int deq(Q* q, uint64_t* out, uint32_t, bool nonblocking) {
        uint32_t item = 0;
        const int rc = nonblocking ? gcq::sfq::dequeue_nb(q, &item) : gcq::sfq::dequeue_blocking(q, &item);
        if (rc == SFQ_SUCCESS) { *out = item; return 1; }
        return 2;
    }
    __device__ static uint64_t tb_value(uint32_t p) { return p; }
};

}  // namespace gcqi
