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
// throughout_bench.cpp:112-292 and history.cpp:44-144.  maybe(q) is a read-only
// hint (the ticket counters say an entry may be there) for consumers that poll.
//   enq: true on success (false = full, or a failed non-blocking attempt)
//   deq: 1 value, 0 empty, 2 failed without effect (SFQ BUSY / timeout)
template <int K> struct qops;

// Per-thread context of a kernel thread that runs many operations on one queue
// (ctx_begin / ctx_end around its loop); only G-WFQ keeps one (gwf::thread_ctx).
struct no_ctx {};

// GCQ_TB_CTX: the throughput chunk keeps G-WFQ's per-thread context (help
// countdowns in registers, pre-checks skipped after the thread's own enqueue).
#ifndef GCQ_TB_CTX
#define GCQ_TB_CTX 1
#endif

template <> struct qops<GCQ_GWFQ> {
    using Q = gcq::gwf::mpmc;
    using ctx = gcq::gwf::thread_ctx;
    __device__ static bool enq(Q* q, uint64_t v, uint32_t tid, bool /*nonblocking*/) {
        return gcq::gwf::enqueue_ptr(q, v, tid);
    }
    __device__ static int deq(Q* q, uint64_t* out, uint32_t tid, bool /*nonblocking*/) {
        return gcq::gwf::dequeue_ptr(q, out, tid) ? 1 : 0;
    }
    __device__ static ctx ctx_begin(Q* q, uint32_t tid) { return gcq::gwf::ctx_load(gcq::gwf::view_of(q), tid); }
    __device__ static void ctx_end(Q* q, uint32_t tid, const ctx& x) { gcq::gwf::ctx_store(gcq::gwf::view_of(q), tid, x); }
    __device__ static bool enq(Q* q, uint64_t v, uint32_t tid, bool, ctx* x) {
        return gcq::gwf::enqueue_ptr(gcq::gwf::view_of(q), v, tid, x);
    }
    __device__ static int deq(Q* q, uint64_t* out, uint32_t tid, bool, ctx* x) {
        return gcq::gwf::dequeue_ptr(gcq::gwf::view_of(q), out, tid, x) ? 1 : 0;
    }
    __device__ static uint64_t tb_value(uint32_t p) { return p; }
    __device__ static bool maybe(Q* q) { return gcq::gwf::maybe_nonempty(&q->aq); }
};
// The other queues keep no per-thread context.
template <int K> struct qops_ctx {
    using ctx = no_ctx;
    __device__ static ctx ctx_begin(typename qops<K>::Q*, uint32_t) { return ctx(); }
    __device__ static void ctx_end(typename qops<K>::Q*, uint32_t, const ctx&) {}
    __device__ static bool enq(typename qops<K>::Q* q, uint64_t v, uint32_t tid, bool nb, ctx*) {
        return qops<K>::enq(q, v, tid, nb);
    }
    __device__ static int deq(typename qops<K>::Q* q, uint64_t* out, uint32_t tid, bool nb, ctx*) {
        return qops<K>::deq(q, out, tid, nb);
    }
};
template <> struct qops_ctx<GCQ_GWFQ> : qops<GCQ_GWFQ> {};

template <> struct qops<GCQ_GLFQ> {
    using Q = gcq::glf::mpmc;
    __device__ static bool enq(Q* q, uint64_t v, uint32_t, bool) { return gcq::glf::enqueue_ptr(q, v); }
    __device__ static int deq(Q* q, uint64_t* out, uint32_t, bool) { return gcq::glf::dequeue_ptr(q, out) ? 1 : 0; }
    __device__ static uint64_t tb_value(uint32_t p) { return p; }
    __device__ static bool maybe(Q* q) { return gcq::ld_rlx(&q->aq.Tail) > gcq::ld_rlx(&q->aq.Head); }
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
    __device__ static bool maybe(Q* q) { return gcq::ld_rlx(&q->T) > gcq::ld_rlx(&q->H); }
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
    __device__ static bool maybe(Q* q) { return (int32_t)(gcq::ld_rlx(&q->tail) - gcq::ld_rlx(&q->head)) > 0; }
};

}  // namespace gcqi
