// SFQ for sm_103a: the Scogland-Feng ticket queue of sfqueue_hip.hpp/.cpp.
//
// Kept from the reference: u32 head/tail tickets, the even/odd slot phase ids
// (GET_ID(t) = (t / L) * 2, MAX_ID wrap; sfqueue_hip.hpp:32-39), blocking and
// non-blocking enqueue/dequeue with SUCCESS/BUSY/CLOSED results
// (sfqueue_hip.cpp:55-128), close (:47-53) and the u64 wrapper that reserves 0
// (:134-144).
// Changed for GB300:
//   * a slot is one 64-bit word {id:32, item:32}; an enqueue publishes id and item
//     with a single release store, and a dequeue reads both with one acquire load
//     (the reference keeps items[] and ids[] apart and publishes with two stores);
//   * loads are acquire loads instead of atomicAdd(p, 0) (sfqueue_hip.cpp:13-15);
//   * the closed flag is read with a relaxed load, not an RMW, on every operation;
//   * blocking waits back off with __nanosleep and give up at the queue's deadline,
//     returning SFQ_TIMEDOUT and setting the error word, where the reference spins
//     without bound (sfqueue_hip.cpp:62-65, 79-82);
//   * the length is a runtime header field (power of two).
#pragma once

#include <limits.h>
#include <stdint.h>
#include "gcq_atomics.cuh"

#ifndef SFQ_QUEUE_LENGTH
#define SFQ_QUEUE_LENGTH 65536u
#endif
#define SFQ_EMPTY 0ull
#define SFQ_SUCCESS 0
#define SFQ_BUSY 1
#define SFQ_CLOSED 2
#define SFQ_TIMEDOUT 3

namespace gcq {
namespace sfq {

struct alignas(128) queue {
    u32a head;
    char _pad0[GCQ_HOT_STRIDE - 4];
    u32a tail;
    char _pad1[GCQ_HOT_STRIDE - 4];
    u32a closed;
    char _pad2[GCQ_HOT_STRIDE - 4];
    u64a* slot;            // L words {id << 32 | item}
    u32a* err;
    uint32_t log2_len;     // L = 1 << log2_len
    uint32_t max_id;       // 2 * (UINT32_MAX / L + 1)
    uint64_t timeout_ns;   // deadline of one blocking wait
    uint32_t nprocs;
    char _pad3[92];
};

struct cfg {
    u64a* slot;
    u32a* err;
    uint32_t log2_len, max_id;
    uint64_t timeout_ns;
    __host__ __device__ __forceinline__ uint32_t len() const { return 1u << log2_len; }
    __host__ __device__ __forceinline__ uint32_t target(uint32_t t) const { return t & (len() - 1); }
    __host__ __device__ __forceinline__ uint32_t get_id(uint32_t t) const { return (t >> log2_len) * 2u; }
    __host__ __device__ __forceinline__ uint32_t next_id(uint32_t id) const {
        const uint32_t n = id + 1u;
        return n == max_id ? 0u : n;
    }
};

__device__ __forceinline__ cfg load_cfg(const queue* q) {
    cfg c;
    c.slot = q->slot; c.err = q->err; c.log2_len = q->log2_len; c.max_id = q->max_id;
    c.timeout_ns = q->timeout_ns;
    return c;
}
__device__ __forceinline__ uint32_t slot_id(uint64_t w) { return (uint32_t)(w >> 32); }
__device__ __forceinline__ uint32_t slot_item(uint64_t w) { return (uint32_t)w; }
__device__ __forceinline__ uint64_t make_slot(uint32_t id, uint32_t item) { return ((uint64_t)id << 32) | item; }

__device__ __forceinline__ bool is_closed(const queue* q) { return ld_rlx(&q->closed) != 0u; }
__device__ __forceinline__ void close(queue* q) { st_rel(&q->closed, 1u); }

// sfq_init_kernel, sfqueue_hip.cpp:164-180, as a grid-stride slice.
__device__ inline void init_slice(queue* q, uint64_t gid, uint64_t nthreads) {
    const cfg c = load_cfg(q);
    for (uint64_t i = gid; i < c.len(); i += nthreads) c.slot[i] = 0;
    if (gid == 0) { q->head = 0; q->tail = 0; q->closed = 0; }
}

// Wait until slot `target` carries phase `id`; returns the slot word, or sets *rc.
__device__ __forceinline__ uint64_t wait_phase(queue* q, const cfg& c, uint32_t target, uint32_t id, int* rc) {
    backoff bo;
    uint64_t deadline = 0;
    for (uint32_t it = 0;; ++it) {
        const uint64_t w = ld_acq(&c.slot[target]);
        if (slot_id(w) == id) { *rc = SFQ_SUCCESS; return w; }
        if (is_closed(q)) { *rc = SFQ_CLOSED; return 0; }
        if ((it & 15) == 0) {
            const uint64_t now = globaltimer_ns();
            if (deadline == 0) deadline = now + c.timeout_ns;
            else if (now > deadline) {
                raise_error(c.err, ERR_TIMEOUT);
                *rc = SFQ_TIMEDOUT;
                return 0;
            }
        }
        bo.pause();
    }
}

// sfq_enqueue_blocking_u32, sfqueue_hip.cpp:55-70
__device__ inline int enqueue_blocking(queue* q, uint32_t item) {
    if (is_closed(q)) return SFQ_CLOSED;
    const cfg c = load_cfg(q);
    const uint32_t t = fetch_add(&q->tail, 1u);
    const uint32_t target = c.target(t), id = c.get_id(t);
    int rc;
    wait_phase(q, c, target, id, &rc);
    if (rc != SFQ_SUCCESS) return rc;
    st_rel(&c.slot[target], make_slot(c.next_id(id), item));
    return SFQ_SUCCESS;
}

// sfq_dequeue_blocking_u32, sfqueue_hip.cpp:72-87
__device__ inline int dequeue_blocking(queue* q, uint32_t* out) {
    if (is_closed(q)) return SFQ_CLOSED;
    const cfg c = load_cfg(q);
    const uint32_t t = fetch_add(&q->head, 1u);
    const uint32_t target = c.target(t), id = c.get_id(t) + 1u;
    int rc;
    const uint64_t w = wait_phase(q, c, target, id, &rc);
    if (rc != SFQ_SUCCESS) return rc;
    *out = slot_item(w);
    st_rel(&c.slot[target], make_slot(c.next_id(id), 0u));
    return SFQ_SUCCESS;
}

// sfq_enqueue_nb_u32, sfqueue_hip.cpp:89-107
__device__ inline int enqueue_nb(queue* q, uint32_t item) {
    if (is_closed(q)) return SFQ_CLOSED;
    const cfg c = load_cfg(q);
    const uint32_t t = ld_acq(&q->tail);
    const uint32_t target = c.target(t), id = c.get_id(t);
    if (slot_id(ld_acq(&c.slot[target])) != id) return SFQ_BUSY;
    if (cas(&q->tail, t, t + 1u) != t) return SFQ_BUSY;
    st_rel(&c.slot[target], make_slot(c.next_id(id), item));
    return SFQ_SUCCESS;
}

// sfq_dequeue_nb_u32, sfqueue_hip.cpp:109-128.  The item comes from the same word
// whose id matched: no other thread can change the slot before the holder of
// ticket t bumps it, and the CAS below makes this thread that holder.
__device__ inline int dequeue_nb(queue* q, uint32_t* out) {
    if (is_closed(q)) return SFQ_CLOSED;
    const cfg c = load_cfg(q);
    const uint32_t t = ld_acq(&q->head);
    const uint32_t target = c.target(t), id = c.get_id(t) + 1u;
    const uint64_t w = ld_acq(&c.slot[target]);
    if (slot_id(w) != id) return SFQ_BUSY;
    if (cas(&q->head, t, t + 1u) != t) return SFQ_BUSY;
    *out = slot_item(w);
    st_rel(&c.slot[target], make_slot(c.next_id(id), 0u));
    return SFQ_SUCCESS;
}

}  // namespace sfq
}  // namespace gcq

// -----------------------------------------------------------------------------
// Reference-named device and host API (sfqueue_hip.hpp:13-102, sfqueue_hip.cpp:130-180,
// 356-399).
//
// sfq_queue is self-contained, as in the reference: the library's queue header
// (head, tail and closed GCQ_HOT_STRIDE apart, then the parameters) followed by
// SFQ_QUEUE_LENGTH slot words, each the reference's ids[i] and items[i] in one
// 64-bit word.  head, tail, closed and nprocs keep the reference's names.
// -----------------------------------------------------------------------------
#ifndef SFQ_MAX_THREADS
#define SFQ_MAX_THREADS 65535u
#endif
#define SFQ_GET_ID(x) (((x) / SFQ_QUEUE_LENGTH) * 2u)
#define SFQ_MAX_ID (2u * ((UINT32_MAX / SFQ_QUEUE_LENGTH) + 1u))
static_assert((SFQ_QUEUE_LENGTH & (SFQ_QUEUE_LENGTH - 1u)) == 0, "SFQ_QUEUE_LENGTH must be a power of two.");
static_assert(SFQ_MAX_ID >= 2u * (SFQ_MAX_THREADS + 1u),
              "SFQ_MAX_ID invariant violated: reduce SFQ_MAX_THREADS or queue length.");
#ifndef SFQ_WAIT_TIMEOUT_NS
#define SFQ_WAIT_TIMEOUT_NS 2000000000ull   // deadline of one blocking wait
#endif

struct sfq_queue : gcq::sfq::queue {
    gcq::u64a slots[SFQ_QUEUE_LENGTH];
    gcq::u32a err_word;
};
struct sfq_handle { uint32_t thread_id; uint32_t dummy[15]; };

__device__ __forceinline__ int sfq_enqueue_blocking_u32(gcq::sfq::queue* q, uint32_t item) { return gcq::sfq::enqueue_blocking(q, item); }
__device__ __forceinline__ int sfq_dequeue_blocking_u32(gcq::sfq::queue* q, uint32_t* out) { return gcq::sfq::dequeue_blocking(q, out); }
__device__ __forceinline__ int sfq_enqueue_nb_u32(gcq::sfq::queue* q, uint32_t item) { return gcq::sfq::enqueue_nb(q, item); }
__device__ __forceinline__ int sfq_dequeue_nb_u32(gcq::sfq::queue* q, uint32_t* out) { return gcq::sfq::dequeue_nb(q, out); }
__device__ __forceinline__ void sfq_close(gcq::sfq::queue* q) { gcq::sfq::close(q); }
__device__ __forceinline__ int sfq_is_closed(const gcq::sfq::queue* q) { return gcq::sfq::is_closed(q) ? 1 : 0; }
// u64 wrapper: payload 0 is reserved for SFQ_EMPTY (sfqueue_hip.cpp:130-144)
__device__ __forceinline__ void sfq_enqueue(gcq::sfq::queue* q, sfq_handle*, uint64_t v) {
    uint32_t item = (uint32_t)v;
    if (item == 0u) item = 1u;
    (void)gcq::sfq::enqueue_blocking(q, item);
}
__device__ __forceinline__ uint64_t sfq_dequeue(gcq::sfq::queue* q, sfq_handle*) {
    uint32_t item = 0;
    return gcq::sfq::dequeue_blocking(q, &item) == SFQ_SUCCESS ? (uint64_t)item : SFQ_EMPTY;
}

// sfq_queue_init / sfq_handle_init, sfqueue_hip.cpp:150-162 (one thread; the slots
// are cleared by sfq_init_kernel).
__device__ inline void sfq_queue_init(sfq_queue* q, uint32_t nprocs) {
    q->head = 0u;
    q->tail = 0u;
    q->closed = 0u;
    q->slot = q->slots;
    q->err_word = 0u;
    q->err = &q->err_word;
    q->log2_len = 31 - __clz(SFQ_QUEUE_LENGTH);
    q->max_id = SFQ_MAX_ID;
    q->timeout_ns = SFQ_WAIT_TIMEOUT_NS;
    q->nprocs = nprocs;
}
__device__ inline void sfq_handle_init(sfq_handle* h, uint32_t tid) {
    h->thread_id = tid;
    for (int i = 0; i < 15; ++i) h->dummy[i] = 0u;
}
// sfq_init_kernel, sfqueue_hip.cpp:164-180
static __global__ void sfq_init_kernel(sfq_queue* q, sfq_handle* handles, int num_threads) {
    const int tid = blockIdx.x * blockDim.x + threadIdx.x;
    const int total = blockDim.x * gridDim.x;
    if (tid == 0) sfq_queue_init(q, (uint32_t)num_threads);
    for (int i = tid; i < (int)SFQ_QUEUE_LENGTH; i += total) q->slots[i] = 0;
    for (int i = tid; i < num_threads; i += total) sfq_handle_init(&handles[i], (uint32_t)i);
}
// sfq_queue_host_init / sfq_queue_destroy, sfqueue_hip.cpp:356-399.  The reference
// aborts the process on an error; this returns the CUDA error instead.
static inline cudaError_t sfq_queue_host_init(sfq_queue** d_q, sfq_handle** d_handles, int num_threads) {
    if (!d_q || !d_handles || num_threads < 0 || (uint32_t)num_threads > SFQ_MAX_THREADS) return cudaErrorInvalidValue;
    cudaError_t e = cudaMalloc((void**)d_q, sizeof(sfq_queue));
    if (e != cudaSuccess) return e;
    e = cudaMalloc((void**)d_handles, (size_t)(num_threads > 0 ? num_threads : 1) * sizeof(sfq_handle));
    if (e != cudaSuccess) { cudaFree(*d_q); return e; }
    const int threads = 256;
    const int blocks = num_threads > 0 ? (num_threads + threads - 1) / threads : 1;
    sfq_init_kernel<<<blocks, threads>>>(*d_q, *d_handles, num_threads);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    return cudaDeviceSynchronize();
}
static inline void sfq_queue_destroy(sfq_queue* d_q, sfq_handle* d_h) {
    if (d_q) cudaFree(d_q);
    if (d_h) cudaFree(d_h);
}
