// Test program for the reference-named device API of include/gcq/*.cuh.
//
// Each queue is created, initialised and driven only through the names a program
// written against the reference's headers uses -- wf_mpmc_t / wf_mpmc_init /
// Enqueue_Ptr / Dequeue_Ptr (gwf_queue.hpp, gwf_ring.hpp), fq_mpmc_t / fq_init /
// fq_enqueue_ptr / fq_dequeue_ptr (glf_queue.hpp), wf_queue_host_init / wf_enqueue /
// wf_dequeue with wf_handle* (wfqueue_hip_opt.hpp), sfq_queue_host_init /
// sfq_enqueue / sfq_dequeue (sfqueue_hip.hpp) -- in the shape of the reference's
// history harness (correctness/history.cpp:151-227): every thread alternates an
// enqueue of (tid << 32) | (seq + 1) and a dequeue, and each operation is
// bracketed by a device-wide logical clock (wf_linlog.hpp:25-45).  The host side
// returns the records in the layout of the oracle's checker.
//
// Built by tests/test_gpu_reference_api.py with nvcc for sm_103a against
// include/ alone; not part of libgcq.so.
#include <cuda_runtime.h>
#include <stdint.h>

#include "gcq/gwf_ring.cuh"
#include "gcq/glf_queue.cuh"
#include "gcq/sfqueue.cuh"
#include "gcq/wfqueue.cuh"

struct rec {   // the oracle's history record
    uint64_t proc;
    uint32_t op, pad;
    uint64_t arg, ret;
    int64_t call, end;
};

typedef wf_mpmc_t<gwf_32k, 32768> gwf_q;

__device__ __forceinline__ int64_t tick(unsigned long long* clk) {
    __threadfence();
    const int64_t t = (int64_t)atomicAdd(clk, 1ull);
    __threadfence();
    return t;
}

__global__ void init_gwf(gwf_q* q) { wf_mpmc_init(q); }
__global__ void init_glf(fq_mpmc_t* q) { fq_init(q); }

// kind 0 G-WFQ, 1 G-LFQ, 2 YMC, 3 SFQ
__global__ void history(int kind, void* qv, void* hv, int ops, rec* log, unsigned long long* clk) {
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    rec* my = log + (uint64_t)tid * 2 * ops;
    for (int i = 0; i < ops; ++i) {
        uint64_t v = ((uint64_t)tid << 32) | (uint64_t)(i + 1);
        if (kind == 3) v = ((uint64_t)tid << 16) | (uint64_t)(i + 1);   // SFQ carries 32-bit items
        rec* e = &my[2 * i];
        e->proc = tid; e->op = 0; e->arg = v;
        e->call = tick(clk);
        bool ok = true;
        if (kind == 0) ok = Enqueue_Ptr((gwf_q*)qv, v);
        else if (kind == 1) ok = fq_enqueue_ptr((fq_mpmc_t*)qv, v);
        else if (kind == 2) ok = wf_enqueue((wf_queue*)qv, &((wf_handle*)hv)[tid], v);
        else sfq_enqueue((sfq_queue*)qv, &((sfq_handle*)hv)[tid], v);
        e->ret = ok ? 1 : 0;
        e->end = tick(clk);

        rec* d = &my[2 * i + 1];
        d->proc = tid; d->op = 1; d->arg = 0;
        d->call = tick(clk);
        uint64_t out = 0;
        if (kind == 0) { if (!Dequeue_Ptr((gwf_q*)qv, &out)) out = 0; }
        else if (kind == 1) { if (!fq_dequeue_ptr((fq_mpmc_t*)qv, &out)) out = 0; }
        else if (kind == 2) out = wf_dequeue((wf_queue*)qv, &((wf_handle*)hv)[tid]);   // WF_EMPTY = 0
        else out = sfq_dequeue((sfq_queue*)qv, &((sfq_handle*)hv)[tid]);              // SFQ_EMPTY = 0
        d->ret = out;
        d->end = tick(clk);
    }
}

// Records of `threads` threads (one block) x `ops` pairs into out (threads*2*ops
// entries); returns 0, or the failing CUDA error.
extern "C" int ref_api_history(int kind, int threads, int ops, rec* out) {
    if (kind < 0 || kind > 3 || threads <= 0 || threads > 1024 || ops <= 0) return -1;
    void* q = nullptr;
    void* h = nullptr;
    cudaError_t e = cudaSuccess;
    if (kind == 0) {
        if ((e = cudaMalloc(&q, sizeof(gwf_q))) != cudaSuccess) return e;
        init_gwf<<<1, 1>>>((gwf_q*)q);
    } else if (kind == 1) {
        if ((e = cudaMalloc(&q, sizeof(fq_mpmc_t))) != cudaSuccess) return e;
        init_glf<<<1, 1>>>((fq_mpmc_t*)q);
    } else if (kind == 2) {
        e = wf_queue_host_init((wf_queue**)&q, (wf_handle**)&h, threads);
    } else {
        e = sfq_queue_host_init((sfq_queue**)&q, (sfq_handle**)&h, threads);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    rec* log = nullptr;
    unsigned long long* clk = nullptr;
    const size_t n = (size_t)threads * 2 * ops;
    if (e == cudaSuccess) e = cudaMalloc(&log, n * sizeof(rec));
    if (e == cudaSuccess) e = cudaMalloc(&clk, sizeof(unsigned long long));
    const unsigned long long one = 1;
    if (e == cudaSuccess) e = cudaMemcpy(clk, &one, sizeof one, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        history<<<1, threads>>>(kind, q, h, ops, log, clk);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(out, log, n * sizeof(rec), cudaMemcpyDeviceToHost);
    if (log) cudaFree(log);
    if (clk) cudaFree(clk);
    if (kind == 2) wf_queue_host_destroy((wf_queue*)q, (wf_handle*)h);
    else if (kind == 3) sfq_queue_destroy((sfq_queue*)q, (sfq_handle*)h);
    else if (q) cudaFree(q);
    return (int)e;
}

// ------------------------------------------------------------------ publication
// A queue of record ids, as a program that hands filled records from producers to
// consumers uses it: a producer writes the four words of record `id` with plain
// stores, then enqueues id; a consumer dequeues an id and reads the record with
// plain loads.  The reference publishes the producer's writes with its enqueue
// (Enqueue_Ptr's __threadfence before the index enqueue, gwf_ring.hpp:1362-1369;
// fq_enqueue_ptr's ordered index enqueue, glf_queue.hpp:566-572; the cell CAS of
// wf_enqueue; SFQ's slot store), so every record must read complete.  The first
// half of the blocks produce, the second half consume; waits end at a deadline
// on the device clock.  cnt: [0] records received, [1] records read incomplete,
// [2] threads that gave up at the deadline, [3] ids received more than once.
__device__ __forceinline__ uint64_t now_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint64_t rec_word(uint64_t id, int k) {
    return (id * 0x9E3779B97F4A7C15ull) ^ ((uint64_t)(k + 1) << 56) ^ (id << (8 * k));
}
__global__ void publish(int kind, void* qv, void* hv, int per, uint64_t* recs, unsigned* seen,
                        unsigned long long* cnt, uint64_t budget_ns) {
    const uint64_t deadline = now_ns() + budget_ns;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t half = (gridDim.x / 2) * blockDim.x;
    const unsigned long long total = (unsigned long long)half * per;
    wf_handle* wh = (wf_handle*)hv;
    if (tid < half) {
        for (int i = 0; i < per; ++i) {
            const uint64_t id = (uint64_t)tid * per + i + 1;
            for (int k = 0; k < 4; ++k) recs[4 * id + k] = rec_word(id, k);
            uint32_t ns = 32;
            for (;;) {
                bool ok;
                if (kind == 0) ok = Enqueue_Ptr((gwf_q*)qv, id);
                else if (kind == 1) ok = fq_enqueue_ptr((fq_mpmc_t*)qv, id);
                else if (kind == 2) ok = wf_enqueue((wf_queue*)qv, &wh[tid], id);
                else ok = sfq_enqueue_nb_u32((sfq_queue*)qv, (uint32_t)id) == SFQ_SUCCESS;
                if (ok) break;
                if (now_ns() > deadline) { atomicAdd(&cnt[2], 1ull); return; }
                __nanosleep(ns);
                ns = ns < 2048 ? 2 * ns : ns;
            }
        }
        return;
    }
    uint32_t ns = 32;
    while (*(volatile unsigned long long*)&cnt[0] < total) {
        if (now_ns() > deadline) { atomicAdd(&cnt[2], 1ull); return; }
        uint64_t id = 0;
        if (kind == 0) { if (!Dequeue_Ptr((gwf_q*)qv, &id)) id = 0; }
        else if (kind == 1) { if (!fq_dequeue_ptr((fq_mpmc_t*)qv, &id)) id = 0; }
        else if (kind == 2) id = wf_dequeue((wf_queue*)qv, &wh[tid]);
        else { uint32_t v = 0; if (sfq_dequeue_nb_u32((sfq_queue*)qv, &v) == SFQ_SUCCESS) id = v; }
        if (id == 0) {
            __nanosleep(ns);
            ns = ns < 2048 ? 2 * ns : ns;
            continue;
        }
        ns = 32;
        bool good = id <= total;
        for (int k = 0; good && k < 4; ++k) good = recs[4 * id + k] == rec_word(id, k);
        if (!good) atomicAdd(&cnt[1], 1ull);
        else if (atomicAdd(&seen[id], 1u) != 0) atomicAdd(&cnt[3], 1ull);
        atomicAdd(&cnt[0], 1ull);
    }
}

// `blocks` blocks of `threads` (blocks even, all resident), `per` records per
// producer; out receives cnt[0..3] and the expected total.  0, or the failing
// CUDA error.
extern "C" int ref_api_publish(int kind, int blocks, int threads, int per, unsigned long long* out) {
    if (kind < 0 || kind > 3 || blocks < 2 || (blocks & 1) || threads <= 0 || threads > 1024 || per <= 0) return -1;
    const int nthreads = blocks * threads;
    const unsigned long long total = (unsigned long long)(blocks / 2) * threads * per;
    if (total >= (kind == 1 ? FQ_N : 32768u)) return -1;   // under every queue's capacity
    void* q = nullptr;
    void* h = nullptr;
    cudaError_t e = cudaSuccess;
    if (kind == 0) {
        if ((e = cudaMalloc(&q, sizeof(gwf_q))) != cudaSuccess) return e;
        init_gwf<<<1, 1>>>((gwf_q*)q);
    } else if (kind == 1) {
        if ((e = cudaMalloc(&q, sizeof(fq_mpmc_t))) != cudaSuccess) return e;
        init_glf<<<1, 1>>>((fq_mpmc_t*)q);
    } else if (kind == 2) {
        e = wf_queue_host_init((wf_queue**)&q, (wf_handle**)&h, nthreads);
    } else {
        e = sfq_queue_host_init((sfq_queue**)&q, (sfq_handle**)&h, nthreads);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    uint64_t* recs = nullptr;
    unsigned long long* cnt = nullptr;
    unsigned* seen = nullptr;
    const size_t rbytes = (size_t)(total + 1) * 4 * sizeof(uint64_t);
    if (e == cudaSuccess) e = cudaMalloc(&recs, rbytes);
    if (e == cudaSuccess) e = cudaMemset(recs, 0, rbytes);
    if (e == cudaSuccess) e = cudaMalloc(&seen, (size_t)(total + 1) * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMemset(seen, 0, (size_t)(total + 1) * sizeof(unsigned));
    if (e == cudaSuccess) e = cudaMalloc(&cnt, 4 * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(cnt, 0, 4 * sizeof(unsigned long long));
    if (e == cudaSuccess) {
        publish<<<blocks, threads>>>(kind, q, h, per, recs, seen, cnt, 2000000000ull);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess) e = cudaMemcpy(out, cnt, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost);
    out[4] = total;
    if (recs) cudaFree(recs);
    if (cnt) cudaFree(cnt);
    if (seen) cudaFree(seen);
    if (kind == 2) wf_queue_host_destroy((wf_queue*)q, (wf_handle*)h);
    else if (kind == 3) sfq_queue_destroy((sfq_queue*)q, (sfq_handle*)h);
    else if (q) cudaFree(q);
    return (int)e;
}
