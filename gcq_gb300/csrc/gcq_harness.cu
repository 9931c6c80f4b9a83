// Harness kernels of libgcq.so: history recording (correctness/history.cpp),
// fixed-duration throughput chunks (throughout_bench.cpp) and the produce-then-drain
// FIFO check (throughout_bench.cpp MODE_FIFO), for all four queues.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <mutex>
#include <vector>

#include <map>
#include <tuple>
#include <vector>

#include "gcq_internal.cuh"

using gcqi::qops;

namespace {

// ------------------------------------------------------------------ helpers
template <int K>
__device__ __forceinline__ typename qops<K>::Q* as_q(void* p) {
    return reinterpret_cast<typename qops<K>::Q*>(p);
}

// Sum four per-thread counters over the block and add them to `out` with one
// atomic per counter per block (the reference adds per thread, :836-839).
__device__ __forceinline__ void block_add_counters(uint64_t a, uint64_t b, uint64_t c, uint64_t d,
                                                   gcq_tb_counters* out) {
    __shared__ unsigned long long s[4][32];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned nwarps = (blockDim.x + 31) >> 5;
    unsigned long long v[4] = {a, b, c, d};
#pragma unroll
    for (int k = 0; k < 4; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    if (lane == 0)
        for (int k = 0; k < 4; ++k) s[k][warp] = v[k];
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            unsigned long long x = lane < nwarps ? s[k][lane] : 0ull;
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            v[k] = x;
        }
        if (lane == 0) {
            unsigned long long* o = reinterpret_cast<unsigned long long*>(out);
            if (v[0]) atomicAdd(&o[0], v[0]);
            if (v[1]) atomicAdd(&o[1], v[1]);
            if (v[2]) atomicAdd(&o[2], v[2]);
            if (v[3]) atomicAdd(&o[3], v[3]);
        }
    }
}

// ------------------------------------------------------------------ throughput
// balanced_chunk_kernel (mode 0, throughout_bench.cpp:810-840) and
// split_chunk_kernel (mode 1, :842-882) in one body.  Payload i of thread t is
// payloads[i * threads + t] when payloads is given, else splitmix64(seed, t, i).
// All lanes stay to the end for the block reduction (the reference returns early).
// Bounded: the sweep's form -- every thread stops at the %globaltimer value in
// *deadline (read once at the start), so one point of a slow configuration cannot
// run past its window; the counters hold what completed.
template <int K, bool Bounded = false>
__global__ void __launch_bounds__(1024) k_tb_chunk(void* qv, int mode, int producer_percent, uint32_t threads,
                                                   uint32_t chunk_ops, uint64_t seed, const uint32_t* payloads,
                                                   gcq_tb_counters* ctr, const uint64_t* deadline = nullptr) {
    auto* q = as_q<K>(qv);
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    uint64_t eo = 0, ef = 0, dok = 0, de = 0;
    if (tid < threads) {
        const bool producer = ((uint64_t)tid * 100u / threads) < (uint64_t)producer_percent;
        const bool nb = (mode == 1);   // SFQ: blocking when balanced, non-blocking when split
        const uint64_t stop = Bounded ? *deadline : 0;
        using O = gcqi::qops_ctx<K>;
        typename O::ctx cx = O::ctx_begin(q, tid);
        typename O::ctx* px = GCQ_TB_CTX ? &cx : nullptr;
        for (uint32_t i = 0; i < chunk_ops; ++i) {
            if (Bounded && gcq::globaltimer_ns() > stop) break;
            if (mode == 0 || producer) {
                const uint32_t p = payloads ? payloads[(uint64_t)i * threads + tid]
                                            : (uint32_t)gcqi::splitmix64(seed ^ (((uint64_t)tid << 32) | i));
                if (O::enq(q, qops<K>::tb_value(p), tid, nb, px)) ++eo; else ++ef;
            }
            if (mode == 0 || !producer) {
                uint64_t out = 0;
                if (O::deq(q, &out, tid, nb, px) == 1) ++dok; else ++de;
            }
        }
        if (GCQ_TB_CTX) O::ctx_end(q, tid, cx);
    }
    block_add_counters(eo, ef, dok, de, ctr);
}

const void* tb_kernel(int kind) {
    switch (kind) {
        case GCQ_GWFQ: return (const void*)k_tb_chunk<GCQ_GWFQ>;
        case GCQ_GLFQ: return (const void*)k_tb_chunk<GCQ_GLFQ>;
        case GCQ_WFQ: return (const void*)k_tb_chunk<GCQ_WFQ>;
        case GCQ_SFQ: return (const void*)k_tb_chunk<GCQ_SFQ>;
    }
    return nullptr;
}

int check_tb_args(gcq_queue* q, int mode, int pct, uint32_t threads, uint32_t block, uint32_t chunk_ops) {
    if (!q || threads == 0 || block == 0 || block > 1024 || (block & 31) || chunk_ops == 0) return GCQ_EINVAL;
    if (mode != 0 && mode != 1) return GCQ_EINVAL;
    if (mode == 1 && (pct < 0 || pct > 100)) return GCQ_EINVAL;
    if (threads > q->max_threads) return GCQ_EINVAL;
    if (q->kind == GCQ_SFQ && mode == 0) {
        // blocking SFQ waits on other threads: all of them must be resident
        uint64_t res = 0;
        int rc = gcqi::resident_threads(tb_kernel(q->kind), (int)block, 0, &res);
        if (rc != GCQ_OK) return rc;
        if (threads > res) return GCQ_EUNSUPPORTED;
    }
    return GCQ_OK;
}

int launch_tb(gcq_queue* q, int mode, int pct, uint32_t threads, uint32_t block, uint32_t chunk_ops,
              uint64_t seed, const uint32_t* payloads, gcq_tb_counters* ctr, cudaStream_t s) {
    const unsigned grid = (threads + block - 1) / block;
    switch (q->kind) {
        case GCQ_GWFQ: k_tb_chunk<GCQ_GWFQ><<<grid, block, 0, s>>>(q->obj, mode, pct, threads, chunk_ops, seed, payloads, ctr); break;
        case GCQ_GLFQ: k_tb_chunk<GCQ_GLFQ><<<grid, block, 0, s>>>(q->obj, mode, pct, threads, chunk_ops, seed, payloads, ctr); break;
        case GCQ_WFQ: k_tb_chunk<GCQ_WFQ><<<grid, block, 0, s>>>(q->obj, mode, pct, threads, chunk_ops, seed, payloads, ctr); break;
        case GCQ_SFQ: k_tb_chunk<GCQ_SFQ><<<grid, block, 0, s>>>(q->obj, mode, pct, threads, chunk_ops, seed, payloads, ctr); break;
        default: return GCQ_EINVAL;
    }
    GCQ_CUDA(cudaGetLastError());
    return GCQ_OK;
}

__global__ void k_stamp_deadline(uint64_t* deadline, uint64_t after_ns) {
    *deadline = gcq::globaltimer_ns() + after_ns;
}

int launch_tb_bounded(gcq_queue* q, int mode, int pct, uint32_t threads, uint32_t block, uint32_t chunk_ops,
                      uint64_t seed, gcq_tb_counters* ctr, const uint64_t* deadline, cudaStream_t s) {
    const unsigned grid = (threads + block - 1) / block;
    switch (q->kind) {
        case GCQ_GWFQ: k_tb_chunk<GCQ_GWFQ, true><<<grid, block, 0, s>>>(q->obj, mode, pct, threads, chunk_ops, seed, nullptr, ctr, deadline); break;
        case GCQ_GLFQ: k_tb_chunk<GCQ_GLFQ, true><<<grid, block, 0, s>>>(q->obj, mode, pct, threads, chunk_ops, seed, nullptr, ctr, deadline); break;
        case GCQ_WFQ: k_tb_chunk<GCQ_WFQ, true><<<grid, block, 0, s>>>(q->obj, mode, pct, threads, chunk_ops, seed, nullptr, ctr, deadline); break;
        case GCQ_SFQ: k_tb_chunk<GCQ_SFQ, true><<<grid, block, 0, s>>>(q->obj, mode, pct, threads, chunk_ops, seed, nullptr, ctr, deadline); break;
        default: return GCQ_EINVAL;
    }
    GCQ_CUDA(cudaGetLastError());
    return GCQ_OK;
}

int read_error_word(gcq_queue* q, cudaStream_t s, uint32_t* err) {
    GCQ_CUDA(cudaMemcpyAsync(err, q->err, 4, cudaMemcpyDeviceToHost, s));
    GCQ_CUDA(cudaStreamSynchronize(s));
    return GCQ_OK;
}

// Map the error word after a harness run: timeouts and bounded loops are errors;
// YMC pool exhaustion is the reference's documented behaviour (failed operations).
int status_of(uint32_t err) {
    if (err & GCQ_ERR_TIMEOUT) return GCQ_ETIMEDOUT;
    if (err & (GCQ_ERR_SPIN | GCQ_ERR_TID | GCQ_ERR_CAPACITY)) return GCQ_EDEVICE;
    return GCQ_OK;
}

// ------------------------------------------------------------------ history
// alternating_history_kernel / split_history_kernel (history.cpp:188-227) with the
// WF_LOG_* bracketing of wf_linlog.hpp:25-45.  The clock RMWs are acq_rel, so a
// record whose end precedes another's call happens before it.
__device__ __forceinline__ uint64_t hist_value(int kind, int value_mode, uint32_t tid, uint32_t seq) {
    if (kind == GCQ_SFQ) return (uint64_t)(((tid & 0x7FFFu) << 16) | ((seq + 1u) & 0xFFFFu));
    if (value_mode == 1) return (uint64_t)(((tid & 0xFFFFu) << 16) | ((seq + 1u) & 0xFFFFu));
    return ((uint64_t)tid << 32) | (uint64_t)(seq + 1u);
}

template <int K>
__global__ void k_history(void* qv, uint32_t threads, uint32_t ops, int mode, int pct, int value_mode,
                          gcq_log_entry* log, uint32_t stride, gcq::u64a* clock) {
    auto* q = as_q<K>(qv);
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= threads) return;
    const bool producer = ((uint64_t)tid * 100u / threads) < (uint64_t)pct;
    gcq_log_entry* my = log + (uint64_t)tid * stride;
    uint32_t k = 0;
    for (uint32_t i = 0; i < ops; ++i) {
        if (mode == 0 || producer) {
            const uint64_t v = hist_value(K, value_mode, tid, i);
            gcq_log_entry* e = &my[k++];
            e->proc = tid; e->op = 0; e->arg = v;
            e->call = (int64_t)gcq::fetch_add(clock, 1ull);
            const bool ok = qops<K>::enq(q, v, tid, true);
            e->ret = ok ? 1 : 0;
            e->end = (int64_t)gcq::fetch_add(clock, 1ull);
        }
        if (mode == 0 || !producer) {
            gcq_log_entry* e = &my[k++];
            e->proc = tid; e->op = 1; e->arg = 0;
            e->call = (int64_t)gcq::fetch_add(clock, 1ull);
            uint64_t out = 0;
            const int r = qops<K>::deq(q, &out, tid, true);
            e->ret = (r == 1) ? out : 0;
            if (r == 2) e->op = 2;   // failed without effect (SFQ BUSY)
            e->end = (int64_t)gcq::fetch_add(clock, 1ull);
        }
    }
}

// ------------------------------------------------------------------ FIFO check
__device__ __forceinline__ uint64_t fifo_token(int kind, uint32_t tid, uint32_t seq) {
    if (kind == GCQ_SFQ) return (uint64_t)(((tid & 0x7FFFu) << 16) | ((seq + 1u) & 0xFFFFu));
    return ((uint64_t)tid << 32) | (uint64_t)(seq + 1u);
}

// fifo_produce_kernel, throughout_bench.cpp:531-542, with a deadline per token.
template <int K>
__global__ void k_fifo_produce(void* qv, uint32_t threads, uint32_t ops, uint64_t timeout_ns, gcq::u32a* err) {
    auto* q = as_q<K>(qv);
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= threads) return;
    for (uint32_t i = 0; i < ops; ++i) {
        const uint64_t tok = fifo_token(K, tid, i);
        gcq::backoff bo;
        const uint64_t t0 = gcq::globaltimer_ns();
        while (!qops<K>::enq(q, tok, tid, true)) {
            if (gcq::globaltimer_ns() - t0 > timeout_ns) { gcq::raise_error(err, gcq::ERR_TIMEOUT); return; }
            bo.pause(512);
        }
    }
}

// fifo_drain_kernel, throughout_bench.cpp:544-590.  Each taken token records its
// dequeue's (call, end) on the logical clock for the order check on the host.
template <int K>
__global__ void k_fifo_drain(void* qv, uint32_t threads, uint32_t ops, uint64_t total, uint32_t* counts,
                             int64_t* calls, int64_t* ends, gcq::u64a* consumed, gcq::u64a* clock,
                             gcq::u32a* oob, uint64_t timeout_ns, gcq::u32a* err) {
    auto* q = as_q<K>(qv);
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= threads) return;
    gcq::backoff bo;
    uint64_t t0 = gcq::globaltimer_ns();
    while (gcq::ld_acq(consumed) < total) {
        // poll through the read-only hint: a YMC dequeue on an empty queue uses up a
        // cell of its pool
        if (!qops<K>::maybe(q)) {
            if (gcq::globaltimer_ns() - t0 > timeout_ns) { gcq::raise_error(err, gcq::ERR_TIMEOUT); return; }
            bo.pause(512);
            continue;
        }
        const int64_t c0 = (int64_t)gcq::fetch_add(clock, 1ull);
        uint64_t v = 0;
        const int r = qops<K>::deq(q, &v, tid, true);
        const int64_t c1 = (int64_t)gcq::fetch_add(clock, 1ull);
        if (r != 1) {
            if (gcq::globaltimer_ns() - t0 > timeout_ns) { gcq::raise_error(err, gcq::ERR_TIMEOUT); return; }
            bo.pause(512);
            continue;
        }
        bo = gcq::backoff();
        t0 = gcq::globaltimer_ns();
        if (gcq::fetch_add(consumed, 1ull) >= total) continue;
        uint32_t ptid, seq;
        if (K == GCQ_SFQ) { ptid = (uint32_t)(v >> 16) & 0x7FFFu; seq = ((uint32_t)v & 0xFFFFu) - 1u; }
        else { ptid = (uint32_t)(v >> 32); seq = (uint32_t)v - 1u; }
        if (ptid >= threads || seq >= ops) { atomicAdd(oob, 1u); continue; }
        const uint64_t slot = (uint64_t)ptid * ops + seq;
        if (atomicAdd(&counts[slot], 1u) == 0u) {
            calls[slot] = c0;
            ends[slot] = c1;
        }
    }
}

// Concurrent split-mode FIFO check (no counterpart in the reference, whose FIFO
// mode produces everything before it drains, throughout_bench.cpp:456-767): the
// threads of the split chunk kernel's producer share (the same thread-to-role rule
// as k_tb_chunk) each enqueue ops tokens, retrying while the queue is full, while
// the other threads dequeue them in the same launch until all are consumed.  Every
// wait has a deadline.  Needs every thread resident (the host checks).
template <int K>
__global__ void k_fifo_split(void* qv, uint32_t threads, int pct, uint32_t nprod, uint32_t ops, uint64_t total,
                             uint32_t* counts,
                             int64_t* calls, int64_t* ends, gcq::u64a* consumed, gcq::u64a* clock, gcq::u32a* oob,
                             uint64_t timeout_ns, gcq::u32a* err) {
    auto* q = as_q<K>(qv);
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= threads) return;
    const bool producer = ((uint64_t)tid * 100u / threads) < (uint64_t)pct;
    if (producer) {
        for (uint32_t i = 0; i < ops; ++i) {
            const uint64_t tok = fifo_token(K, tid, i);
            gcq::backoff bo;
            const uint64_t t0 = gcq::globaltimer_ns();
            while (!qops<K>::enq(q, tok, tid, true)) {
                if (gcq::globaltimer_ns() - t0 > timeout_ns) { gcq::raise_error(err, gcq::ERR_TIMEOUT); return; }
                bo.pause(512);
            }
        }
        return;
    }
    gcq::backoff bo;
    uint64_t t0 = gcq::globaltimer_ns();
    while (gcq::ld_acq(consumed) < total) {
        // poll through the read-only hint: a YMC dequeue on an empty queue uses up a
        // cell of its pool
        if (!qops<K>::maybe(q)) {
            if (gcq::globaltimer_ns() - t0 > timeout_ns) { gcq::raise_error(err, gcq::ERR_TIMEOUT); return; }
            bo.pause(512);
            continue;
        }
        const int64_t c0 = (int64_t)gcq::fetch_add(clock, 1ull);
        uint64_t v = 0;
        const int r = qops<K>::deq(q, &v, tid, true);
        const int64_t c1 = (int64_t)gcq::fetch_add(clock, 1ull);
        if (r != 1) {
            if (gcq::globaltimer_ns() - t0 > timeout_ns) { gcq::raise_error(err, gcq::ERR_TIMEOUT); return; }
            bo.pause(512);
            continue;
        }
        bo = gcq::backoff();
        t0 = gcq::globaltimer_ns();
        if (gcq::fetch_add(consumed, 1ull) >= total) continue;
        uint32_t ptid, seq;
        if (K == GCQ_SFQ) { ptid = (uint32_t)(v >> 16) & 0x7FFFu; seq = ((uint32_t)v & 0xFFFFu) - 1u; }
        else { ptid = (uint32_t)(v >> 32); seq = (uint32_t)v - 1u; }
        // counts/calls/ends hold nprod * ops slots: producers are threads 0..nprod-1
        if (ptid >= nprod || seq >= ops) { atomicAdd(oob, 1u); continue; }
        const uint64_t slot = (uint64_t)ptid * ops + seq;
        if (atomicAdd(&counts[slot], 1u) == 0u) {
            calls[slot] = c0;
            ends[slot] = c1;
        }
    }
}

// Drain a quiescent queue into out[0 .. cap): each thread dequeues until its
// dequeue reports empty (SFQ's non-blocking dequeue cannot tell empty from a lost
// race, so there a run of failed attempts ends the thread).
template <int K>
__global__ void k_drain(void* qv, uint32_t threads, uint64_t* out, uint64_t cap, gcq::u64a* n) {
    auto* q = as_q<K>(qv);
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    if (tid >= threads) return;
    uint32_t fails = 0;
    gcq::backoff bo;
    for (uint32_t k = 0; k < GCQ_SPIN_LIMIT; ++k) {
        uint64_t v = 0;
        const int r = qops<K>::deq(q, &v, tid, true);
        if (r == 0) return;
        if (r == 2) {
            if (++fails > 256) return;
            bo.pause(1024);
            continue;
        }
        fails = 0;
        const uint64_t i = gcq::fetch_add(n, 1ull);
        if (i < cap) out[i] = v;
    }
}

template <typename F>
int dispatch(int kind, F&& f) {
    switch (kind) {
        case GCQ_GWFQ: return f(std::integral_constant<int, GCQ_GWFQ>());
        case GCQ_GLFQ: return f(std::integral_constant<int, GCQ_GLFQ>());
        case GCQ_WFQ: return f(std::integral_constant<int, GCQ_WFQ>());
        case GCQ_SFQ: return f(std::integral_constant<int, GCQ_SFQ>());
    }
    return GCQ_EINVAL;
}

// RAII device buffer
struct dbuf {
    void* p = nullptr;
    ~dbuf() { if (p) cudaFree(p); }
    cudaError_t alloc(size_t n) { return cudaMalloc(&p, n); }
};

}  // namespace

extern "C" {

int gcq_tb_launch(gcq_queue* q, int mode, int producer_percent, uint32_t threads, uint32_t block,
                  uint32_t chunk_ops, uint64_t seed, void* dev_counters, void* stream) {
    int rc = check_tb_args(q, mode, producer_percent, threads, block, chunk_ops);
    if (rc != GCQ_OK) return rc;
    if (!dev_counters) return GCQ_EINVAL;
    return launch_tb(q, mode, producer_percent, threads, block, chunk_ops, seed, nullptr,
                     (gcq_tb_counters*)dev_counters, gcqi::as_stream(stream));
}

int gcq_tb_chunk_host(gcq_queue* q, int mode, int producer_percent, uint32_t threads, uint32_t block,
                      uint32_t chunk_ops, const uint32_t* host_payloads, gcq_tb_counters* host_counters,
                      void* stream) {
    int rc = check_tb_args(q, mode, producer_percent, threads, block, chunk_ops);
    if (rc != GCQ_OK) return rc;
    if (!host_payloads || !host_counters) return GCQ_EINVAL;
    cudaStream_t s = gcqi::as_stream(stream);
    const size_t pbytes = (size_t)threads * chunk_ops * sizeof(uint32_t);
    // Pinned host payloads are read by the kernel in place, over NVLink-C2C: each
    // warp reads one 128-byte row per iteration, at the top of the iteration, so the
    // transfer overlaps the queue operations instead of preceding them.  Pageable
    // memory is staged through a device copy as before.
    const uint32_t* direct = nullptr;
    {
        cudaPointerAttributes at;
        if (cudaPointerGetAttributes(&at, host_payloads) == cudaSuccess && at.type == cudaMemoryTypeHost &&
            at.devicePointer)
            direct = (const uint32_t*)at.devicePointer;
        else
            cudaGetLastError();
    }
    // device staging: payloads (pageable callers) + counters, kept across calls
    static thread_local void* stage = nullptr;
    static thread_local size_t stage_bytes = 0;
    const size_t need = (direct ? 0 : pbytes) + 256;
    if (stage_bytes < need) {
        if (stage) cudaFree(stage);
        stage = nullptr;
        stage_bytes = 0;
        GCQ_CUDA(cudaMalloc(&stage, need));
        stage_bytes = need;
    }
    uint32_t* d_pay = (uint32_t*)stage;
    gcq_tb_counters* d_ctr =
        (gcq_tb_counters*)((char*)stage + (direct ? 0 : ((pbytes + 127) / 128) * 128));
    if (!direct) GCQ_CUDA(cudaMemcpyAsync(d_pay, host_payloads, pbytes, cudaMemcpyHostToDevice, s));
    GCQ_CUDA(cudaMemsetAsync(d_ctr, 0, sizeof(gcq_tb_counters), s));
    rc = launch_tb(q, mode, producer_percent, threads, block, chunk_ops, 0, direct ? direct : d_pay, d_ctr, s);
    if (rc != GCQ_OK) return rc;
    GCQ_CUDA(cudaMemcpyAsync(host_counters, d_ctr, sizeof(gcq_tb_counters), cudaMemcpyDeviceToHost, s));
    uint32_t err = 0;
    rc = read_error_word(q, s, &err);   // synchronises s
    if (rc != GCQ_OK) return rc;
    return status_of(err);
}

int gcq_tb_run(gcq_queue* q, int mode, int producer_percent, uint32_t threads, uint32_t block,
               uint32_t chunk_ops, double warmup_ms, double run_ms, uint32_t graph_chunks,
               gcq_tb_result* out) {
    int rc = check_tb_args(q, mode, producer_percent, threads, block, chunk_ops);
    if (rc != GCQ_OK) return rc;
    if (!out || graph_chunks == 0) return GCQ_EINVAL;
    memset(out, 0, sizeof(*out));
    cudaStream_t s;
    GCQ_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    dbuf ctr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&]() {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        cudaStreamDestroy(s);
    };
    auto fail = [&](int r) { cleanup(); return r; };
    if (ctr.alloc(sizeof(gcq_tb_counters)) != cudaSuccess) return fail(GCQ_ENOMEM);
    gcq_tb_counters* d_ctr = (gcq_tb_counters*)ctr.p;
    // capture graph_chunks chunk launches (distinct payload seeds) as one graph
    if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) return fail(GCQ_ECUDA);
    for (uint32_t g = 0; g < graph_chunks; ++g) {
        rc = launch_tb(q, mode, producer_percent, threads, block, chunk_ops, 0x5eedULL + g, nullptr, d_ctr, s);
        if (rc != GCQ_OK) { cudaStreamEndCapture(s, &graph); return fail(rc); }
    }
    if (cudaStreamEndCapture(s, &graph) != cudaSuccess) return fail(GCQ_ECUDA);
    if (cudaGraphInstantiate(&exec, graph, 0) != cudaSuccess) return fail(GCQ_ECUDA);
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return fail(GCQ_ECUDA);
    using clk = std::chrono::steady_clock;
    // warm-up
    auto t0 = clk::now();
    do {
        if (cudaGraphLaunch(exec, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) return fail(GCQ_ECUDA);
    } while (std::chrono::duration<double, std::milli>(clk::now() - t0).count() < warmup_ms);
    if (cudaMemsetAsync(d_ctr, 0, sizeof(gcq_tb_counters), s) != cudaSuccess) return fail(GCQ_ECUDA);
    // timed window: graph replays until run_ms of host time
    uint64_t reps = 0;
    cudaEventRecord(e0, s);
    t0 = clk::now();
    do {
        if (cudaGraphLaunch(exec, s) != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess) return fail(GCQ_ECUDA);
        ++reps;
    } while (std::chrono::duration<double, std::milli>(clk::now() - t0).count() < run_ms);
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) != cudaSuccess) return fail(GCQ_ECUDA);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (cudaMemcpy(&out->counters, d_ctr, sizeof(gcq_tb_counters), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(GCQ_ECUDA);
    out->gpu_ms = ms;
    out->launches = reps * graph_chunks;
    uint32_t err = 0;
    rc = read_error_word(q, s, &err);
    cleanup();
    if (rc != GCQ_OK) return rc;
    return status_of(err);
}

int gcq_tb_run_bounded(gcq_queue* q, int mode, int producer_percent, uint32_t threads, uint32_t block,
                       uint32_t chunk_ops, double warmup_ms, double run_ms, uint32_t reset_every,
                       gcq_tb_result* out) {
    int rc = check_tb_args(q, mode, producer_percent, threads, block, chunk_ops);
    if (rc != GCQ_OK) return rc;
    if (!out || warmup_ms < 0 || run_ms <= 0) return GCQ_EINVAL;
    memset(out, 0, sizeof(*out));
    cudaStream_t s;
    GCQ_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    dbuf buf;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&]() {
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        cudaStreamDestroy(s);
    };
    auto fail = [&](int r) { cleanup(); return r; };
    if (buf.alloc(256) != cudaSuccess) return fail(GCQ_ENOMEM);
    gcq_tb_counters* d_ctr = (gcq_tb_counters*)buf.p;
    uint64_t* d_deadline = (uint64_t*)((char*)buf.p + 128);
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return fail(GCQ_ECUDA);
    using clk = std::chrono::steady_clock;
    uint64_t chunks = 0, seed = 0x5eedULL;
    double ms = 0.0;
    // one window: the device deadline is stamped at its start, then chunks run until
    // host time passes the window (each chunk also stops at the device deadline)
    auto window = [&](double win_ms, bool timed) -> int {
        if (cudaMemsetAsync(d_ctr, 0, sizeof(gcq_tb_counters), s) != cudaSuccess) return GCQ_ECUDA;
        k_stamp_deadline<<<1, 1, 0, s>>>(d_deadline, (uint64_t)(win_ms * 1e6));
        const auto t0 = clk::now();
        do {
            if (reset_every && chunks % reset_every == 0) {
                const int r = gcq_reset(q, s);
                if (r != GCQ_OK) return r;
            }
            if (timed && cudaEventRecord(e0, s) != cudaSuccess) return GCQ_ECUDA;
            const int r = launch_tb_bounded(q, mode, producer_percent, threads, block, chunk_ops, seed++, d_ctr,
                                            d_deadline, s);
            if (r != GCQ_OK) return r;
            if (timed && cudaEventRecord(e1, s) != cudaSuccess) return GCQ_ECUDA;
            if (cudaStreamSynchronize(s) != cudaSuccess) return GCQ_ECUDA;
            ++chunks;
            if (timed) {
                float m = 0.f;
                cudaEventElapsedTime(&m, e0, e1);
                ms += m;
                ++out->launches;
            }
        } while (std::chrono::duration<double, std::milli>(clk::now() - t0).count() < win_ms);
        return GCQ_OK;
    };
    if (warmup_ms > 0 && (rc = window(warmup_ms, false)) != GCQ_OK) return fail(rc);
    if ((rc = window(run_ms, true)) != GCQ_OK) return fail(rc);
    if (cudaMemcpy(&out->counters, d_ctr, sizeof(gcq_tb_counters), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(GCQ_ECUDA);
    out->gpu_ms = ms;
    uint32_t err = 0;
    rc = read_error_word(q, s, &err);
    cleanup();
    if (rc != GCQ_OK) return rc;
    return status_of(err);
}

int gcq_run_history(gcq_queue* q, uint32_t threads, uint32_t block, uint32_t ops, int mode,
                    int producer_percent, int value_mode, gcq_log_entry* host_out, size_t cap,
                    size_t* n_out, void* stream) {
    if (!q || !host_out || !n_out || threads == 0 || ops == 0 || block == 0 || block > 1024) return GCQ_EINVAL;
    if (mode != 0 && mode != 1) return GCQ_EINVAL;
    if (threads > q->max_threads) return GCQ_EINVAL;
    if (q->kind == GCQ_SFQ && (threads > 32768u || ops > 0xFFFFu)) return GCQ_EUNSUPPORTED;  // history.cpp:285-292
    const uint32_t stride = (mode == 0 ? 2u : 1u) * ops;
    const size_t total = (size_t)threads * stride;
    cudaStream_t s = gcqi::as_stream(stream);
    int rc = gcq_reset(q, stream);
    if (rc != GCQ_OK) return rc;
    dbuf log, clk;
    if (log.alloc(total * sizeof(gcq_log_entry)) != cudaSuccess || clk.alloc(256) != cudaSuccess) return GCQ_ENOMEM;
    GCQ_CUDA(cudaMemsetAsync(log.p, 0, total * sizeof(gcq_log_entry), s));
    const unsigned long long one = 1;
    GCQ_CUDA(cudaMemcpyAsync(clk.p, &one, sizeof one, cudaMemcpyHostToDevice, s));
    const unsigned grid = (threads + block - 1) / block;
    rc = dispatch(q->kind, [&](auto kc) {
        constexpr int K = decltype(kc)::value;
        k_history<K><<<grid, block, 0, s>>>(q->obj, threads, ops, mode, producer_percent, value_mode,
                                            (gcq_log_entry*)log.p, stride, (gcq::u64a*)clk.p);
        return GCQ_OK;
    });
    GCQ_CUDA(cudaGetLastError());
    std::vector<gcq_log_entry> h(total);
    GCQ_CUDA(cudaMemcpyAsync(h.data(), log.p, total * sizeof(gcq_log_entry), cudaMemcpyDeviceToHost, s));
    GCQ_CUDA(cudaStreamSynchronize(s));
    uint32_t err = 0;
    rc = read_error_word(q, s, &err);
    if (rc != GCQ_OK) return rc;
    // keep completed records and sort as wf_log_dump_jsonl does (history.cpp:257-267)
    std::vector<gcq_log_entry> used;
    used.reserve(total);
    for (const auto& e : h) if (e.end != 0) used.push_back(e);
    std::sort(used.begin(), used.end(), [](const gcq_log_entry& a, const gcq_log_entry& b) {
        if (a.call != b.call) return a.call < b.call;
        if (a.end != b.end) return a.end < b.end;
        if (a.proc != b.proc) return a.proc < b.proc;
        return a.op < b.op;
    });
    *n_out = used.size();
    if (used.size() > cap) return GCQ_ECAPACITY;
    memcpy(host_out, used.data(), used.size() * sizeof(gcq_log_entry));
    return status_of(err);
}

}  // extern "C"

namespace {

// Device buffers of one FIFO check and the host-side verdict: exactly once (in and
// out counts, duplicates, missing, out of range) and per-producer order -- for
// tokens a < b of one producer, the dequeue of b must not return before the
// dequeue of a was called (logical clock).  The reference's order check
// (throughout_bench.cpp:585-588) starts its atomicMax from 0xFFFFFFFF (:691) and
// never fires.
struct fifo_bufs {
    dbuf counts, calls, ends, misc;
    gcq::u64a* consumed() { return (gcq::u64a*)misc.p; }
    gcq::u64a* clock() { return (gcq::u64a*)misc.p + 1; }
    gcq::u32a* oob() { return (gcq::u32a*)((gcq::u64a*)misc.p + 2); }
    int alloc(uint64_t total) {
        if (counts.alloc(total * 4) != cudaSuccess || calls.alloc(total * 8) != cudaSuccess ||
            ends.alloc(total * 8) != cudaSuccess || misc.alloc(256) != cudaSuccess)
            return GCQ_ENOMEM;
        GCQ_CUDA(cudaMemset(counts.p, 0, total * 4));
        GCQ_CUDA(cudaMemset(misc.p, 0, 256));
        const unsigned long long one = 1;
        GCQ_CUDA(cudaMemcpy(clock(), &one, 8, cudaMemcpyHostToDevice));
        return GCQ_OK;
    }
};

// producers: thread indices p with slots p*ops .. p*ops+ops-1
int fifo_verify(gcq_queue* q, fifo_bufs& b, const std::vector<uint32_t>& producers, uint64_t ops, uint64_t total,
                gcq_fifo_result* out) {
    GCQ_CUDA(cudaGetLastError());
    GCQ_CUDA(cudaDeviceSynchronize());
    const uint64_t nslots = (uint64_t)(producers.empty() ? 0 : producers.back() + 1) * ops;
    std::vector<uint32_t> hc(nslots);
    std::vector<int64_t> hcall(nslots), hend(nslots);
    uint64_t hmisc[4];
    GCQ_CUDA(cudaMemcpy(hc.data(), b.counts.p, nslots * 4, cudaMemcpyDeviceToHost));
    GCQ_CUDA(cudaMemcpy(hcall.data(), b.calls.p, nslots * 8, cudaMemcpyDeviceToHost));
    GCQ_CUDA(cudaMemcpy(hend.data(), b.ends.p, nslots * 8, cudaMemcpyDeviceToHost));
    GCQ_CUDA(cudaMemcpy(hmisc, b.misc.p, sizeof hmisc, cudaMemcpyDeviceToHost));
    out->out_count = std::min<uint64_t>(hmisc[0], total);
    out->err_oob = (uint32_t)hmisc[2];
    for (uint32_t p : producers) {
        int64_t max_call = -1;
        for (uint64_t sq = 0; sq < ops; ++sq) {
            const uint64_t slot = (uint64_t)p * ops + sq;
            if (hc[slot] == 0) { out->err_missing++; continue; }
            if (hc[slot] > 1) { out->err_gt1++; out->err_dup += hc[slot] - 1; }
            if (hend[slot] < max_call) out->err_order++;
            max_call = std::max(max_call, hcall[slot]);
        }
    }
    uint32_t err = 0;
    GCQ_CUDA(cudaMemcpy(&err, q->err, 4, cudaMemcpyDeviceToHost));
    out->verified = (out->out_count == out->in_count && !out->err_oob && !out->err_dup && !out->err_order &&
                     !out->err_missing && !out->err_gt1) ? 1 : 0;
    return status_of(err);
}

}  // namespace

extern "C" {

int gcq_fifo_check(gcq_queue* q, uint32_t threads, uint32_t block, uint32_t ops_per_thread,
                   gcq_fifo_result* out) {
    if (!q || !out || threads == 0 || block == 0 || block > 1024) return GCQ_EINVAL;
    if (threads > q->max_threads) return GCQ_EINVAL;
    memset(out, 0, sizeof(*out));
    // fifo_effective_ops_per_thread, throughout_bench.cpp:627-653
    uint64_t ops = std::max<uint32_t>(1u, ops_per_thread);
    if (q->kind != GCQ_WFQ) {
        const uint64_t cap = 1ull << q->order;
        const uint64_t lim = cap / threads;
        if (lim == 0) { out->verified = -1; return GCQ_OK; }
        ops = std::min<uint64_t>(ops, lim);
    }
    if (q->kind == GCQ_SFQ) {
        if (threads > 32768u) { out->verified = -1; return GCQ_OK; }
        ops = std::min<uint64_t>(ops, 0xFFFFu);
    }
    out->ops_per_thread = (uint32_t)ops;
    const uint64_t total = (uint64_t)threads * ops;
    out->in_count = total;
    int rc = gcq_reset(q, nullptr);
    if (rc != GCQ_OK) return rc;
    fifo_bufs b;
    rc = b.alloc(total);
    if (rc != GCQ_OK) return rc;
    const unsigned grid = (threads + block - 1) / block;
    const uint64_t tmo = std::max<uint64_t>(q->knobs.wait_timeout_ns, 1000000000ull) * 4;
    rc = dispatch(q->kind, [&](auto kc) {
        constexpr int K = decltype(kc)::value;
        k_fifo_produce<K><<<grid, block>>>(q->obj, threads, (uint32_t)ops, tmo, q->err);
        k_fifo_drain<K><<<grid, block>>>(q->obj, threads, (uint32_t)ops, total, (uint32_t*)b.counts.p,
                                         (int64_t*)b.calls.p, (int64_t*)b.ends.p, b.consumed(), b.clock(), b.oob(),
                                         tmo, q->err);
        return GCQ_OK;
    });
    std::vector<uint32_t> producers(threads);
    for (uint32_t p = 0; p < threads; ++p) producers[p] = p;
    return fifo_verify(q, b, producers, ops, total, out);
}

int gcq_drain_host(gcq_queue* q, uint32_t threads, uint32_t block, uint64_t* host_out, size_t cap,
                   size_t* n_out) {
    if (!q || !n_out || (cap && !host_out) || threads == 0 || block == 0 || block > 1024 || (block & 31))
        return GCQ_EINVAL;
    if (threads > q->max_threads) return GCQ_EINVAL;
    dbuf buf, cnt;
    if ((cap && buf.alloc(cap * 8) != cudaSuccess) || cnt.alloc(256) != cudaSuccess) return GCQ_ENOMEM;
    GCQ_CUDA(cudaMemset(cnt.p, 0, 256));
    const unsigned grid = (threads + block - 1) / block;
    int rc = dispatch(q->kind, [&](auto kc) {
        constexpr int K = decltype(kc)::value;
        k_drain<K><<<grid, block>>>(q->obj, threads, (uint64_t*)buf.p, (uint64_t)cap, (gcq::u64a*)cnt.p);
        return GCQ_OK;
    });
    if (rc != GCQ_OK) return rc;
    GCQ_CUDA(cudaGetLastError());
    GCQ_CUDA(cudaDeviceSynchronize());
    uint64_t n = 0;
    GCQ_CUDA(cudaMemcpy(&n, cnt.p, 8, cudaMemcpyDeviceToHost));
    const uint64_t keep = std::min<uint64_t>(n, cap);
    if (keep) GCQ_CUDA(cudaMemcpy(host_out, buf.p, keep * 8, cudaMemcpyDeviceToHost));
    *n_out = (size_t)keep;
    uint32_t err = 0;
    GCQ_CUDA(cudaMemcpy(&err, q->err, 4, cudaMemcpyDeviceToHost));
    if (n > cap) return GCQ_ECAPACITY;
    return status_of(err);
}

int gcq_fifo_check_split(gcq_queue* q, uint32_t threads, uint32_t block, int producer_percent,
                         uint32_t ops_per_producer, gcq_fifo_result* out) {
    if (!q || !out || threads == 0 || block == 0 || block > 1024 || (block & 31) || ops_per_producer == 0)
        return GCQ_EINVAL;
    if (producer_percent <= 0 || producer_percent >= 100) return GCQ_EINVAL;
    if (threads > q->max_threads) return GCQ_EINVAL;
    memset(out, 0, sizeof(*out));
    uint64_t ops = ops_per_producer;
    if (q->kind == GCQ_SFQ) {
        if (threads > 32768u) return GCQ_EUNSUPPORTED;   // 15-bit producer field of the token
        ops = std::min<uint64_t>(ops, 0xFFFFu);
    }
    // producers wait for consumers and consumers for producers: all must be resident
    uint64_t res = 0;
    int rc = dispatch(q->kind, [&](auto kc) {
        constexpr int K = decltype(kc)::value;
        return gcqi::resident_threads((const void*)k_fifo_split<K>, (int)block, 0, &res);
    });
    if (rc != GCQ_OK) return rc;
    if (threads > res) return GCQ_EUNSUPPORTED;
    std::vector<uint32_t> producers;
    for (uint32_t t = 0; t < threads; ++t)
        if ((uint64_t)t * 100u / threads < (uint64_t)producer_percent) producers.push_back(t);
    if (producers.empty() || producers.size() == threads || producers.back() + 1 != producers.size())
        return GCQ_EINVAL;
    const uint64_t total = (uint64_t)producers.size() * ops;
    out->ops_per_thread = (uint32_t)ops;
    out->in_count = total;
    rc = gcq_reset(q, nullptr);
    if (rc != GCQ_OK) return rc;
    fifo_bufs b;
    rc = b.alloc((uint64_t)(producers.back() + 1) * ops);
    if (rc != GCQ_OK) return rc;
    const unsigned grid = (threads + block - 1) / block;
    const uint64_t tmo = std::max<uint64_t>(q->knobs.wait_timeout_ns, 1000000000ull) * 4;
    rc = dispatch(q->kind, [&](auto kc) {
        constexpr int K = decltype(kc)::value;
        k_fifo_split<K><<<grid, block>>>(q->obj, threads, producer_percent, (uint32_t)producers.size(),
                                         (uint32_t)ops, total,
                                         (uint32_t*)b.counts.p, (int64_t*)b.calls.p, (int64_t*)b.ends.p,
                                         b.consumed(), b.clock(), b.oob(), tmo, q->err);
        return GCQ_OK;
    });
    return fifo_verify(q, b, producers, ops, total, out);
}

}  // extern "C"

// ------------------------------------------------------------------ no-allocation chunk
// gcq_tb_chunk_host_noalloc: the end-to-end chunk of gcq_tb_chunk_host for callers
// that must not allocate device memory during the call, with its device staging in
// a fixed array of this file instead of a cudaMalloc'd buffer.
namespace {

// 16 MiB of payload staging (GCQ_NOALLOC_MAX_PAYLOADS uint32 values) followed by one
// 256-byte block for the counters.  Every GPU that loads the library holds it until
// the process exits.
constexpr uint64_t kNoallocPayloadWords = GCQ_NOALLOC_MAX_PAYLOADS;
constexpr uint64_t kNoallocWords = kNoallocPayloadWords + 64;
static __device__ __align__(256) uint32_t g_noalloc_scratch[kNoallocWords];

// Device address of g_noalloc_scratch, looked up once per CUDA context.  In host
// code the array's name stands for a host-side shadow, not a device address, so it
// must never be passed to a kernel; cudaGetSymbolAddress gives the address in the
// current device's context.  The cache is keyed by the context's unique id
// (cuCtxGetId, reached through the runtime's driver entry points, so the library
// does not link libcuda): after cudaDeviceReset the device's new primary context
// has a new id, and the first call in it looks the address up again.
typedef int (*ctx_get_current_fn)(void** ctx);
typedef int (*ctx_get_id_fn)(void* ctx, unsigned long long* id);
std::mutex g_noalloc_mu;
ctx_get_current_fn g_ctx_get_current = nullptr;
ctx_get_id_fn g_ctx_get_id = nullptr;
std::map<unsigned long long, void*> g_noalloc_ptr;   // context id -> device address

int current_ctx_id(unsigned long long* id) {
    void* ctx = nullptr;
    if (g_ctx_get_current(&ctx) != 0 || !ctx) return GCQ_ECUDA;
    if (g_ctx_get_id(ctx, id) != 0) return GCQ_ECUDA;
    return GCQ_OK;
}

int noalloc_scratch(void** out) {
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_ctx_get_current || !g_ctx_get_id) {
        cudaDriverEntryPointQueryResult r1, r2;
        void *f1 = nullptr, *f2 = nullptr;
        GCQ_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &r1));
        GCQ_CUDA(cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &r2));
        if (r1 != cudaDriverEntryPointSuccess || r2 != cudaDriverEntryPointSuccess || !f1 || !f2) return GCQ_ECUDA;
        g_ctx_get_current = (ctx_get_current_fn)f1;
        g_ctx_get_id = (ctx_get_id_fn)f2;
    }
    unsigned long long id = 0;
    if (current_ctx_id(&id) == GCQ_OK) {
        auto it = g_noalloc_ptr.find(id);
        if (it != g_noalloc_ptr.end()) {
            *out = it->second;
            return GCQ_OK;
        }
    }
    // set-up in this context (it also makes the device's primary context current
    // when no runtime call has done so in this thread yet)
    void* p = nullptr;
    GCQ_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    if (!p) return GCQ_ECUDA;
    if (current_ctx_id(&id) != GCQ_OK) return GCQ_ECUDA;
    g_noalloc_ptr[id] = p;
    *out = p;
    return GCQ_OK;
}

}  // namespace

extern "C" int gcq_tb_chunk_host_noalloc(gcq_queue* q, int mode, int producer_percent, uint32_t threads,
                                         uint32_t block, uint32_t chunk_ops, const uint32_t* host_payloads,
                                         gcq_tb_counters* host_counters, void* stream) {
    int rc = check_tb_args(q, mode, producer_percent, threads, block, chunk_ops);
    if (rc != GCQ_OK) return rc;
    if (!host_payloads || !host_counters) return GCQ_EINVAL;
    if ((uint64_t)threads * chunk_ops > kNoallocPayloadWords) return GCQ_ECAPACITY;
    void* base = nullptr;
    rc = noalloc_scratch(&base);
    if (rc != GCQ_OK) return rc;
    cudaStream_t s = gcqi::as_stream(stream);
    uint32_t* d_pay = (uint32_t*)base;
    gcq_tb_counters* d_ctr = (gcq_tb_counters*)((uint32_t*)base + kNoallocPayloadWords);
    const size_t pbytes = (size_t)threads * chunk_ops * sizeof(uint32_t);
    GCQ_CUDA(cudaMemcpyAsync(d_pay, host_payloads, pbytes, cudaMemcpyHostToDevice, s));
    // the array keeps the previous call's counters: clear them before the kernel adds
    GCQ_CUDA(cudaMemsetAsync(d_ctr, 0, sizeof(gcq_tb_counters), s));
    rc = launch_tb(q, mode, producer_percent, threads, block, chunk_ops, 0, d_pay, d_ctr, s);
    if (rc != GCQ_OK) return rc;
    GCQ_CUDA(cudaMemcpyAsync(host_counters, d_ctr, sizeof(gcq_tb_counters), cudaMemcpyDeviceToHost, s));
    uint32_t err = 0;
    rc = read_error_word(q, s, &err);   // synchronises s
    if (rc != GCQ_OK) return rc;
    return status_of(err);
}

// ------------------------------------------------------------------ autotuner
// Coordinate descent over the launch shape and the queue knobs of one throughput
// configuration (the reference fixes them at compile time and sweeps by hand:
// throughout_bench.cpp:1088, Makefile TB_* knobs).  Each candidate is a fresh queue
// and a short gcq_tb_run; a knob moves to the value with the highest successful
// operation rate while the others stay at their current best, and the sweep makes
// `passes` rounds over the knobs.
namespace {

struct tune_space {
    std::vector<uint32_t> block, chunk, deq_wait, remap;
};

int tune_point(int kind, uint32_t capacity_log2, uint32_t threads, int mode, int pp, double ms,
               const gcq_tune_point& p, double* mops) {
    gcq_knobs k;
    gcq_default_knobs(&k);
    k.deq_wait = p.deq_wait;
    k.remap = p.remap;
    gcq_queue* q = nullptr;
    int rc = gcq_create(kind, capacity_log2, threads, &k, &q);
    if (rc != GCQ_OK) return rc;
    gcq_tb_result r;
    rc = gcq_tb_run(q, mode, pp, threads, p.block, p.chunk_ops, ms / 3, ms, 8, &r);
    if (rc == GCQ_OK) {
        uint32_t err = 0;
        gcq_error_word(q, &err, 0);
        if (err & ~GCQ_ERR_POOL) rc = GCQ_EDEVICE;
    }
    gcq_destroy(q);
    if (rc != GCQ_OK) return rc;
    *mops = r.gpu_ms > 0 ? (double)(r.counters.enq_success + r.counters.deq_success) / (r.gpu_ms * 1e3) : 0.0;
    return GCQ_OK;
}

}  // namespace

extern "C" int gcq_tb_autotune(int kind, uint32_t capacity_log2, uint32_t threads, int mode, int producer_percent,
                               double ms_per_point, uint32_t passes, gcq_tune_point* best, gcq_tune_point* table,
                               size_t cap, size_t* n_out) {
    if (!best || threads == 0 || ms_per_point <= 0 || passes == 0) return GCQ_EINVAL;
    tune_space sp;
    sp.block = {128, 256, 512, 1024};
    sp.chunk = {32, 64, 128, 256};
    if (kind == GCQ_GWFQ || kind == GCQ_GLFQ) {
        sp.deq_wait = {0, 2, 8, 32};
        sp.remap = {0, 1};
    } else {
        sp.deq_wait = {8};
        sp.remap = {0};
    }
    gcq_knobs dk;
    gcq_default_knobs(&dk);
    gcq_tune_point cur;
    memset(&cur, 0, sizeof cur);
    cur.block = 256;
    cur.chunk_ops = 128;
    cur.deq_wait = (kind == GCQ_GWFQ || kind == GCQ_GLFQ) ? dk.deq_wait : 8;
    cur.remap = kind == GCQ_GLFQ ? 1u : 0u;
    size_t n = 0;
    std::map<std::tuple<uint32_t, uint32_t, uint32_t, uint32_t>, double> seen;
    auto eval = [&](gcq_tune_point p) -> double {
        const auto key = std::make_tuple(p.block, p.chunk_ops, p.deq_wait, p.remap);
        auto it = seen.find(key);
        if (it != seen.end()) return it->second;
        double mops = -1.0;
        if (threads % p.block == 0) {
            const int rc = tune_point(kind, capacity_log2, threads, mode, producer_percent, ms_per_point, p, &mops);
            if (rc == GCQ_ECUDA) return -2.0;   // the context may be unusable: stop
            if (rc != GCQ_OK) mops = -1.0;
        }
        seen[key] = mops;
        p.succ_mops = mops;
        p.status = mops >= 0 ? 0 : -1;
        if (table && n < cap) table[n] = p;
        ++n;
        return mops;
    };
    double best_v = eval(cur);
    if (best_v == -2.0) return GCQ_ECUDA;
    for (uint32_t pass = 0; pass < passes; ++pass) {
        for (int knob = 0; knob < 4; ++knob) {
            const std::vector<uint32_t>& vals =
                knob == 0 ? sp.block : knob == 1 ? sp.chunk : knob == 2 ? sp.deq_wait : sp.remap;
            for (uint32_t v : vals) {
                gcq_tune_point p = cur;
                (knob == 0 ? p.block : knob == 1 ? p.chunk_ops : knob == 2 ? p.deq_wait : p.remap) = v;
                const double m = eval(p);
                if (m == -2.0) return GCQ_ECUDA;
                if (m > best_v) {
                    best_v = m;
                    cur = p;
                }
            }
        }
    }
    cur.succ_mops = best_v;
    cur.status = best_v >= 0 ? 0 : -1;
    *best = cur;
    if (n_out) *n_out = n;
    return best_v >= 0 ? GCQ_OK : GCQ_EDEVICE;
}
