// Queue lifecycle of libgcq.so: creation with the reference's envelope checks,
// one device allocation per queue, grid-stride initialisation, error word access.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <string>

#include "gcq_internal.cuh"

namespace {

std::mutex g_err_mu;
std::string g_last_cuda;

constexpr uint32_t REMAP_AUTO = 0xFFFFFFFFu;

inline uint64_t align_up(uint64_t x, uint64_t a) { return (x + a - 1) / a * a; }

// ---------------------------------------------------------------- init kernels
__global__ void k_init_gwf(gcq::gwf::mpmc* q) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t n = (uint64_t)gridDim.x * blockDim.x;
    gcq::gwf::init_slice(&q->aq, false, gid, n);
    gcq::gwf::init_slice(&q->fq, true, gid, n);
    for (uint64_t i = gid; i < (1ull << q->aq.order); i += n) q->data[i] = 0;
    if (gid < 2 * gcq::gwf::stat::COUNT && q->aq.stats) q->aq.stats[gid] = 0;
    if (gid == 0) *q->err = 0;
}

__global__ void k_init_glf(gcq::glf::mpmc* q) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t n = (uint64_t)gridDim.x * blockDim.x;
    gcq::glf::init_slice(&q->aq, false, gid, n);
    gcq::glf::init_slice(&q->fq, true, gid, n);
    if (gid == 0) *q->err = 0;
}

__global__ void k_init_sfq(gcq::sfq::queue* q) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t n = (uint64_t)gridDim.x * blockDim.x;
    gcq::sfq::init_slice(q, gid, n);
    if (gid == 0) *q->err = 0;
}

// YMC reset in two launches: clear the cells that can have been touched (all of
// them on creation, otherwise those below max(T, H) + 1), then the handles and
// counters.  The split keeps the reads of T and H ahead of their reset.
__global__ void k_clear_ymc(gcq::ymc::queue* q, int all) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t n = (uint64_t)gridDim.x * blockDim.x;
    uint64_t used = q->cap_cells;
    if (!all) {
        const uint64_t t = q->T, h = q->H;
        const uint64_t span = (t > h ? t : h) + 1;
        used = span < q->cap_cells ? span : q->cap_cells;
    }
    for (uint64_t i = gid; i < used; i += n) {
        gcq::ymc::cell* c = &q->cells[i];
        c->val = gcq::ymc::BOTTOM; c->enq = gcq::ymc::REQ_NULL; c->deq = gcq::ymc::REQ_NULL; c->_pad = 0;
    }
}
__global__ void k_init_ymc(gcq::ymc::queue* q) {
    const uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t n = (uint64_t)gridDim.x * blockDim.x;
    gcq::ymc::init_slice(q, 0, gid, n);
    if (gid == 0) *q->err = 0;
}

int thr_bits_for(uint32_t max_threads) {
    int b = 5;
    while ((((uint64_t)1 << b) - 1) < (uint64_t)max_threads) ++b;
    return b;
}

int launch_init(gcq_queue* q, cudaStream_t s, bool first) {
    const unsigned block = 256;
    switch (q->kind) {
        case GCQ_GWFQ: {
            const uint64_t work = std::max<uint64_t>(2ull << q->order, q->max_threads);
            k_init_gwf<<<gcqi::grid_for(work, block), block, 0, s>>>((gcq::gwf::mpmc*)q->obj);
            break;
        }
        case GCQ_GLFQ:
            k_init_glf<<<gcqi::grid_for(2ull << q->order, block), block, 0, s>>>((gcq::glf::mpmc*)q->obj);
            break;
        case GCQ_SFQ:
            k_init_sfq<<<gcqi::grid_for(1ull << q->order, block), block, 0, s>>>((gcq::sfq::queue*)q->obj);
            break;
        case GCQ_WFQ:
            k_clear_ymc<<<gcqi::grid_for(q->ymc_cells, block, 152u * 64u), block, 0, s>>>(
                (gcq::ymc::queue*)q->obj, first ? 1 : 0);
            k_init_ymc<<<gcqi::grid_for(q->max_threads, block), block, 0, s>>>((gcq::ymc::queue*)q->obj);
            break;
        default:
            return GCQ_EINVAL;
    }
    GCQ_CUDA(cudaGetLastError());
    return GCQ_OK;
}

}  // namespace

namespace gcqi {
int cuda_fail(cudaError_t e, const char* what, const char* file, int line) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    char buf[512];
    snprintf(buf, sizeof buf, "%s:%d %s: %s", file, line, what, cudaGetErrorString(e));
    g_last_cuda = buf;
    return GCQ_ECUDA;
}
int resident_threads(const void* kernel, int block, size_t smem, uint64_t* out) {
    int dev = 0, sms = 0, per_sm = 0;
    GCQ_CUDA(cudaGetDevice(&dev));
    GCQ_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    GCQ_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem));
    *out = (uint64_t)per_sm * (uint64_t)sms * (uint64_t)block;
    return GCQ_OK;
}
}  // namespace gcqi

extern "C" {

void gcq_default_knobs(gcq_knobs* k) {
    if (!k) return;
    k->help_delay = WF_HELP_DELAY;
    k->enq_patience = WF_ENQ_PATIENCE;
    k->deq_patience = WF_DEQ_PATIENCE;
    k->remap = REMAP_AUTO;
    k->ymc_patience = WF_PATIENCE;
    k->ymc_ops_per_thread = WF_PREALLOC_OPS_PER_THREAD;
    k->wait_timeout_ns = 2000000000ull;
    k->deq_wait = 8;
    k->_pad = 0;
}

const char* gcq_strerror(int s) {
    switch (s) {
        case GCQ_OK: return "ok";
        case GCQ_EINVAL: return "invalid argument";
        case GCQ_ENOMEM: return "out of memory";
        case GCQ_ECUDA: return "CUDA runtime error";
        case GCQ_ETIMEDOUT: return "bounded device wait timed out";
        case GCQ_EDEVICE: return "queue device error word set";
        case GCQ_EUNSUPPORTED: return "configuration outside the algorithm's envelope";
        case GCQ_ECAPACITY: return "input does not fit the queue";
        default: return "unknown status";
    }
}

const char* gcq_last_cuda_error(void) {
    std::lock_guard<std::mutex> lk(g_err_mu);
    static thread_local std::string copy;
    copy = g_last_cuda;
    return copy.c_str();
}

int gcq_create(int kind, uint32_t capacity_log2, uint32_t max_threads, const gcq_knobs* knobs,
               gcq_queue** out) {
    if (!out) return GCQ_EINVAL;
    *out = nullptr;
    gcq_knobs k;
    if (knobs) k = *knobs; else gcq_default_knobs(&k);
    if (max_threads == 0) return GCQ_EINVAL;
    if (kind != GCQ_WFQ && (capacity_log2 < 1 || capacity_log2 > 30)) return GCQ_EINVAL;
    // the SCQ rings keep Threshold = 3N - 1 in an int (gwf_queue.hpp:313-323,
    // glf_queue.hpp:127-138): N = 2^30 would overflow it
    if ((kind == GCQ_GWFQ || kind == GCQ_GLFQ) && capacity_log2 > 29) return GCQ_EINVAL;
    // Identity slot mapping for both rings.  The reference's G-LFQ spreads
    // consecutive tickets over 128-B lines (glf_queue.hpp:116-120), against false
    // sharing between AMD wavefronts; with warp-aggregated tickets a warp's 32
    // consecutive slots share two lines and its CASes coalesce in L2 instead
    // (balanced G-LFQ, 262144 threads: 22.1 Gops/s spread, 60.8 identity).
    if (k.remap == REMAP_AUTO) k.remap = 0u;

    gcq_queue* q = new (std::nothrow) gcq_queue();
    if (!q) return GCQ_ENOMEM;
    q->kind = kind;
    q->order = capacity_log2;
    q->max_threads = max_threads;
    q->knobs = k;

    const uint64_t A = 256;
    uint64_t off = 0;
    cudaError_t hdr_rc = cudaSuccess;
    auto take = [&](uint64_t bytes) { uint64_t at = align_up(off, A); off = at + bytes; return at; };

    switch (kind) {
        case GCQ_GWFQ: {
            const uint64_t n = 1ull << capacity_log2;
            const int bits = thr_bits_for(max_threads);
            // envelope of gwf_queue.hpp:55-61 and :319-323
            if (bits > 20 || 64 - bits < 44 || max_threads > n ||
                !(gcq::gwf::CYCLE_RANGE > 2ull * ((uint64_t)k.help_delay * max_threads / (2 * n) + 3)) ||
                k.help_delay == 0 || k.enq_patience < 2 || k.deq_patience < 2) {
                delete q;
                return GCQ_EUNSUPPORTED;
            }
            const uint64_t o_hdr = take(sizeof(gcq::gwf::mpmc));
            const uint64_t o_err = take(4);
            const uint64_t o_ae = take(2 * n * 8), o_fe = take(2 * n * 8);
            const uint64_t o_ar = take((uint64_t)max_threads * sizeof(gcq::gwf::record));
            const uint64_t o_fr = take((uint64_t)max_threads * sizeof(gcq::gwf::record));
            const uint64_t o_ah = take((uint64_t)max_threads * sizeof(gcq::gwf::helper_state));
            const uint64_t o_fh = take((uint64_t)max_threads * sizeof(gcq::gwf::helper_state));
            const uint64_t o_d = take(n * 8);
            const uint64_t o_ao = take(2 * n * 4), o_fo = take(2 * n * 4);
            const uint64_t o_st = take(2 * gcq::gwf::stat::COUNT * 8);
            q->bytes = align_up(off, A);
            if (cudaMalloc(&q->base, q->bytes) != cudaSuccess) { delete q; return GCQ_ENOMEM; }
            char* b = (char*)q->base;
            gcq::gwf::mpmc h;
            memset(&h, 0, sizeof h);
            auto fill = [&](gcq::gwf::ring& r, uint64_t oe, uint64_t orr, uint64_t oh, uint64_t oo) {
                r.Entry = (gcq::u64a*)(b + oe);
                r.Owner = (gcq::u32a*)(b + oo);
                r.Record = (gcq::gwf::record*)(b + orr);
                r.Help = (gcq::gwf::helper_state*)(b + oh);
                r.err = (gcq::u32a*)(b + o_err);
                r.order = capacity_log2;
                r.thr_bits = (uint32_t)bits;
                r.max_threads = max_threads;
                r.help_delay = k.help_delay;
                r.enq_patience = k.enq_patience;
                r.deq_patience = k.deq_patience;
                r.remap = k.remap ? 1u : 0u;
                r.deq_wait = k.deq_wait;
            };
            fill(h.aq, o_ae, o_ar, o_ah, o_ao);
            fill(h.fq, o_fe, o_fr, o_fh, o_fo);
            h.aq.stats = (gcq::u64a*)(b + o_st);
            h.fq.stats = h.aq.stats + gcq::gwf::stat::COUNT;
            q->stats = h.aq.stats;
            h.data = (gcq::u64a*)(b + o_d);
            h.err = (gcq::u32a*)(b + o_err);
            q->obj = b + o_hdr;
            q->err = (gcq::u32a*)(b + o_err);
            hdr_rc = cudaMemcpy(q->obj, &h, sizeof h, cudaMemcpyHostToDevice);
            break;
        }
        case GCQ_GLFQ: {
            const uint64_t n = 1ull << capacity_log2;
            const uint64_t o_hdr = take(sizeof(gcq::glf::mpmc));
            const uint64_t o_err = take(4);
            const uint64_t o_ae = take(2 * n * 8), o_fe = take(2 * n * 8);
            const uint64_t o_d = take(n * 8);
            q->bytes = align_up(off, A);
            if (cudaMalloc(&q->base, q->bytes) != cudaSuccess) { delete q; return GCQ_ENOMEM; }
            char* b = (char*)q->base;
            gcq::glf::mpmc h;
            memset(&h, 0, sizeof h);
            const uint32_t line_log2 = k.remap ? 4u : 0u;   // 16 entries per 128-B line
            h.aq.Entry = (gcq::u64a*)(b + o_ae);
            h.fq.Entry = (gcq::u64a*)(b + o_fe);
            h.aq.err = h.fq.err = h.err = (gcq::u32a*)(b + o_err);
            h.aq.order = h.fq.order = capacity_log2;
            h.aq.line_log2 = h.fq.line_log2 = line_log2;
            h.aq.deq_wait = h.fq.deq_wait = k.deq_wait;
            h.data = (gcq::u64a*)(b + o_d);
            q->obj = b + o_hdr;
            q->err = (gcq::u32a*)(b + o_err);
            hdr_rc = cudaMemcpy(q->obj, &h, sizeof h, cudaMemcpyHostToDevice);
            break;
        }
        case GCQ_WFQ: {
            if (k.ymc_ops_per_thread == 0) { delete q; return GCQ_EINVAL; }
            // pool sizing of wf_queue_host_init_ex, wfqueue_hip_opt.hpp:595-599
            const uint64_t per = 3ull * k.ymc_ops_per_thread + 128;
            uint64_t segs = ((uint64_t)max_threads * per + WF_SEGMENT_SIZE - 1) / WF_SEGMENT_SIZE + WF_SEGMENT_SAFETY;
            if (segs < 2) segs = 2;
            q->ymc_cells = segs * WF_SEGMENT_SIZE;
            const uint64_t o_hdr = take(sizeof(gcq::ymc::queue));
            const uint64_t o_err = take(4);
            const uint64_t o_c = take(q->ymc_cells * sizeof(gcq::ymc::cell));
            const uint64_t o_h = take((uint64_t)max_threads * sizeof(gcq::ymc::handle));
            q->bytes = align_up(off, A);
            if (cudaMalloc(&q->base, q->bytes) != cudaSuccess) { delete q; return GCQ_ENOMEM; }
            char* b = (char*)q->base;
            gcq::ymc::queue h;
            memset(&h, 0, sizeof h);
            h.cells = (gcq::ymc::cell*)(b + o_c);
            h.handles = (gcq::ymc::handle*)(b + o_h);
            h.err = (gcq::u32a*)(b + o_err);
            h.cap_cells = q->ymc_cells;
            h.nhandles = max_threads;
            h.patience = k.ymc_patience;
            q->obj = b + o_hdr;
            q->err = (gcq::u32a*)(b + o_err);
            hdr_rc = cudaMemcpy(q->obj, &h, sizeof h, cudaMemcpyHostToDevice);
            break;
        }
        case GCQ_SFQ: {
            const uint64_t len = 1ull << capacity_log2;
            const uint64_t max_id = 2ull * ((0xFFFFFFFFull / len) + 1);   // sfqueue_hip.hpp:39
            // envelope of sfqueue_hip.hpp:45-51
            if (max_id < 2ull * ((uint64_t)max_threads + 1) || len + max_threads >= 0x80000000ull) {
                delete q;
                return GCQ_EUNSUPPORTED;
            }
            const uint64_t o_hdr = take(sizeof(gcq::sfq::queue));
            const uint64_t o_err = take(4);
            const uint64_t o_s = take(len * 8);
            q->bytes = align_up(off, A);
            if (cudaMalloc(&q->base, q->bytes) != cudaSuccess) { delete q; return GCQ_ENOMEM; }
            char* b = (char*)q->base;
            gcq::sfq::queue h;
            memset(&h, 0, sizeof h);
            h.slot = (gcq::u64a*)(b + o_s);
            h.err = (gcq::u32a*)(b + o_err);
            h.log2_len = capacity_log2;
            h.max_id = (uint32_t)max_id;
            h.timeout_ns = k.wait_timeout_ns;
            h.nprocs = max_threads;
            q->obj = b + o_hdr;
            q->err = (gcq::u32a*)(b + o_err);
            hdr_rc = cudaMemcpy(q->obj, &h, sizeof h, cudaMemcpyHostToDevice);
            break;
        }
        default:
            delete q;
            return GCQ_EINVAL;
    }
    int rc = (hdr_rc == cudaSuccess) ? launch_init(q, 0, true)
                                     : gcqi::cuda_fail(hdr_rc, "header copy", __FILE__, __LINE__);
    if (rc == GCQ_OK) {
        cudaError_t e = cudaDeviceSynchronize();
        if (e != cudaSuccess) rc = gcqi::cuda_fail(e, "init", __FILE__, __LINE__);
    }
    if (rc != GCQ_OK) {
        cudaFree(q->base);
        delete q;
        return rc;
    }
    *out = q;
    return GCQ_OK;
}

int gcq_destroy(gcq_queue* q) {
    if (!q) return GCQ_EINVAL;
    cudaError_t e = cudaFree(q->base);
    delete q;
    return e == cudaSuccess ? GCQ_OK : gcqi::cuda_fail(e, "cudaFree", __FILE__, __LINE__);
}

int gcq_reset(gcq_queue* q, void* stream) {
    if (!q) return GCQ_EINVAL;
    return launch_init(q, gcqi::as_stream(stream), false);
}

int gcq_device_info(char* name, int name_cap, int* sms) {
    int dev = 0;
    GCQ_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    GCQ_CUDA(cudaGetDeviceProperties(&prop, dev));
    if (name && name_cap > 0) {
        strncpy(name, prop.name, (size_t)name_cap - 1);
        name[name_cap - 1] = '\0';
    }
    if (sms) *sms = prop.multiProcessorCount;
    return GCQ_OK;
}

int gcq_device_ptr(gcq_queue* q, void** dev) {
    if (!q || !dev) return GCQ_EINVAL;
    *dev = q->obj;
    return GCQ_OK;
}

int gcq_error_word(gcq_queue* q, uint32_t* err, int clear) {
    if (!q || !err) return GCQ_EINVAL;
    GCQ_CUDA(cudaDeviceSynchronize());
    GCQ_CUDA(cudaMemcpy(err, q->err, 4, cudaMemcpyDeviceToHost));
    if (clear) GCQ_CUDA(cudaMemset(q->err, 0, 4));
    return GCQ_OK;
}

uint64_t gcq_device_bytes(const gcq_queue* q) { return q ? q->bytes : 0; }

int gcq_stats(gcq_queue* q, uint64_t* out, int clear) {
    if (!q || !out) return GCQ_EINVAL;
    memset(out, 0, 16 * sizeof(uint64_t));
    if (q->kind != GCQ_GWFQ || !q->stats) return GCQ_OK;
    GCQ_CUDA(cudaDeviceSynchronize());
    GCQ_CUDA(cudaMemcpy(out, q->stats, 16 * sizeof(uint64_t), cudaMemcpyDeviceToHost));
    if (clear) GCQ_CUDA(cudaMemset(q->stats, 0, 16 * sizeof(uint64_t)));
    return GCQ_OK;
}

int gcq_info(const gcq_queue* q, int* kind, uint32_t* capacity_log2, uint32_t* max_threads) {
    if (!q) return GCQ_EINVAL;
    if (kind) *kind = q->kind;
    if (capacity_log2) *capacity_log2 = q->order;
    if (max_threads) *max_threads = q->max_threads;
    return GCQ_OK;
}

}  // extern "C"
