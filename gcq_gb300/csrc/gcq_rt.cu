// Persistent wavefront ray tracer with one queue per tile (concurrent_rt/rt_final.cpp):
// k_generate writes every tile's primary rays and enqueues their pixel indices;
// k_trace is one persistent launch in which each tile's threads dequeue rays, trace
// them against the scene, accumulate colour with float atomicAdd and re-enqueue the
// reflection ray until the tile's alive count reaches zero.
//
// This translation unit is compiled with --fmad=false: every a*b+c stays two
// rounded operations, so with IEEE sqrtf and division the image equals a serial CPU
// render that performs the same float operations in the same order.  A pixel's
// contributions are added in bounce order (each bounce accumulates before it
// re-enqueues the next), so the float sums are deterministic too.
#include <chrono>
#include <cstring>
#include <type_traits>
#include <vector>

#include "gcq_scene.cuh"

namespace {

// rt_final.cpp:350-366
struct Sphere { V3 c; float r; V3 albedo; float refl; };
struct Plane { V3 n; float d; V3 albedo; float refl; };
struct Ray { V3 o, d; int px, py, depth; V3 atten; };   // 48 bytes, as the reference's Ray
struct Hit { float t; V3 n, p, albedo; float refl; bool did_hit; };

// intersect_sphere / intersect_plane / trace_scene, rt_final.cpp:371-419
__device__ __forceinline__ Hit hit_sphere(const Ray& ray, const Sphere& s) {
    Hit h; h.did_hit = false; h.t = 1e30f;
    const V3 oc = sub(ray.o, s.c);
    const float b = dot3(oc, ray.d);
    const float c = dot3(oc, oc) - s.r * s.r;
    const float disc = b * b - c;
    if (disc >= 0.f) {
        const float t = -b - sqrtf(disc);
        if (t > 1e-4f) {
            h.t = t; h.did_hit = true;
            h.p = add(ray.o, scale(ray.d, t));
            h.n = normalize(sub(h.p, s.c));
            h.albedo = s.albedo;
            h.refl = s.refl;
        }
    }
    return h;
}
__device__ __forceinline__ Hit hit_plane(const Ray& ray, const Plane& pl) {
    Hit h; h.did_hit = false; h.t = 1e30f;
    const float denom = dot3(pl.n, ray.d);
    if (fabsf(denom) > 1e-5f) {
        const float t = -(dot3(pl.n, ray.o) + pl.d) / denom;
        if (t > 1e-4f) {
            h.t = t; h.did_hit = true;
            h.p = add(ray.o, scale(ray.d, t));
            h.n = pl.n;
            h.albedo = pl.albedo;
            h.refl = pl.refl;
        }
    }
    return h;
}
__device__ __forceinline__ Hit trace_scene(const Ray& ray, const Sphere* sph, int ns, const Plane* pln, int np) {
    Hit best; best.did_hit = false; best.t = 1e30f;
    for (int i = 0; i < ns; i++) {
        const Hit h = hit_sphere(ray, sph[i]);
        if (h.did_hit && h.t < best.t) best = h;
    }
    for (int i = 0; i < np; i++) {
        const Hit h = hit_plane(ray, pln[i]);
        if (h.did_hit && h.t < best.t) best = h;
    }
    return best;
}

__device__ __forceinline__ void accum_pixel(float* img, int w, int x, int y, V3 c) {
    float* p = img + 3 * (size_t)(y * w + x);
    atomicAdd(p + 0, c.x);
    atomicAdd(p + 1, c.y);
    atomicAdd(p + 2, c.z);
}

// ---------------------------------------------------------------- per-tile queues
// Raw index rings as the reference uses them (rt_final.cpp:53-298): G-WFQ wf_t,
// G-LFQ fq_ring_t, SFQ with the index shifted by one (0 is reserved).
struct tile_queues {
    int kind;
    void* rings;          // array of gwf::ring / glf::ring / sfq::queue, one per tile
    size_t stride;        // bytes between consecutive ring headers
};

template <int K> struct rtq;
// maybe(q): a read-only hint that the ring may hold an entry (its Tail counter is
// ahead of Head).  Idle G-LFQ and SFQ tracer threads poll through it, so an empty
// ring costs them two loads instead of Head tickets per poll (5x faster traces on
// the 512-sphere scene with G-LFQ).  G-WFQ needs none: its dequeue returns on the
// first load once the Threshold is negative, and timing showed the hint no faster
// and less steady there.
// G-WFQ tracer threads use the lock-free fast path on both sides: a thousand
// pollers per ring keep the wait-free slow path from finishing promptly (its
// tickets come one CAS at a time while pollers take Head tickets), and about one
// render in ten of the 512-sphere scene took 33-36 ms instead of 3.4 once an
// enqueue went slow.  With fast-path retries the trace is steady at 2.8 ms.
template <> struct rtq<GCQ_GWFQ> {
    using R = gcq::gwf::ring;
    __device__ static bool maybe(const R*) { return true; }
    __device__ static bool enq(R* q, uint32_t idx, uint32_t) {
        const gcq::gwf::cfg c = gcq::gwf::load_cfg(q);
        for (uint32_t k = 0; k < GCQ_SPIN_LIMIT; ++k)
            if (gcq::gwf::try_enq(q, c, idx) == 0) return true;   // release CAS publishes the ray
        gcq::raise_error(c.err, gcq::ERR_SPIN);
        return false;
    }
    __device__ static bool deq(R* q, uint32_t* out, uint32_t tid) {
        *out = gcq::gwf::try_dequeue(q, tid, 2);
        return *out != gcq::gwf::BOT;
    }
};
template <> struct rtq<GCQ_GLFQ> {
    using R = gcq::glf::ring;
    __device__ static bool maybe(const R* q) { return gcq::ld_rlx(&q->Tail) > gcq::ld_rlx(&q->Head); }
    __device__ static bool enq(R* q, uint32_t idx, uint32_t) { return gcq::glf::enqueue(q, idx); }
    __device__ static bool deq(R* q, uint32_t* out, uint32_t) {
        *out = gcq::glf::dequeue(q);
        return *out != gcq::glf::BOT;
    }
};
// YMC (the reference's USE_WFQ tracer, rt_final.cpp:141-170): a per-tile wf_queue
// with one handle per tile thread, ray indices stored + 1 (0 is WF_BOTTOM).
// Consumers poll with ymc::try_dequeue, which takes H tickets only below T, so the
// per-tile cell pool holds one cell per enqueue and the image is exact; the
// reference's consumers poll with wf_dequeue, whose failed polls each use up a cell.
template <> struct rtq<GCQ_WFQ> {
    using R = gcq::ymc::queue;
    __device__ static bool maybe(const R* q) { return gcq::ld_rlx(&q->T) > gcq::ld_rlx(&q->H); }
    __device__ static bool enq(R* q, uint32_t idx, uint32_t tid) { return gcq::ymc::enqueue(q, tid, (uint64_t)idx + 1); }
    __device__ static bool deq(R* q, uint32_t* out, uint32_t) {
        uint64_t v = 0;
        if (!gcq::ymc::try_dequeue(q, &v)) return false;
        *out = (uint32_t)(v - 1);
        return true;
    }
};
template <> struct rtq<GCQ_SFQ> {
    using R = gcq::sfq::queue;
    __device__ static bool maybe(const R* q) {
        return (int32_t)(gcq::ld_rlx(&q->tail) - gcq::ld_rlx(&q->head)) > 0;
    }
    __device__ static bool enq(R* q, uint32_t idx, uint32_t) { return gcq::sfq::enqueue_blocking(q, idx + 1u) == SFQ_SUCCESS; }
    __device__ static bool deq(R* q, uint32_t* out, uint32_t) {
        uint32_t item = 0;
        if (gcq::sfq::dequeue_nb(q, &item) != SFQ_SUCCESS) return false;
        *out = item - 1u;
        return true;
    }
};

struct rt_params {
    int img_w, img_h, tiles_x, tile_w, tile_h, threads_per_tile, max_depth;
    V3 cam_o, cam_f, cam_r, cam_u;
    uint64_t timeout_ns;
};

// k_generate, rt_final.cpp:435-511
template <int K>
__global__ void k_generate(char* rings, size_t stride, Ray* __restrict__ rays, rt_params P,
                           unsigned long long* __restrict__ alive) {
    const int tile = (int)blockIdx.y;
    const int tid = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (tid >= P.threads_per_tile) return;
    auto* q = reinterpret_cast<typename rtq<K>::R*>(rings + (size_t)tile * stride);
    const int tx = tile % P.tiles_x, ty = tile / P.tiles_x;
    const int x0 = tx * P.tile_w, y0 = ty * P.tile_h;
    const int tw = min(P.tile_w, P.img_w - x0), th = min(P.tile_h, P.img_h - y0);
    const int tile_pixels = tw * th;
    const float aspect = (float)P.img_w / (float)P.img_h;
    int enqueued = 0;
    for (int i = tid; i < tile_pixels; i += P.threads_per_tile) {
        const int lx = i % tw, ly = i / tw;
        const int px = x0 + lx, py = y0 + ly;
        const float u = ((px + 0.5f) / P.img_w - 0.5f) * 2.f * aspect;
        const float v = -((py + 0.5f) / P.img_h - 0.5f) * 2.f;
        Ray r;
        r.o = P.cam_o;
        r.d = normalize(add(add(P.cam_f, scale(P.cam_r, u)), scale(P.cam_u, v)));
        r.px = px; r.py = py;
        r.depth = 0;
        r.atten = v3(1.f, 1.f, 1.f);
        rays[py * P.img_w + px] = r;
        // the queue's release CAS publishes the ray written above
        if (rtq<K>::enq(q, (uint32_t)i, (uint32_t)tid)) ++enqueued;
    }
    if (enqueued > 0) atomicAdd(&alive[tile], (unsigned long long)enqueued);
}

// k_trace, rt_final.cpp:516-645.  The wait for in-flight rays is bounded: with no
// progress for timeout_ns the thread records ERR_TIMEOUT and leaves.
template <int K>
__global__ void k_trace(char* rings, size_t stride, const Sphere* __restrict__ sph, int ns,
                        const Plane* __restrict__ pln, int np, Ray* __restrict__ rays, float* __restrict__ img,
                        rt_params P, unsigned long long* __restrict__ alive, unsigned long long* __restrict__ traced,
                        gcq::u32a* err) {
    const int tile = (int)blockIdx.y;
    const int tid = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (tid >= P.threads_per_tile) return;
    auto* q = reinterpret_cast<typename rtq<K>::R*>(rings + (size_t)tile * stride);
    const int tx = tile % P.tiles_x, ty = tile / P.tiles_x;
    const int x0 = tx * P.tile_w, y0 = ty * P.tile_h;
    const int tw = min(P.tile_w, P.img_w - x0);
    const V3 light_dir = normalize(v3(-0.5f, 1.f, 0.2f));
    const V3 ambient = v3(0.05f, 0.05f, 0.05f);
    unsigned long long local_traced = 0;
    gcq::backoff bo;
    uint64_t last_progress = gcq::globaltimer_ns();
    for (uint32_t it = 0;; ++it) {
        if (gcq::ld_rlx((const gcq::u64a*)&alive[tile]) == 0) break;
        uint32_t local_idx;
        if (!rtq<K>::maybe(q) || !rtq<K>::deq(q, &local_idx, (uint32_t)tid)) {
            if ((it & 63) == 0 && gcq::globaltimer_ns() - last_progress > P.timeout_ns) {
                gcq::raise_error(err, gcq::ERR_TIMEOUT);
                break;
            }
            bo.pause(1024);
            continue;
        }
        bo = gcq::backoff();
        last_progress = gcq::globaltimer_ns();
        const int lx = (int)local_idx % tw, ly = (int)local_idx / tw;
        const int gidx = (y0 + ly) * P.img_w + (x0 + lx);
        const Ray r = rays[gidx];
        const Hit hit = trace_scene(r, sph, ns, pln, np);
        if (hit.did_hit) {
            const float NdotL = fmaxf(0.f, dot3(hit.n, light_dir));
            const V3 direct = add(ambient, scale(hit.albedo, NdotL));
            const V3 contrib = mulv(direct, r.atten);
            if (hit.refl > 0.f && r.depth < P.max_depth) {
                const V3 non_refl = clamp01(scale(contrib, 1.f - hit.refl));
                if (non_refl.x > 0.f || non_refl.y > 0.f || non_refl.z > 0.f)
                    accum_pixel(img, P.img_w, r.px, r.py, non_refl);
                Ray refl;
                refl.o = add(hit.p, scale(hit.n, 1e-4f));
                refl.d = normalize(reflect3(r.d, hit.n));
                refl.px = r.px; refl.py = r.py;
                refl.depth = r.depth + 1;
                refl.atten = scale(mulv(r.atten, hit.albedo), hit.refl);
                rays[gidx] = refl;
                if (!rtq<K>::enq(q, local_idx, (uint32_t)tid)) atomicAdd(&alive[tile], (unsigned long long)(-1LL));
            } else {
                accum_pixel(img, P.img_w, r.px, r.py, clamp01(contrib));
                atomicAdd(&alive[tile], (unsigned long long)(-1LL));
            }
        } else {
            const float t = 0.5f * (r.d.y + 1.f);
            const V3 sky = add(scale(v3(1.f, 1.f, 1.f), 1.f - t), scale(v3(0.5f, 0.7f, 1.f), t));
            accum_pixel(img, P.img_w, r.px, r.py, clamp01(mulv(sky, r.atten)));
            atomicAdd(&alive[tile], (unsigned long long)(-1LL));
        }
        ++local_traced;
    }
    if (local_traced > 0) atomicAdd(&traced[tile], local_traced);
}

// Per-tile ring initialisation (the reference's k_init_queue, rt_final.cpp:84-139).
__global__ void k_init_tiles_gwf(char* rings, size_t stride, int tiles) {
    for (int t = blockIdx.y; t < tiles; t += gridDim.y)
        gcq::gwf::init_slice((gcq::gwf::ring*)(rings + (size_t)t * stride), false,
                             (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, (uint64_t)gridDim.x * blockDim.x);
}
__global__ void k_init_tiles_glf(char* rings, size_t stride, int tiles) {
    for (int t = blockIdx.y; t < tiles; t += gridDim.y)
        gcq::glf::init_slice((gcq::glf::ring*)(rings + (size_t)t * stride), false,
                             (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, (uint64_t)gridDim.x * blockDim.x);
}
__global__ void k_init_tiles_sfq(char* rings, size_t stride, int tiles);
__global__ void k_init_tiles_ymc(char* rings, size_t stride, int tiles) {
    for (int t = blockIdx.y; t < tiles; t += gridDim.y) {
        gcq::ymc::queue* q = (gcq::ymc::queue*)(rings + (size_t)t * stride);
        gcq::ymc::init_slice(q, q->cap_cells, (uint64_t)blockIdx.x * blockDim.x + threadIdx.x,
                             (uint64_t)gridDim.x * blockDim.x);
    }
}
// Launch f(integral_constant<int, kind>) for the queue kind of a tracer.
template <typename F>
void rt_dispatch(int kind, F&& f) {
    switch (kind) {
        case GCQ_GWFQ: f(std::integral_constant<int, GCQ_GWFQ>()); break;
        case GCQ_GLFQ: f(std::integral_constant<int, GCQ_GLFQ>()); break;
        case GCQ_WFQ: f(std::integral_constant<int, GCQ_WFQ>()); break;
        default: f(std::integral_constant<int, GCQ_SFQ>()); break;
    }
}
void init_tiles(int kind, char* rings, size_t stride, int tiles, dim3 grid) {
    if (kind == GCQ_GWFQ) k_init_tiles_gwf<<<grid, 256>>>(rings, stride, tiles);
    else if (kind == GCQ_GLFQ) k_init_tiles_glf<<<grid, 256>>>(rings, stride, tiles);
    else if (kind == GCQ_WFQ) k_init_tiles_ymc<<<grid, 256>>>(rings, stride, tiles);
    else k_init_tiles_sfq<<<grid, 256>>>(rings, stride, tiles);
}
__global__ void k_init_tiles_sfq(char* rings, size_t stride, int tiles) {
    for (int t = blockIdx.y; t < tiles; t += gridDim.y)
        gcq::sfq::init_slice((gcq::sfq::queue*)(rings + (size_t)t * stride),
                             (uint64_t)blockIdx.x * blockDim.x + threadIdx.x, (uint64_t)gridDim.x * blockDim.x);
}

// Scenes of rt_final.cpp:650-684 and cameras of :849-859.
void build_scene(int scene, std::vector<Sphere>& sph, std::vector<Plane>& pln, rt_params& P) {
    if (scene == 0) {
        pln.push_back({v3(0, 1, 0), 1.f, v3(0.75f, 0.75f, 0.75f), 0.05f});
        const int gx = 10, gz = 10;
        const float sp = 0.55f, rad = 0.22f, base_y = 0.25f;
        for (int iz = 0; iz < gz; iz++)
            for (int ix = 0; ix < gx; ix++) {
                const float x = (ix - (gx - 1) * 0.5f) * sp;
                const float z = -2.f - iz * sp;
                const int m = (ix + iz * 7) % 7;
                const float r = (m == 0) ? 0.9f : (m == 1) ? 0.6f : (m == 2) ? 0.3f : (m == 3) ? 0.1f : 0.f;
                const V3 a = (m == 0) ? v3(.9f, .9f, .9f) : (m == 1) ? v3(.9f, .5f, .2f)
                           : (m == 2) ? v3(.2f, .8f, .9f) : (m == 3) ? v3(.7f, .2f, .8f)
                           : (m == 4) ? v3(.2f, .9f, .3f) : (m == 5) ? v3(.9f, .2f, .2f) : v3(.8f, .8f, .3f);
                sph.push_back({v3(x, base_y, z), rad, a, r});
            }
        sph.push_back({v3(-1.2f, 0.6f, -3.5f), 0.6f, v3(.9f, .3f, .3f), 0.7f});
        sph.push_back({v3(1.4f, 0.9f, -4.2f), 0.9f, v3(.3f, .9f, .4f), 0.2f});
        sph.push_back({v3(0.0f, 1.3f, -5.5f), 1.3f, v3(.4f, .6f, .95f), 0.0f});
        P.cam_o = v3(0, 0.3f, 0.5f);
        P.cam_f = normalize(v3(0, -0.2f, -1.f));
    } else if (scene == 2) {
        // the compaction baseline's "mirror tunnel" (rt_compaction.cpp:554-592, camera
        // :705-707): mirror walls, matte absorbers, a chain of near-perfect mirrors
        for (const Plane& p : {Plane{v3(1, 0, 0), 2.0f, v3(.95f, .95f, .95f), 0.985f},
                               Plane{v3(-1, 0, 0), 2.0f, v3(.95f, .95f, .95f), 0.985f},
                               Plane{v3(0, 1, 0), 1.2f, v3(.95f, .95f, .95f), 0.985f},
                               Plane{v3(0, -1, 0), 1.2f, v3(.95f, .95f, .95f), 0.985f},
                               Plane{v3(0, 0, 1), 20.0f, v3(.95f, .95f, .95f), 0.985f},
                               Plane{v3(0, 0, -1), 2.5f, v3(.95f, .95f, .95f), 0.985f}})
            pln.push_back(p);
        for (const Sphere& q : {Sphere{v3(-1.45f, -0.25f, -4.2f), 0.70f, v3(.85f, .20f, .20f), 0.00f},
                                Sphere{v3(1.35f, 0.20f, -5.3f), 0.80f, v3(.20f, .85f, .25f), 0.00f},
                                Sphere{v3(0.00f, -0.75f, -8.5f), 0.40f, v3(.85f, .85f, .20f), 0.00f},
                                Sphere{v3(0.00f, 0.00f, -4.8f), 0.90f, v3(.95f, .95f, .95f), 0.995f},
                                Sphere{v3(-0.75f, 0.35f, -7.2f), 0.85f, v3(.95f, .85f, .85f), 0.995f},
                                Sphere{v3(0.80f, -0.25f, -9.8f), 0.90f, v3(.85f, .95f, .85f), 0.995f},
                                Sphere{v3(-0.55f, 0.30f, -12.2f), 0.95f, v3(.85f, .85f, .95f), 0.995f},
                                Sphere{v3(0.70f, -0.20f, -14.7f), 1.00f, v3(.95f, .95f, .80f), 0.995f},
                                Sphere{v3(0.00f, 0.10f, -17.2f), 1.05f, v3(.90f, .90f, .95f), 0.995f}})
            sph.push_back(q);
        P.cam_o = v3(0.0f, 0.0f, 1.6f);
        P.cam_f = normalize(v3(0.0f, 0.0f, -1.0f));
    } else {
        sph.push_back({v3(-0.6f, 0.5f, -2.5f), 0.5f, v3(.9f, .3f, .3f), 0.85f});
        sph.push_back({v3(0.6f, 0.6f, -2.8f), 0.6f, v3(.95f, .95f, .95f), 0.95f});
        pln.push_back({v3(0, 1, 0), 1.f, v3(.9f, .9f, .9f), 0.3f});
        pln.push_back({v3(0, 0, 1), 5.f, v3(.6f, .65f, .8f), 0.7f});
        pln.push_back({v3(1, 0, 0), 2.f, v3(.8f, .2f, .2f), 0.6f});
        pln.push_back({v3(-1, 0, 0), 2.f, v3(.2f, .8f, .3f), 0.6f});
        pln.push_back({v3(0, -1, 0), 2.5f, v3(.95f, .95f, .95f), 0.2f});
        P.cam_o = v3(0, 0.5f, 1.5f);
        P.cam_f = normalize(v3(0, -0.1f, -1.f));
    }
    P.cam_r = normalize(v3(1, 0, 0));
    P.cam_u = normalize(v3(0, 1, 0));
}



// Path tracing of the benchmark scenes (scene code in gcq_scene.cuh) over the
// per-tile queues.  blockIdx.y = j, the position in a list of tiles (tile = list[j],
// or j without a list); ring j serves it and its rays and path states live at
// [j * tile pixels, +tile pixels).
__device__ __forceinline__ int btile(const int32_t* list, int j) { return list ? list[j] : j; }

// primary rays of a tile into its queue (as k_generate)
template <int K>
__global__ void k_bgen(char* rings, size_t stride, const int32_t* __restrict__ list, BRay* __restrict__ rays,
                       BPix* __restrict__ pix, bparams P, unsigned long long* __restrict__ alive) {
    const int j = (int)blockIdx.y;
    const int tid = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (tid >= P.threads_per_tile) return;
    auto* q = reinterpret_cast<typename rtq<K>::R*>(rings + (size_t)j * stride);
    const int tile = btile(list, j);
    const int x0 = (tile % P.tiles_x) * P.tile_w, y0 = (tile / P.tiles_x) * P.tile_h;
    const int tw = min(P.tile_w, P.img_w - x0), th = min(P.tile_h, P.img_h - y0);
    const size_t base = (size_t)j * P.tile_w * P.tile_h;
    int enqueued = 0;
    for (int i = tid; i < tw * th; i += P.threads_per_tile) {
        const int px = x0 + i % tw, py = y0 + i / tw;
        BRay r;
        BPix st;
        bprimary(P, px, py, (uint32_t)(py * P.img_w + px), &r, &st);
        rays[base + i] = r;
        pix[base + i] = st;
        if (rtq<K>::enq(q, (uint32_t)i, (uint32_t)tid)) ++enqueued;   // release publishes the ray
    }
    if (enqueued > 0) atomicAdd(&alive[j], (unsigned long long)enqueued);
}

template <int K>
__global__ void k_btrace(char* rings, size_t stride, const int32_t* __restrict__ list,
                         const BSphere* __restrict__ sph, int ns, const BQuad* __restrict__ quad, int nq,
                         BRay* __restrict__ rays, BPix* __restrict__ pix, float* __restrict__ img, bparams P,
                         unsigned long long* __restrict__ alive, unsigned long long* __restrict__ traced,
                         gcq::u32a* err) {
    // sphere centres and radii staged in shared memory (16 bytes a sphere, 8 KB for
    // the 512-sphere scene), read by every lane at the same index: broadcast loads
    extern __shared__ float4 s_cr[];
    for (int i = (int)threadIdx.x; i < ns; i += (int)blockDim.x) s_cr[i] = sphere_cr(sph[i]);
    __syncthreads();
    const int j = (int)blockIdx.y;
    const int tid = (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (tid >= P.threads_per_tile) return;
    auto* q = reinterpret_cast<typename rtq<K>::R*>(rings + (size_t)j * stride);
    const size_t base = (size_t)j * P.tile_w * P.tile_h;
    unsigned long long local_traced = 0;
    gcq::backoff bo;
    uint64_t last_progress = gcq::globaltimer_ns();
    for (uint32_t it = 0;; ++it) {
        if (gcq::ld_rlx((const gcq::u64a*)&alive[j]) == 0) break;
        uint32_t li;
        if (!rtq<K>::maybe(q) || !rtq<K>::deq(q, &li, (uint32_t)tid)) {
            if ((it & 63) == 0 && gcq::globaltimer_ns() - last_progress > P.timeout_ns) {
                gcq::raise_error(err, gcq::ERR_TIMEOUT);
                break;
            }
            bo.pause(1024);
            continue;
        }
        bo = gcq::backoff();
        last_progress = gcq::globaltimer_ns();
        BRay r = rays[base + li];
        BPix st = pix[base + li];
        const BHit hit = btrace_with(r, [](int i) { return s_cr[i]; }, sph, ns, quad, nq);
        ++local_traced;
        V3 c;
        if (bshade(r, st, hit, P, &c)) {
            rays[base + li] = r;
            pix[base + li] = st;
            if (!rtq<K>::enq(q, li, (uint32_t)tid)) atomicAdd(&alive[j], (unsigned long long)(-1LL));
        } else {
            float* o = img + 3 * (size_t)r.pix;
            o[0] = c.x; o[1] = c.y; o[2] = c.z;
            atomicAdd(&alive[j], (unsigned long long)(-1LL));
        }
    }
    if (local_traced > 0) atomicAdd(&traced[j], local_traced);
}

// ---------------------------------------------------------------- per-tile rings
// One allocation holding a ring header per tile (stride apart) and each tile's
// arrays, initialised for kind with threads_per_tile thread indices: the reference
// allocates and initialises one queue per tile (rt_final.cpp:794-833).
struct tile_rings {
    char* dq = nullptr;
    size_t stride = 0;
    gcq::u32a* err = nullptr;
};

void free_tile_rings(tile_rings* tr) {
    cudaFree(tr->dq);
    tr->dq = nullptr;
}

// ymc_cells: the cell pool of a YMC tile queue, one cell per enqueue of the tile's
// rays (its pixels x (bounces + 1)) with a margin; other kinds ignore it.
int make_tile_rings(int kind, int tiles, int threads_per_tile, uint32_t queue_log2, uint64_t timeout_ns,
                    tile_rings* tr, uint64_t ymc_cells = 0) {
    const uint64_t n = 1ull << queue_log2;
    size_t stride = 0, per_tile = 0;
    int bits = 5;
    if (kind == GCQ_WFQ) {
        if (ymc_cells == 0) return GCQ_EINVAL;
        stride = sizeof(gcq::ymc::queue);
        per_tile = (size_t)threads_per_tile * sizeof(gcq::ymc::handle) + ymc_cells * sizeof(gcq::ymc::cell);
    } else if (kind == GCQ_GWFQ) {
        if ((uint64_t)threads_per_tile > n) return GCQ_EUNSUPPORTED;
        while ((((uint64_t)1 << bits) - 1) < (uint64_t)threads_per_tile) ++bits;
        stride = sizeof(gcq::gwf::ring);
        // entries (256-B aligned), records (128 B each), help countdowns (8 B), owners
        per_tile = ((2 * n * 8 + 255) / 256 * 256) + (size_t)threads_per_tile * (sizeof(gcq::gwf::record) + 8) +
                   2 * n * 4;
    } else if (kind == GCQ_GLFQ) {
        stride = sizeof(gcq::glf::ring);
        per_tile = 2 * n * 8;
    } else {
        const uint64_t max_id = 2ull * ((0xFFFFFFFFull / n) + 1);
        if (max_id < 2ull * ((uint64_t)threads_per_tile + 1)) return GCQ_EUNSUPPORTED;
        stride = sizeof(gcq::sfq::queue);
        per_tile = n * 8;
    }
    auto a256 = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t hdr_bytes = a256(stride * tiles);
    const size_t tile_bytes = a256(per_tile);
    char* dq = nullptr;
    if (cudaMalloc(&dq, hdr_bytes + tile_bytes * tiles + 256) != cudaSuccess) {
        cudaGetLastError();
        return GCQ_ENOMEM;
    }
    gcq::u32a* d_err = (gcq::u32a*)(dq + hdr_bytes + tile_bytes * tiles);
    std::vector<char> hh(hdr_bytes, 0);
    for (int t = 0; t < tiles; ++t) {
        char* tb = dq + hdr_bytes + tile_bytes * t;
        if (kind == GCQ_GWFQ) {
            gcq::gwf::ring r;
            memset(&r, 0, sizeof r);
            r.Entry = (gcq::u64a*)tb;
            r.Record = (gcq::gwf::record*)(tb + a256(2 * n * 8));
            r.Help = (gcq::gwf::helper_state*)((char*)r.Record + (size_t)threads_per_tile * sizeof(gcq::gwf::record));
            r.Owner = (gcq::u32a*)((char*)r.Help + (size_t)threads_per_tile * 8);
            r.err = d_err;
            r.order = queue_log2;
            r.thr_bits = (uint32_t)bits;
            r.max_threads = (uint32_t)threads_per_tile;
            r.help_delay = WF_HELP_DELAY;
            r.enq_patience = WF_ENQ_PATIENCE;
            r.deq_patience = WF_DEQ_PATIENCE;
            r.remap = 0;
            r.deq_wait = 0;
            r.stats = nullptr;
            memcpy(&hh[t * stride], &r, sizeof r);
        } else if (kind == GCQ_WFQ) {
            gcq::ymc::queue r;
            memset(&r, 0, sizeof r);
            r.handles = (gcq::ymc::handle*)tb;
            r.cells = (gcq::ymc::cell*)(tb + (size_t)threads_per_tile * sizeof(gcq::ymc::handle));
            r.err = d_err;
            r.cap_cells = ymc_cells;
            r.nhandles = (uint32_t)threads_per_tile;
            r.patience = WF_PATIENCE;
            memcpy(&hh[t * stride], &r, sizeof r);
        } else if (kind == GCQ_GLFQ) {
            gcq::glf::ring r;
            memset(&r, 0, sizeof r);
            r.Entry = (gcq::u64a*)tb;
            r.err = d_err;
            r.order = queue_log2;
            r.line_log2 = 3;   // the reference's 64-byte remap (glf_queue.hpp:50-51)
            r.deq_wait = 0;
            memcpy(&hh[t * stride], &r, sizeof r);
        } else {
            gcq::sfq::queue r;
            memset(&r, 0, sizeof r);
            r.slot = (gcq::u64a*)tb;
            r.err = d_err;
            r.log2_len = queue_log2;
            r.max_id = (uint32_t)(2ull * ((0xFFFFFFFFull / n) + 1));
            r.timeout_ns = timeout_ns;
            r.nprocs = (uint32_t)threads_per_tile;
            memcpy(&hh[t * stride], &r, sizeof r);
        }
    }
    cudaError_t e = cudaMemcpy(dq, hh.data(), hdr_bytes, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d_err, 0, 4);
    if (e == cudaSuccess) {
        const uint64_t work = kind == GCQ_WFQ ? ymc_cells : 2 * n;
        const dim3 ig((unsigned)std::min<uint64_t>(64, (work + 255) / 256), (unsigned)std::min(tiles, 1024));
        init_tiles(kind, dq, stride, tiles, ig);
        e = cudaGetLastError();
        if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    if (e != cudaSuccess) {
        cudaFree(dq);
        return gcqi::cuda_fail(e, "tile rings", __FILE__, __LINE__);
    }
    tr->dq = dq;
    tr->stride = stride;
    tr->err = d_err;
    return GCQ_OK;
}

// ------------------------------------------------ stream-compaction comparator
// The double-buffer + stream-compaction renderer of concurrent_rt/baselines/
// rt_compaction.cpp, the non-queue baseline: every pass traces the whole active
// ray list, marks the rays that continue, and packs them in order (the reference's
// Blelloch scan + scatter, :327-470) for the next pass.  Here a pass is three
// launches with the counts kept on the device: the trace writes each warp's
// continuation ballot and each block's count, one block scans the block counts,
// and the scatter places each continuing ray at its block offset + warp prefix +
// lane rank -- the same order an exclusive scan of the flags gives.
struct CRay { V3 o, d; int pix, depth; };   // 32 bytes

__global__ void k_cgen(CRay* __restrict__ rays, rt_params P) {
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= P.img_w * P.img_h) return;
    const int px = idx % P.img_w, py = idx / P.img_w;
    const float aspect = (float)P.img_w / (float)P.img_h;
    const float u = ((px + 0.5f) / P.img_w - 0.5f) * 2.f * aspect;
    const float v = -((py + 0.5f) / P.img_h - 0.5f) * 2.f;
    CRay r;
    r.o = P.cam_o;
    r.d = normalize(add(P.cam_f, add(scale(P.cam_r, u), scale(P.cam_u, v))));   // :240-241
    r.pix = idx;
    r.depth = 0;
    rays[idx] = r;
}

// kernel_trace_rays, rt_compaction.cpp:258-326, plus the flags and block counts
__global__ void __launch_bounds__(256) k_ctrace(const CRay* __restrict__ in, const uint32_t* __restrict__ count,
                                                CRay* __restrict__ tmp, uint32_t* __restrict__ masks,
                                                uint32_t* __restrict__ block_cnt, const Sphere* __restrict__ sph,
                                                int ns, const Plane* __restrict__ pln, int np,
                                                float* __restrict__ img, int max_depth) {
    const uint32_t n = *count;
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    bool cont = false;
    if (idx < n) {
        const CRay r = in[idx];
        const V3 light_dir = normalize(v3(-0.5f, 1.f, 0.2f));
        const V3 ambient = v3(0.05f, 0.05f, 0.05f);
        Ray q;
        q.o = r.o;
        q.d = r.d;
        const Hit hit = trace_scene(q, sph, ns, pln, np);
        V3 color;
        if (hit.did_hit) {
            const float NdotL = fmaxf(0.f, dot3(hit.n, light_dir));
            color = add(ambient, scale(hit.albedo, NdotL));
            if (hit.refl > 0.f && r.depth < max_depth) {
                CRay o;
                o.o = add(hit.p, scale(hit.n, 1e-4f));
                o.d = normalize(reflect3(r.d, hit.n));
                o.pix = r.pix;
                o.depth = r.depth + 1;
                tmp[idx] = o;
                cont = true;
            }
        } else {
            const float t = 0.5f * (r.d.y + 1.f);
            color = add(scale(v3(1.f, 1.f, 1.f), 1.f - t), scale(v3(0.5f, 0.7f, 1.f), t));
        }
        color = scale(clamp01(color), r.depth == 0 ? 1.0f : 0.5f);
        float* p = img + 3 * (size_t)r.pix;
        // one ray per pixel per pass: the reference's atomicAdd is a plain add here
        if (r.depth == 0) { p[0] = color.x; p[1] = color.y; p[2] = color.z; }
        else { p[0] += color.x; p[1] += color.y; p[2] += color.z; }
    }
    const unsigned m = __ballot_sync(0xffffffffu, cont);
    if ((threadIdx.x & 31) == 0) masks[idx >> 5] = m;
    const int c = __syncthreads_count(cont);
    if (threadIdx.x == 0) block_cnt[blockIdx.x] = (uint32_t)c;
}

// exclusive scan of the block counts in one block of 1024 threads; the total is
// the next pass's ray count
__global__ void __launch_bounds__(1024) k_cscan(const uint32_t* __restrict__ block_cnt, uint32_t nblocks,
                                                uint32_t* __restrict__ block_off, uint32_t* __restrict__ total,
                                                unsigned long long* __restrict__ traced, const uint32_t* __restrict__ count) {
    __shared__ uint32_t warp_sum[32];
    const uint32_t per = (nblocks + blockDim.x - 1) / blockDim.x;
    const uint32_t b0 = threadIdx.x * per;
    uint32_t mine = 0;
    for (uint32_t b = b0; b < b0 + per && b < nblocks; ++b) mine += block_cnt[b];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = mine;   // inclusive warp scan
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_sum[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_sum[lane] = w;
    }
    __syncthreads();
    uint32_t run = (x - mine) + (warp > 0 ? warp_sum[warp - 1] : 0u);
    for (uint32_t b = b0; b < b0 + per && b < nblocks; ++b) {
        block_off[b] = run;
        run += block_cnt[b];
    }
    if (threadIdx.x == blockDim.x - 1) {
        *total = run;
        atomicAdd(traced, (unsigned long long)*count);
    }
}

__global__ void __launch_bounds__(256) k_cscatter(const CRay* __restrict__ tmp, const uint32_t* __restrict__ masks,
                                                  const uint32_t* __restrict__ block_off, const uint32_t* __restrict__ count,
                                                  CRay* __restrict__ out) {
    __shared__ uint32_t wpre[8];
    const uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t m = idx < *count ? masks[idx >> 5] : 0u;
    if (lane == 0) wpre[warp] = (uint32_t)__popc(m);
    __syncthreads();
    uint32_t base = block_off[blockIdx.x];
    for (int w = 0; w < warp; ++w) base += wpre[w];
    if ((m >> lane) & 1u) out[base + (uint32_t)__popc(m & ((1u << lane) - 1u))] = tmp[idx];
}

}  // namespace

struct gcq_rt_ctx {
    int kind = 0, tiles = 0, max_tiles = 0, ns = 0, nq = 0;
    bool fresh = false;      // rings initialised and unused
    bparams P;
    tile_rings tr;
    BRay* rays = nullptr;
    BPix* pix = nullptr;
    float* img = nullptr;
    unsigned long long* cnt = nullptr;   // alive[max_tiles], traced[max_tiles]
    int32_t* list = nullptr;
    BSphere* sph = nullptr;
    BQuad* quad = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
    ~gcq_rt_ctx() {
        free_tile_rings(&tr);
        cudaFree(rays); cudaFree(pix); cudaFree(img); cudaFree(cnt); cudaFree(list); cudaFree(sph); cudaFree(quad);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (e2) cudaEventDestroy(e2);
    }
};

extern "C" {

// Render one frame (rt_final.cpp:705-1018).  kind: any of the four queues.  image
// receives width*height RGB float pixels (may be NULL).
int gcq_rt_render(int kind, int scene, int width, int height, int tiles_x, int tiles_y, int threads_per_tile,
                  int max_bounces, uint32_t queue_log2, float* image, gcq_rt_result* out) {
    if (!out || width <= 0 || height <= 0 || tiles_x <= 0 || tiles_y <= 0 || threads_per_tile <= 0 ||
        max_bounces < 0 || scene < 0 || scene > 2 || queue_log2 < 4 || queue_log2 > 24)
        return GCQ_EINVAL;
    if (kind != GCQ_GWFQ && kind != GCQ_GLFQ && kind != GCQ_WFQ && kind != GCQ_SFQ) return GCQ_EUNSUPPORTED;
    memset(out, 0, sizeof(*out));
    const int tiles = tiles_x * tiles_y;
    rt_params P;
    memset(&P, 0, sizeof P);
    P.img_w = width; P.img_h = height; P.tiles_x = tiles_x;
    P.tile_w = (width + tiles_x - 1) / tiles_x;
    P.tile_h = (height + tiles_y - 1) / tiles_y;
    P.threads_per_tile = threads_per_tile;
    P.max_depth = max_bounces;
    P.timeout_ns = 5000000000ull;
    const uint64_t tile_px = (uint64_t)P.tile_w * P.tile_h;
    const uint64_t n = 1ull << queue_log2;
    if (tile_px > n) return GCQ_ECAPACITY;   // a tile's rays must fit its queue
    std::vector<Sphere> sph;
    std::vector<Plane> pln;
    build_scene(scene, sph, pln, P);

    tile_rings tr;
    int rc = make_tile_rings(kind, tiles, threads_per_tile, queue_log2, P.timeout_ns, &tr,
                             tile_px * ((uint64_t)max_bounces + 1) + 1024);
    if (rc != GCQ_OK) return rc;
    char* dq = tr.dq;
    const size_t stride = tr.stride;
    gcq::u32a* d_err = tr.err;
    const size_t ray_bytes = (size_t)width * height * sizeof(Ray);
    const size_t img_bytes = (size_t)width * height * 3 * sizeof(float);
    Ray* d_rays = nullptr;
    float* d_img = nullptr;
    unsigned long long* d_cnt = nullptr;   // alive[tiles], traced[tiles]
    Sphere* d_sph = nullptr;
    Plane* d_pln = nullptr;
    auto cleanup = [&]() { free_tile_rings(&tr); cudaFree(d_rays); cudaFree(d_img); cudaFree(d_cnt); cudaFree(d_sph); cudaFree(d_pln); };
    if (cudaMalloc(&d_rays, ray_bytes) != cudaSuccess || cudaMalloc(&d_img, img_bytes) != cudaSuccess ||
        cudaMalloc(&d_cnt, 2 * tiles * 8) != cudaSuccess ||
        cudaMalloc(&d_sph, std::max<size_t>(1, sph.size()) * sizeof(Sphere)) != cudaSuccess ||
        cudaMalloc(&d_pln, std::max<size_t>(1, pln.size()) * sizeof(Plane)) != cudaSuccess) {
        cudaGetLastError();
        cleanup();
        return GCQ_ENOMEM;
    }
    GCQ_CUDA(cudaMemset(d_img, 0, img_bytes));
    GCQ_CUDA(cudaMemset(d_cnt, 0, 2 * tiles * 8));
    if (!sph.empty()) GCQ_CUDA(cudaMemcpy(d_sph, sph.data(), sph.size() * sizeof(Sphere), cudaMemcpyHostToDevice));
    if (!pln.empty()) GCQ_CUDA(cudaMemcpy(d_pln, pln.data(), pln.size() * sizeof(Plane), cudaMemcpyHostToDevice));
    const int TPB = 256;
    const dim3 grid((unsigned)((threads_per_tile + TPB - 1) / TPB), (unsigned)tiles);
    cudaEvent_t e0, e1, e2;
    cudaEventCreate(&e0); cudaEventCreate(&e1); cudaEventCreate(&e2);
    unsigned long long* d_alive = d_cnt;
    unsigned long long* d_traced = d_cnt + tiles;
    const int ns = (int)sph.size(), np = (int)pln.size();
    cudaEventRecord(e0);
    rt_dispatch(kind, [&](auto kc) {
        constexpr int K = decltype(kc)::value;
        k_generate<K><<<grid, TPB>>>(dq, stride, d_rays, P, d_alive);
        cudaEventRecord(e1);
        k_trace<K><<<grid, TPB>>>(dq, stride, d_sph, ns, d_pln, np, d_rays, d_img, P, d_alive, d_traced, d_err);
    });
    cudaEventRecord(e2);
    cudaError_t ke = cudaEventSynchronize(e2);
    if (ke == cudaSuccess) ke = cudaGetLastError();
    if (ke != cudaSuccess) {
        cleanup();
        return gcqi::cuda_fail(ke, "rt kernels", __FILE__, __LINE__);
    }
    float gen_ms = 0, trace_ms = 0;
    cudaEventElapsedTime(&gen_ms, e0, e1);
    cudaEventElapsedTime(&trace_ms, e1, e2);
    cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2);
    std::vector<unsigned long long> cnt(2 * tiles);
    GCQ_CUDA(cudaMemcpy(cnt.data(), d_cnt, 2 * tiles * 8, cudaMemcpyDeviceToHost));
    uint32_t err = 0;
    GCQ_CUDA(cudaMemcpy(&err, d_err, 4, cudaMemcpyDeviceToHost));
    uint64_t leftover = 0, traced = 0;
    for (int t = 0; t < tiles; ++t) { leftover += cnt[t]; traced += cnt[tiles + t]; }
    out->gen_ms = gen_ms;
    out->trace_ms = trace_ms;
    out->total_ms = gen_ms + trace_ms;
    out->primary_rays = (uint64_t)width * height;
    out->total_rays = traced;
    out->leftover = leftover;
    if (image) GCQ_CUDA(cudaMemcpy(image, d_img, img_bytes, cudaMemcpyDeviceToHost));
    cleanup();
    if (err & GCQ_ERR_TIMEOUT) return GCQ_ETIMEDOUT;
    if (err & (GCQ_ERR_SPIN | GCQ_ERR_TID)) return GCQ_EDEVICE;
    if (err & GCQ_ERR_POOL) return GCQ_ECAPACITY;   // a YMC tile pool ran dry: rays were dropped
    return leftover ? GCQ_EDEVICE : GCQ_OK;
}

// Render one frame with the stream-compaction baseline (rt_compaction.cpp:593-897):
// scenes 0, 1 and 2, every pass's rays packed in order for the next.  gen_ms is the
// primary-ray launch, trace_ms the passes (trace + scan + scatter); total_rays sums
// the rays of every pass, as the reference counts them.
int gcq_rt_compact_render(int scene, int width, int height, int max_bounces, float* image, gcq_rt_result* out) {
    if (!out || width <= 0 || height <= 0 || max_bounces < 0 || max_bounces > 64 || scene < 0 || scene > 2 ||
        (uint64_t)width * height > (1u << 30))
        return GCQ_EINVAL;
    memset(out, 0, sizeof(*out));
    rt_params P;
    memset(&P, 0, sizeof P);
    P.img_w = width;
    P.img_h = height;
    std::vector<Sphere> sph;
    std::vector<Plane> pln;
    build_scene(scene, sph, pln, P);
    const uint32_t N = (uint32_t)width * height;
    const uint32_t nblocks = (N + 255) / 256;
    const int passes = max_bounces + 1;
    CRay *d_a = nullptr, *d_b = nullptr, *d_t = nullptr;
    uint32_t *d_masks = nullptr, *d_bcnt = nullptr, *d_boff = nullptr, *d_count = nullptr;
    unsigned long long* d_traced = nullptr;
    float* d_img = nullptr;
    Sphere* d_sph = nullptr;
    Plane* d_pln = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
    auto cleanup = [&]() {
        cudaFree(d_a); cudaFree(d_b); cudaFree(d_t); cudaFree(d_masks); cudaFree(d_bcnt); cudaFree(d_boff);
        cudaFree(d_count); cudaFree(d_traced); cudaFree(d_img); cudaFree(d_sph); cudaFree(d_pln);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        if (e2) cudaEventDestroy(e2);
    };
    const size_t rb = (size_t)N * sizeof(CRay);
    if (cudaMalloc(&d_a, rb) != cudaSuccess || cudaMalloc(&d_b, rb) != cudaSuccess || cudaMalloc(&d_t, rb) != cudaSuccess ||
        cudaMalloc(&d_masks, (size_t)nblocks * 8 * 4) != cudaSuccess ||
        cudaMalloc(&d_bcnt, (size_t)nblocks * 4) != cudaSuccess || cudaMalloc(&d_boff, (size_t)nblocks * 4) != cudaSuccess ||
        cudaMalloc(&d_count, (size_t)(passes + 1) * 4) != cudaSuccess || cudaMalloc(&d_traced, 8) != cudaSuccess ||
        cudaMalloc(&d_img, (size_t)N * 12) != cudaSuccess ||
        cudaMalloc(&d_sph, std::max<size_t>(1, sph.size()) * sizeof(Sphere)) != cudaSuccess ||
        cudaMalloc(&d_pln, std::max<size_t>(1, pln.size()) * sizeof(Plane)) != cudaSuccess) {
        cudaGetLastError();
        cleanup();
        return GCQ_ENOMEM;
    }
    auto fail = [&](cudaError_t e, const char* what) { cleanup(); return gcqi::cuda_fail(e, what, __FILE__, __LINE__); };
    std::vector<uint32_t> hc(passes + 1, 0);
    hc[0] = N;
    cudaError_t ce = cudaMemcpy(d_count, hc.data(), hc.size() * 4, cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaMemset(d_traced, 0, 8);
    if (ce == cudaSuccess) ce = cudaMemset(d_img, 0, (size_t)N * 12);
    if (ce == cudaSuccess && !sph.empty()) ce = cudaMemcpy(d_sph, sph.data(), sph.size() * sizeof(Sphere), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess && !pln.empty()) ce = cudaMemcpy(d_pln, pln.data(), pln.size() * sizeof(Plane), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e2);
    if (ce != cudaSuccess) return fail(ce, "rt compaction setup");
    cudaEventRecord(e0);
    k_cgen<<<nblocks, 256>>>(d_a, P);
    cudaEventRecord(e1);
    CRay* in = d_a;
    CRay* outb = d_b;
    for (int pass = 0; pass < passes; ++pass) {
        k_ctrace<<<nblocks, 256>>>(in, d_count + pass, d_t, d_masks, d_bcnt, d_sph, (int)sph.size(), d_pln,
                                   (int)pln.size(), d_img, max_bounces);
        k_cscan<<<1, 1024>>>(d_bcnt, nblocks, d_boff, d_count + pass + 1, d_traced, d_count + pass);
        if (pass + 1 < passes) k_cscatter<<<nblocks, 256>>>(d_t, d_masks, d_boff, d_count + pass, outb);
        std::swap(in, outb);
    }
    cudaEventRecord(e2);
    ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaEventSynchronize(e2);
    if (ce != cudaSuccess) return fail(ce, "rt compaction passes");
    float gen_ms = 0, trace_ms = 0;
    cudaEventElapsedTime(&gen_ms, e0, e1);
    cudaEventElapsedTime(&trace_ms, e1, e2);
    unsigned long long traced = 0;
    ce = cudaMemcpy(&traced, d_traced, 8, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess && image) ce = cudaMemcpy(image, d_img, (size_t)N * 12, cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return fail(ce, "rt compaction results");
    out->gen_ms = gen_ms;
    out->trace_ms = trace_ms;
    out->total_ms = gen_ms + trace_ms;
    out->primary_rays = N;
    out->total_rays = traced;
    out->leftover = 0;
    cleanup();
    return GCQ_OK;
}

// A render context for the benchmark scenes: scene, rings for up to max_tiles tiles
// at a time, ray and path storage for them and the image, all allocated once.
int gcq_rt_ctx_create(int kind, int scene, int width, int height, int tile_px, int threads_per_tile,
                      int max_bounces, uint32_t queue_log2, uint64_t seed, int max_tiles, gcq_rt_ctx** out) {
    if (!out) return GCQ_EINVAL;
    *out = nullptr;
    if (width <= 0 || height <= 0 || tile_px <= 0 || threads_per_tile <= 0 || max_bounces < 0 ||
        max_bounces > 1000 || scene < 0 || scene > 1 || queue_log2 < 4 || queue_log2 > 24 ||
        (int64_t)width * height > (1ll << 30))
        return GCQ_EINVAL;
    if (kind != GCQ_GWFQ && kind != GCQ_GLFQ && kind != GCQ_WFQ && kind != GCQ_SFQ) return GCQ_EUNSUPPORTED;
    if ((uint64_t)tile_px * tile_px > (1ull << queue_log2)) return GCQ_ECAPACITY;   // a tile must fit its queue
    gcq_rt_ctx* c = new gcq_rt_ctx();
    bparams& P = c->P;
    memset(&P, 0, sizeof P);
    P.img_w = width;
    P.img_h = height;
    P.tile_w = P.tile_h = tile_px;
    P.tiles_x = (width + tile_px - 1) / tile_px;
    c->tiles = P.tiles_x * ((height + tile_px - 1) / tile_px);
    c->max_tiles = (max_tiles <= 0 || max_tiles > c->tiles) ? c->tiles : max_tiles;
    P.threads_per_tile = threads_per_tile;
    P.max_depth = max_bounces;
    P.seed = seed;
    P.timeout_ns = 5000000000ull;
    c->kind = kind;
    std::vector<BSphere> sph;
    std::vector<BQuad> quad;
    build_bscene(scene, seed, sph, quad, P);
    c->ns = (int)sph.size();
    c->nq = (int)quad.size();
    int rc = make_tile_rings(kind, c->max_tiles, threads_per_tile, queue_log2, P.timeout_ns, &c->tr,
                             (uint64_t)tile_px * tile_px * ((uint64_t)max_bounces + 1) + 1024);
    if (rc != GCQ_OK) { delete c; return rc; }
    const size_t npx = (size_t)width * height, tpx = (size_t)tile_px * tile_px * c->max_tiles;
    if (cudaMalloc(&c->rays, tpx * sizeof(BRay)) != cudaSuccess || cudaMalloc(&c->pix, tpx * sizeof(BPix)) != cudaSuccess ||
        cudaMalloc(&c->img, npx * 12) != cudaSuccess || cudaMalloc(&c->cnt, 2 * (size_t)c->max_tiles * 8) != cudaSuccess ||
        cudaMalloc(&c->list, (size_t)c->max_tiles * 4) != cudaSuccess ||
        cudaMalloc(&c->sph, std::max<size_t>(1, sph.size()) * sizeof(BSphere)) != cudaSuccess ||
        cudaMalloc(&c->quad, std::max<size_t>(1, quad.size()) * sizeof(BQuad)) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return GCQ_ENOMEM;
    }
    cudaError_t ce = cudaMemset(c->img, 0, npx * 12);
    if (ce == cudaSuccess && !sph.empty()) ce = cudaMemcpy(c->sph, sph.data(), sph.size() * sizeof(BSphere), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess && !quad.empty()) ce = cudaMemcpy(c->quad, quad.data(), quad.size() * sizeof(BQuad), cudaMemcpyHostToDevice);
    if (ce == cudaSuccess) ce = cudaEventCreate(&c->e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&c->e1);
    if (ce == cudaSuccess) ce = cudaEventCreate(&c->e2);
    if (ce != cudaSuccess) {
        delete c;
        return gcqi::cuda_fail(ce, "rt context", __FILE__, __LINE__);
    }
    c->fresh = true;
    *out = c;
    return GCQ_OK;
}

int gcq_rt_ctx_destroy(gcq_rt_ctx* c) {
    if (!c) return GCQ_EINVAL;
    delete c;
    return GCQ_OK;
}

// Render the listed tiles (row-major tile indices; NULL: every tile, in order)
// into the context's image; image (may be NULL) receives the whole image.
int gcq_rt_ctx_render(gcq_rt_ctx* c, const int32_t* tiles, int ntiles, float* image, gcq_rt_result* out) {
    if (!c || !out || (tiles && (ntiles <= 0 || ntiles > c->max_tiles))) return GCQ_EINVAL;
    if (!tiles) {
        if (c->max_tiles < c->tiles) return GCQ_EINVAL;
        ntiles = c->tiles;
    }
    const bparams& P = c->P;
    uint64_t primary = 0;
    if (tiles) {
        for (int j = 0; j < ntiles; ++j) {
            if (tiles[j] < 0 || tiles[j] >= c->tiles) return GCQ_EINVAL;
            const int x0 = (tiles[j] % P.tiles_x) * P.tile_w, y0 = (tiles[j] / P.tiles_x) * P.tile_h;
            primary += (uint64_t)std::min(P.tile_w, P.img_w - x0) * (uint64_t)std::min(P.tile_h, P.img_h - y0);
        }
    } else {
        primary = (uint64_t)P.img_w * P.img_h;
    }
    memset(out, 0, sizeof(*out));
    cudaError_t ce = cudaSuccess;
    if (tiles) ce = cudaMemcpyAsync(c->list, tiles, (size_t)ntiles * 4, cudaMemcpyHostToDevice, 0);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(c->cnt, 0, 2 * (size_t)c->max_tiles * 8, 0);
    if (ce == cudaSuccess) ce = cudaMemsetAsync(c->tr.err, 0, 4, 0);
    if (ce != cudaSuccess) return gcqi::cuda_fail(ce, "rt render setup", __FILE__, __LINE__);
    const int kind = c->kind;
    if (!c->fresh) {   // re-initialise the rings this render uses
        init_tiles(kind, c->tr.dq, c->tr.stride, ntiles, dim3(64u, (unsigned)std::min(ntiles, 1024)));
    }
    c->fresh = false;
    const int TPB = 256;
    const dim3 grid((unsigned)((P.threads_per_tile + TPB - 1) / TPB), (unsigned)ntiles);
    const int32_t* dl = tiles ? c->list : nullptr;
    const size_t smem = sizeof(float4) * (size_t)std::max(c->ns, 1);
    unsigned long long* d_alive = c->cnt;
    unsigned long long* d_traced = c->cnt + c->max_tiles;
    cudaEventRecord(c->e0);
    rt_dispatch(kind, [&](auto kc) {
        constexpr int K = decltype(kc)::value;
        k_bgen<K><<<grid, TPB>>>(c->tr.dq, c->tr.stride, dl, c->rays, c->pix, P, d_alive);
        cudaEventRecord(c->e1);
        k_btrace<K><<<grid, TPB, smem>>>(c->tr.dq, c->tr.stride, dl, c->sph, c->ns, c->quad, c->nq, c->rays, c->pix,
                                         c->img, P, d_alive, d_traced, c->tr.err);
    });
    cudaEventRecord(c->e2);
    ce = cudaGetLastError();
    if (ce == cudaSuccess) ce = cudaEventSynchronize(c->e2);
    if (ce != cudaSuccess) return gcqi::cuda_fail(ce, "rt bounce kernels", __FILE__, __LINE__);
    float gen_ms = 0, trace_ms = 0;
    cudaEventElapsedTime(&gen_ms, c->e0, c->e1);
    cudaEventElapsedTime(&trace_ms, c->e1, c->e2);
    std::vector<unsigned long long> cnt(2 * (size_t)ntiles);
    uint32_t err = 0;
    ce = cudaMemcpy(cnt.data(), c->cnt, (size_t)ntiles * 8, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess) ce = cudaMemcpy(cnt.data() + ntiles, c->cnt + c->max_tiles, (size_t)ntiles * 8, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess) ce = cudaMemcpy(&err, c->tr.err, 4, cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess && image) ce = cudaMemcpy(image, c->img, (size_t)P.img_w * P.img_h * 12, cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return gcqi::cuda_fail(ce, "rt bounce results", __FILE__, __LINE__);
    uint64_t leftover = 0, traced = 0;
    for (int t = 0; t < ntiles; ++t) { leftover += cnt[t]; traced += cnt[ntiles + t]; }
    out->gen_ms = gen_ms;
    out->trace_ms = trace_ms;
    out->total_ms = gen_ms + trace_ms;
    out->primary_rays = primary;
    out->total_rays = traced;
    out->leftover = leftover;
    if (err & GCQ_ERR_TIMEOUT) return GCQ_ETIMEDOUT;
    if (err & (GCQ_ERR_SPIN | GCQ_ERR_TID)) return GCQ_EDEVICE;
    if (err & GCQ_ERR_POOL) return GCQ_ECAPACITY;   // a YMC tile pool ran dry: rays were dropped
    return leftover ? GCQ_EDEVICE : GCQ_OK;
}

// Render a whole benchmark scene in one call (a context over every tile).
int gcq_rt_bounce_render(int kind, int scene, int width, int height, int tile_px, int threads_per_tile,
                         int max_bounces, uint32_t queue_log2, uint64_t seed, float* image, gcq_rt_result* out) {
    if (!out) return GCQ_EINVAL;
    gcq_rt_ctx* c = nullptr;
    int rc = gcq_rt_ctx_create(kind, scene, width, height, tile_px, threads_per_tile, max_bounces, queue_log2, seed,
                               0, &c);
    if (rc != GCQ_OK) return rc;
    rc = gcq_rt_ctx_render(c, nullptr, 0, image, out);
    gcq_rt_ctx_destroy(c);
    return rc;
}

}  // extern "C"
