// Scene geometry and shading shared by the ray-tracing translation units (the
// per-tile queue renderer and the served engine).  Both are compiled with
// --fmad=false so that every a*b+c stays two rounded operations; with IEEE sqrtf
// and division the device performs exactly the float operations of the serial CPU
// restatement, in the same order.
#pragma once

#include <cstring>
#include <vector>

#include "gcq_internal.cuh"

namespace {

struct V3 { float x, y, z; };
__host__ __device__ __forceinline__ V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
__host__ __device__ __forceinline__ V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ V3 scale(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ V3 mulv(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__host__ __device__ __forceinline__ float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ V3 normalize(V3 v) {
    const float d = sqrtf(dot3(v, v));
    return d > 0.f ? scale(v, 1.f / d) : v;
}
__host__ __device__ __forceinline__ V3 reflect3(V3 v, V3 n) { return sub(v, scale(n, 2.f * dot3(v, n))); }
__host__ __device__ __forceinline__ V3 clamp01(V3 c) {
    return v3(fminf(fmaxf(c.x, 0.f), 1.f), fminf(fmaxf(c.y, 0.f), 1.f), fminf(fmaxf(c.z, 0.f), 1.f));
}

// ------------------------------------------------ benchmark scenes, 1 sample/pixel
// The ray-tracing workload of the benchmark configuration (the reference has no
// such scenes; its two scenes are above): 1024x1024 pixels in 32x32-pixel tiles,
// one sample per pixel, 32-byte rays (origin, direction, pixel id, depth) in the
// per-tile ray-bounce queues.  Scene 0: 512 seeded spheres (60 % diffuse, 30 % metal,
// 10 % glass) over a 40 x 40 ground quad under a sky.  Scene 1: a box room of five
// diffuse quads, two axis-aligned boxes and an emitting ceiling quad.  A path
// scatters per material (Lambertian, fuzzy metal, glass with Schlick reflectance)
// until it leaves the scene, reaches the light, is absorbed or uses up max_bounces;
// a pixel's one path contributes once, so the image needs no float atomics.
// Sampling uses no transcendental function (PCG integers, rejection sampling,
// Schlick as products), so the render is bit-identical to its CPU restatement.
struct BRay { V3 o, d; uint32_t pix, depth; };   // 32 bytes
struct BPix { V3 tp; uint32_t rng; };            // path throughput and RNG state, per pixel
enum { B_DIFFUSE = 0, B_METAL = 1, B_GLASS = 2, B_LIGHT = 3 };
struct BSphere { V3 c; float r; V3 albedo; float param; int mat; int _p[3]; };   // param: fuzz or index
struct BQuad { int axis; float k, a0, a1, b0, b1; V3 albedo; int mat; };          // axis-aligned rectangle
struct BCam { V3 o, lower_left, horiz, vert; };
struct BHit { float t; V3 p, n; V3 albedo; float param; int mat; bool front, did_hit; };
struct bparams {
    int img_w, img_h, tiles_x, tile_w, tile_h, threads_per_tile, max_depth, sky;
    BCam cam;
    uint64_t seed, timeout_ns;
};

__host__ __device__ __forceinline__ float comp(V3 v, int i) { return i == 0 ? v.x : i == 1 ? v.y : v.z; }
__host__ __device__ __forceinline__ uint32_t pcg_next(uint32_t& s) {
    s = s * 747796405u + 2891336453u;
    const uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
}
__host__ __device__ __forceinline__ float rand01(uint32_t& s) { return (float)(pcg_next(s) >> 8) * (1.0f / 16777216.0f); }
__device__ __forceinline__ V3 rand_in_unit_sphere(uint32_t& s) {
    for (int k = 0; k < 64; ++k) {
        const float x = 2.f * rand01(s) - 1.f;
        const float y = 2.f * rand01(s) - 1.f;
        const float z = 2.f * rand01(s) - 1.f;
        const V3 p = v3(x, y, z);
        if (dot3(p, p) < 1.f) return p;
    }
    return v3(0.f, 0.f, 0.f);
}

// Closest hit in two passes: the loops find the nearest root (sphere centre and
// radius as a float4, read through `cr`, which may be shared memory) and the
// nearest quad, keeping only (t, index); the hit record is then built once for the
// winner.  The roots, the comparisons and the record are the same float operations
// as a loop that builds a record for every closer hit, so the result is too.
__device__ __forceinline__ bool sphere_root(const BRay& r, float a, float4 s, float tmax, float* root_out) {
    const V3 oc = sub(r.o, v3(s.x, s.y, s.z));
    const float half_b = dot3(oc, r.d);
    const float c = dot3(oc, oc) - s.w * s.w;
    const float disc = half_b * half_b - a * c;
    if (disc < 0.f) return false;
    const float sq = sqrtf(disc);
    float root = (-half_b - sq) / a;
    if (root <= 1e-3f || root >= tmax) {
        root = (-half_b + sq) / a;
        if (root <= 1e-3f || root >= tmax) return false;
    }
    *root_out = root;
    return true;
}
__device__ __forceinline__ bool quad_t(const BRay& r, const BQuad& q, float tmax, float* t_out) {
    const float da = comp(r.d, q.axis);
    if (fabsf(da) < 1e-8f) return false;
    const float t = (q.k - comp(r.o, q.axis)) / da;
    if (t <= 1e-3f || t >= tmax) return false;
    const V3 p = add(r.o, scale(r.d, t));
    const float u = q.axis == 0 ? p.y : p.x;
    const float w = q.axis == 2 ? p.y : p.z;
    if (u < q.a0 || u > q.a1 || w < q.b0 || w > q.b1) return false;
    *t_out = t;
    return true;
}
__device__ __forceinline__ float4 sphere_cr(const BSphere& sp) { return make_float4(sp.c.x, sp.c.y, sp.c.z, sp.r); }

template <typename CR>
__device__ __forceinline__ BHit btrace_with(const BRay& r, CR cr, const BSphere* sph, int ns, const BQuad* quad, int nq) {
    const float a = dot3(r.d, r.d);
    float best_t = 1e30f;
    int best = -1;
#pragma unroll 4
    for (int i = 0; i < ns; ++i) {
        float root;
        if (sphere_root(r, a, cr(i), best_t, &root)) {
            best_t = root;
            best = i;
        }
    }
    int best_q = -1;
    for (int i = 0; i < nq; ++i) {
        float t;
        if (quad_t(r, quad[i], best_t, &t)) {
            best_t = t;
            best_q = i;
        }
    }
    BHit h;
    h.t = best_t;
    h.did_hit = (best_q >= 0 || best >= 0);
    if (best_q >= 0) {
        const BQuad& q = quad[best_q];
        h.p = add(r.o, scale(r.d, best_t));
        const V3 outward = v3(q.axis == 0 ? 1.f : 0.f, q.axis == 1 ? 1.f : 0.f, q.axis == 2 ? 1.f : 0.f);
        h.front = comp(r.d, q.axis) < 0.f;
        h.n = h.front ? outward : scale(outward, -1.f);
        h.albedo = q.albedo;
        h.param = 0.f;
        h.mat = q.mat;
    } else if (best >= 0) {
        const BSphere& sp = sph[best];
        h.p = add(r.o, scale(r.d, best_t));
        const V3 outward = scale(sub(h.p, sp.c), 1.f / sp.r);
        h.front = dot3(r.d, outward) < 0.f;
        h.n = h.front ? outward : scale(outward, -1.f);
        h.albedo = sp.albedo;
        h.param = sp.param;
        h.mat = sp.mat;
    }
    return h;
}
__device__ __forceinline__ BHit btrace(const BRay& r, const BSphere* sph, int ns, const BQuad* quad, int nq) {
    return btrace_with(r, [sph](int i) { return sphere_cr(sph[i]); }, sph, ns, quad, nq);
}

// One bounce of a path: true with r and st updated when the path continues; false
// with *contrib set when it ends.
__device__ __forceinline__ bool bshade(BRay& r, BPix& st, const BHit& hit, const bparams& P, V3* contrib) {
    if (!hit.did_hit) {
        if (P.sky) {
            const V3 unit = normalize(r.d);
            const float t = 0.5f * (unit.y + 1.f);
            const V3 sky = add(scale(v3(1.f, 1.f, 1.f), 1.f - t), scale(v3(0.5f, 0.7f, 1.f), t));
            *contrib = mulv(st.tp, sky);
        } else {
            *contrib = v3(0.f, 0.f, 0.f);
        }
        return false;
    }
    if (hit.mat == B_LIGHT) {
        *contrib = mulv(st.tp, hit.albedo);
        return false;
    }
    if ((int)r.depth >= P.max_depth) {
        *contrib = v3(0.f, 0.f, 0.f);
        return false;
    }
    V3 dir;
    V3 att = hit.albedo;
    if (hit.mat == B_DIFFUSE) {
        dir = add(hit.n, normalize(rand_in_unit_sphere(st.rng)));
        if (fabsf(dir.x) < 1e-8f && fabsf(dir.y) < 1e-8f && fabsf(dir.z) < 1e-8f) dir = hit.n;
    } else if (hit.mat == B_METAL) {
        const V3 refl = reflect3(normalize(r.d), hit.n);
        dir = add(refl, scale(rand_in_unit_sphere(st.rng), hit.param));
        if (dot3(dir, hit.n) <= 0.f) {
            *contrib = v3(0.f, 0.f, 0.f);
            return false;
        }
    } else {
        const float ratio = hit.front ? 1.f / hit.param : hit.param;
        const V3 unit = normalize(r.d);
        const float cos_t = fminf(dot3(scale(unit, -1.f), hit.n), 1.f);
        const float sin_t = sqrtf(1.f - cos_t * cos_t);
        float r0 = (1.f - ratio) / (1.f + ratio);
        r0 = r0 * r0;
        const float x = 1.f - cos_t;
        const float schlick = r0 + (1.f - r0) * (x * x * x * x * x);
        const float u = rand01(st.rng);
        if (ratio * sin_t > 1.f || schlick > u) {
            dir = reflect3(unit, hit.n);
        } else {
            const V3 perp = scale(add(unit, scale(hit.n, cos_t)), ratio);
            const V3 par = scale(hit.n, -sqrtf(fabsf(1.f - dot3(perp, perp))));
            dir = add(perp, par);
        }
        att = v3(1.f, 1.f, 1.f);
    }
    r.o = hit.p;
    r.d = normalize(dir);
    r.depth += 1;
    st.tp = mulv(st.tp, att);
    return true;
}

// Primary ray and path state of pixel (px, py), g = py * width + px.
__device__ __forceinline__ void bprimary(const bparams& P, int px, int py, uint32_t g, BRay* r, BPix* st) {
    const float s = ((float)px + 0.5f) / (float)P.img_w;
    const float t = 1.0f - ((float)py + 0.5f) / (float)P.img_h;
    r->o = P.cam.o;
    r->d = normalize(sub(add(add(P.cam.lower_left, scale(P.cam.horiz, s)), scale(P.cam.vert, t)), P.cam.o));
    r->pix = g;
    r->depth = 0;
    st->tp = v3(1.f, 1.f, 1.f);
    st->rng = (uint32_t)gcqi::splitmix64(P.seed ^ ((uint64_t)g << 20)) | 1u;
}

uint64_t bscene_rand(uint64_t& s) {
    s += 0x9e3779b97f4a7c15ULL;
    return gcqi::splitmix64(s - 0x9e3779b97f4a7c15ULL);
}
float bscene_u01(uint64_t& s) { return (float)(bscene_rand(s) >> 40) * (1.0f / 16777216.0f); }

BCam make_bcam(V3 from, V3 at, float half_h, float aspect) {
    const V3 w = normalize(sub(from, at));
    const V3 vup = v3(0.f, 1.f, 0.f);
    const V3 u = normalize(v3(vup.y * w.z - vup.z * w.y, vup.z * w.x - vup.x * w.z, vup.x * w.y - vup.y * w.x));
    const V3 v = v3(w.y * u.z - w.z * u.y, w.z * u.x - w.x * u.z, w.x * u.y - w.y * u.x);
    BCam c;
    c.o = from;
    c.horiz = scale(u, 2.f * half_h * aspect);
    c.vert = scale(v, 2.f * half_h);
    c.lower_left = sub(sub(sub(from, scale(c.horiz, 0.5f)), scale(c.vert, 0.5f)), w);
    return c;
}

void add_box(std::vector<BQuad>& q, V3 lo, V3 hi, V3 albedo) {
    q.push_back({0, lo.x, lo.y, hi.y, lo.z, hi.z, albedo, B_DIFFUSE});
    q.push_back({0, hi.x, lo.y, hi.y, lo.z, hi.z, albedo, B_DIFFUSE});
    q.push_back({1, lo.y, lo.x, hi.x, lo.z, hi.z, albedo, B_DIFFUSE});
    q.push_back({1, hi.y, lo.x, hi.x, lo.z, hi.z, albedo, B_DIFFUSE});
    q.push_back({2, lo.z, lo.x, hi.x, lo.y, hi.y, albedo, B_DIFFUSE});
    q.push_back({2, hi.z, lo.x, hi.x, lo.y, hi.y, albedo, B_DIFFUSE});
}

void build_bscene(int scene, uint64_t seed, std::vector<BSphere>& sph, std::vector<BQuad>& quad, bparams& P) {
    const float aspect = (float)P.img_w / (float)P.img_h;
    if (scene == 0) {
        quad.push_back({1, 0.f, -20.f, 20.f, -20.f, 20.f, v3(0.5f, 0.5f, 0.5f), B_DIFFUSE});
        uint64_t s = seed;
        for (int i = 0; i < 512; ++i) {
            const float r = 0.2f + 0.8f * bscene_u01(s);
            const float x = -20.f + 40.f * bscene_u01(s);
            const float z = -20.f + 40.f * bscene_u01(s);
            const float m = bscene_u01(s);
            BSphere b;
            memset(&b, 0, sizeof b);
            b.c = v3(x, r, z);
            b.r = r;
            if (m < 0.6f) {
                const float a0 = bscene_u01(s), a1 = bscene_u01(s), a2 = bscene_u01(s);
                b.albedo = v3(a0 * a0, a1 * a1, a2 * a2);
                b.mat = B_DIFFUSE;
            } else if (m < 0.9f) {
                const float a0 = bscene_u01(s), a1 = bscene_u01(s), a2 = bscene_u01(s), f = bscene_u01(s);
                b.albedo = v3(0.5f + 0.5f * a0, 0.5f + 0.5f * a1, 0.5f + 0.5f * a2);
                b.param = 0.5f * f;
                b.mat = B_METAL;
            } else {
                b.albedo = v3(1.f, 1.f, 1.f);
                b.param = 1.5f;
                b.mat = B_GLASS;
            }
            sph.push_back(b);
        }
        P.sky = 1;
        P.cam = make_bcam(v3(13.f, 2.f, 3.f), v3(0.f, 0.f, 0.f), 0.17632698f /* tan 10 deg */, aspect);
    } else {
        const V3 white = v3(0.73f, 0.73f, 0.73f);
        quad.push_back({1, 0.f, -1.f, 1.f, -1.f, 1.f, white, B_DIFFUSE});                           // floor
        quad.push_back({1, 2.f, -1.f, 1.f, -1.f, 1.f, white, B_DIFFUSE});                           // ceiling
        quad.push_back({2, -1.f, -1.f, 1.f, 0.f, 2.f, white, B_DIFFUSE});                           // back
        quad.push_back({0, -1.f, 0.f, 2.f, -1.f, 1.f, v3(0.65f, 0.05f, 0.05f), B_DIFFUSE});         // left
        quad.push_back({0, 1.f, 0.f, 2.f, -1.f, 1.f, v3(0.12f, 0.45f, 0.15f), B_DIFFUSE});          // right
        quad.push_back({1, 1.999f, -0.3f, 0.3f, -0.3f, 0.3f, v3(15.f, 15.f, 15.f), B_LIGHT});      // light
        add_box(quad, v3(-0.6f, 0.f, -0.6f), v3(-0.1f, 1.2f, -0.1f), white);
        add_box(quad, v3(0.15f, 0.f, 0.f), v3(0.65f, 0.6f, 0.5f), white);
        P.sky = 0;
        P.cam = make_bcam(v3(0.f, 1.f, 3.4f), v3(0.f, 1.f, 0.f), 0.36397023f /* tan 20 deg */, aspect);
    }
}

}  // namespace
