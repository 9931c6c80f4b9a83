// Serial CPU render of the reference ray tracer: test infrastructure (the oracle for
// images).  Restates concurrent_rt/rt_final.cpp: the vector helpers (:329-345), scene
// structures (:350-366), intersection (:371-419), primary rays (:485-499), shading of
// k_trace (:568-639), scenes (:650-684) and cameras (:849-859).  Each pixel's bounces
// run in order and add into the pixel in that order, with the same float operations
// as the device code; built with -ffp-contract=off so no multiply-add is fused.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

struct F3 { float x, y, z; };
F3 f3(float x, float y, float z) { F3 r; r.x = x; r.y = y; r.z = z; return r; }
F3 operator+(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
F3 operator-(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
F3 operator*(F3 a, float s) { return f3(a.x * s, a.y * s, a.z * s); }
F3 mul(F3 a, F3 b) { return f3(a.x * b.x, a.y * b.y, a.z * b.z); }
float dot(F3 a, F3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
F3 norm(F3 v) {
    float d = sqrtf(dot(v, v));
    return d > 0.f ? v * (1.f / d) : v;
}
F3 reflect(F3 v, F3 n) { return v - n * (2.f * dot(v, n)); }
F3 clamp01(F3 c) {
    return f3(fminf(fmaxf(c.x, 0.f), 1.f), fminf(fmaxf(c.y, 0.f), 1.f), fminf(fmaxf(c.z, 0.f), 1.f));
}
struct Sphere { F3 c; float r; F3 albedo; float refl; };
struct Plane { F3 n; float d; F3 albedo; float refl; };
struct Ray { F3 o, d; int px, py, depth; F3 atten; };
struct Hit { float t; F3 n, p, albedo; float refl; bool did_hit; };

Hit isect_sphere(const Ray& ray, const Sphere& s) {
    Hit h; h.did_hit = false; h.t = 1e30f;
    F3 oc = ray.o - s.c;
    float b = dot(oc, ray.d);
    float c = dot(oc, oc) - s.r * s.r;
    float disc = b * b - c;
    if (disc >= 0.f) {
        float t = -b - sqrtf(disc);
        if (t > 1e-4f) {
            h.t = t; h.did_hit = true;
            h.p = ray.o + ray.d * t;
            h.n = norm(h.p - s.c);
            h.albedo = s.albedo;
            h.refl = s.refl;
        }
    }
    return h;
}
Hit isect_plane(const Ray& ray, const Plane& pl) {
    Hit h; h.did_hit = false; h.t = 1e30f;
    float denom = dot(pl.n, ray.d);
    if (fabsf(denom) > 1e-5f) {
        float t = -(dot(pl.n, ray.o) + pl.d) / denom;
        if (t > 1e-4f) {
            h.t = t; h.did_hit = true;
            h.p = ray.o + ray.d * t;
            h.n = pl.n;
            h.albedo = pl.albedo;
            h.refl = pl.refl;
        }
    }
    return h;
}
Hit trace(const Ray& ray, const std::vector<Sphere>& sph, const std::vector<Plane>& pln) {
    Hit best; best.did_hit = false; best.t = 1e30f;
    for (const Sphere& s : sph) { Hit h = isect_sphere(ray, s); if (h.did_hit && h.t < best.t) best = h; }
    for (const Plane& p : pln) { Hit h = isect_plane(ray, p); if (h.did_hit && h.t < best.t) best = h; }
    return best;
}

// Scenes 0 and 1 of rt_final.cpp:650-684 (identical in rt_compaction.cpp:501-552) with
// their cameras (:849-859), and the compaction baseline's scene 2.
void build_scene(int scene, std::vector<Sphere>& sph, std::vector<Plane>& pln, F3& cam_o, F3& cam_f) {
    if (scene == 0) {
        pln.push_back({f3(0, 1, 0), 1.f, f3(0.75f, 0.75f, 0.75f), 0.05f});
        const int gx = 10, gz = 10;
        const float sp = 0.55f, rad = 0.22f, base_y = 0.25f;
        for (int iz = 0; iz < gz; iz++)
            for (int ix = 0; ix < gx; ix++) {
                float x = (ix - (gx - 1) * 0.5f) * sp;
                float z = -2.f - iz * sp;
                int m = (ix + iz * 7) % 7;
                float r = (m == 0) ? 0.9f : (m == 1) ? 0.6f : (m == 2) ? 0.3f : (m == 3) ? 0.1f : 0.f;
                F3 a = (m == 0) ? f3(.9f, .9f, .9f) : (m == 1) ? f3(.9f, .5f, .2f) : (m == 2) ? f3(.2f, .8f, .9f)
                     : (m == 3) ? f3(.7f, .2f, .8f) : (m == 4) ? f3(.2f, .9f, .3f) : (m == 5) ? f3(.9f, .2f, .2f)
                     : f3(.8f, .8f, .3f);
                sph.push_back({f3(x, base_y, z), rad, a, r});
            }
        sph.push_back({f3(-1.2f, 0.6f, -3.5f), 0.6f, f3(.9f, .3f, .3f), 0.7f});
        sph.push_back({f3(1.4f, 0.9f, -4.2f), 0.9f, f3(.3f, .9f, .4f), 0.2f});
        sph.push_back({f3(0.0f, 1.3f, -5.5f), 1.3f, f3(.4f, .6f, .95f), 0.0f});
        cam_o = f3(0, 0.3f, 0.5f);
        cam_f = norm(f3(0, -0.2f, -1.f));
    } else if (scene == 1) {
        sph.push_back({f3(-0.6f, 0.5f, -2.5f), 0.5f, f3(.9f, .3f, .3f), 0.85f});
        sph.push_back({f3(0.6f, 0.6f, -2.8f), 0.6f, f3(.95f, .95f, .95f), 0.95f});
        pln.push_back({f3(0, 1, 0), 1.f, f3(.9f, .9f, .9f), 0.3f});
        pln.push_back({f3(0, 0, 1), 5.f, f3(.6f, .65f, .8f), 0.7f});
        pln.push_back({f3(1, 0, 0), 2.f, f3(.8f, .2f, .2f), 0.6f});
        pln.push_back({f3(-1, 0, 0), 2.f, f3(.2f, .8f, .3f), 0.6f});
        pln.push_back({f3(0, -1, 0), 2.5f, f3(.95f, .95f, .95f), 0.2f});
        cam_o = f3(0, 0.5f, 1.5f);
        cam_f = norm(f3(0, -0.1f, -1.f));
    } else {
        // mirror tunnel (rt_compaction.cpp:554-592): reflective walls, matte absorbers,
        // a chain of near-perfect mirrors; camera :705-707
        pln.push_back({f3(1, 0, 0), 2.0f, f3(0.95f, 0.95f, 0.95f), 0.985f});
        pln.push_back({f3(-1, 0, 0), 2.0f, f3(0.95f, 0.95f, 0.95f), 0.985f});
        pln.push_back({f3(0, 1, 0), 1.2f, f3(0.95f, 0.95f, 0.95f), 0.985f});
        pln.push_back({f3(0, -1, 0), 1.2f, f3(0.95f, 0.95f, 0.95f), 0.985f});
        pln.push_back({f3(0, 0, 1), 20.0f, f3(0.95f, 0.95f, 0.95f), 0.985f});
        pln.push_back({f3(0, 0, -1), 2.5f, f3(0.95f, 0.95f, 0.95f), 0.985f});
        sph.push_back({f3(-1.45f, -0.25f, -4.2f), 0.70f, f3(0.85f, 0.20f, 0.20f), 0.00f});
        sph.push_back({f3(1.35f, 0.20f, -5.3f), 0.80f, f3(0.20f, 0.85f, 0.25f), 0.00f});
        sph.push_back({f3(0.00f, -0.75f, -8.5f), 0.40f, f3(0.85f, 0.85f, 0.20f), 0.00f});
        sph.push_back({f3(0.00f, 0.00f, -4.8f), 0.90f, f3(0.95f, 0.95f, 0.95f), 0.995f});
        sph.push_back({f3(-0.75f, 0.35f, -7.2f), 0.85f, f3(0.95f, 0.85f, 0.85f), 0.995f});
        sph.push_back({f3(0.80f, -0.25f, -9.8f), 0.90f, f3(0.85f, 0.95f, 0.85f), 0.995f});
        sph.push_back({f3(-0.55f, 0.30f, -12.2f), 0.95f, f3(0.85f, 0.85f, 0.95f), 0.995f});
        sph.push_back({f3(0.70f, -0.20f, -14.7f), 1.00f, f3(0.95f, 0.95f, 0.80f), 0.995f});
        sph.push_back({f3(0.00f, 0.10f, -17.2f), 1.05f, f3(0.90f, 0.90f, 0.95f), 0.995f});
        cam_o = f3(0.0f, 0.0f, 1.6f);
        cam_f = norm(f3(0.0f, 0.0f, -1.0f));
    }

}

}  // namespace

// Renders into img (width*height*3 floats); returns the number of rays traced.
extern "C" int64_t oracle_rt_render(int scene, int width, int height, int max_bounces, float* img) {
    std::vector<Sphere> sph;
    std::vector<Plane> pln;
    F3 cam_o, cam_f;
    build_scene(scene, sph, pln, cam_o, cam_f);
    const F3 cam_r = norm(f3(1, 0, 0)), cam_u = norm(f3(0, 1, 0));
    const F3 light_dir = norm(f3(-0.5f, 1.f, 0.2f));
    const F3 ambient = f3(0.05f, 0.05f, 0.05f);
    const float aspect = (float)width / (float)height;
    std::memset(img, 0, sizeof(float) * 3 * (size_t)width * height);
    int64_t traced = 0;
    for (int py = 0; py < height; ++py)
        for (int px = 0; px < width; ++px) {
            float u = ((px + 0.5f) / width - 0.5f) * 2.f * aspect;
            float v = -((py + 0.5f) / height - 0.5f) * 2.f;
            Ray r;
            r.o = cam_o;
            r.d = norm(cam_f + cam_r * u + cam_u * v);
            r.px = px; r.py = py; r.depth = 0;
            r.atten = f3(1.f, 1.f, 1.f);
            float* pix = img + 3 * ((size_t)py * width + px);
            for (;;) {
                ++traced;
                Hit hit = trace(r, sph, pln);
                if (hit.did_hit) {
                    float NdotL = fmaxf(0.f, dot(hit.n, light_dir));
                    F3 direct = ambient + hit.albedo * NdotL;
                    F3 contrib = mul(direct, r.atten);
                    if (hit.refl > 0.f && r.depth < max_bounces) {
                        F3 nr = clamp01(contrib * (1.f - hit.refl));
                        if (nr.x > 0.f || nr.y > 0.f || nr.z > 0.f) { pix[0] += nr.x; pix[1] += nr.y; pix[2] += nr.z; }
                        Ray refl;
                        refl.o = hit.p + hit.n * 1e-4f;
                        refl.d = norm(reflect(r.d, hit.n));
                        refl.px = r.px; refl.py = r.py;
                        refl.depth = r.depth + 1;
                        refl.atten = mul(r.atten, hit.albedo) * hit.refl;
                        r = refl;
                        continue;
                    }
                    F3 c = clamp01(contrib);
                    pix[0] += c.x; pix[1] += c.y; pix[2] += c.z;
                } else {
                    float t = 0.5f * (r.d.y + 1.f);
                    F3 sky = f3(1, 1, 1) * (1.f - t) + f3(0.5f, 0.7f, 1.f) * t;
                    F3 c = clamp01(mul(sky, r.atten));
                    pix[0] += c.x; pix[1] += c.y; pix[2] += c.z;
                }
                break;
            }
        }
    return traced;
}

// The double-buffer + stream-compaction baseline (concurrent_rt/baselines/
// rt_compaction.cpp): primary rays as its kernel_generate_rays (:219-250, direction
// f + (r*u + up*v)), and per bounce the shading of kernel_trace_rays (:258-326): a
// hit gives ambient + albedo * max(0, N.L), a miss the sky gradient; the colour is
// clamped to [0,1] and weighted 1.0 at depth 0 (written) and 0.5 after (added); a
// surface with reflectivity > 0 continues the ray while depth < max_bounces.
extern "C" int64_t oracle_rt_compact_render(int scene, int width, int height, int max_bounces, float* img) {
    std::vector<Sphere> sph;
    std::vector<Plane> pln;
    F3 cam_o, cam_f;
    build_scene(scene, sph, pln, cam_o, cam_f);
    const F3 cam_r = norm(f3(1, 0, 0)), cam_u = norm(f3(0, 1, 0));
    const F3 light_dir = norm(f3(-0.5f, 1.f, 0.2f));
    const F3 ambient = f3(0.05f, 0.05f, 0.05f);
    const float aspect = (float)width / (float)height;
    std::memset(img, 0, sizeof(float) * 3 * (size_t)width * height);
    int64_t traced = 0;
    for (int py = 0; py < height; ++py)
        for (int px = 0; px < width; ++px) {
            const float u = ((px + 0.5f) / width - 0.5f) * 2.f * aspect;
            const float v = -((py + 0.5f) / height - 0.5f) * 2.f;
            Ray r;
            r.o = cam_o;
            r.d = norm(cam_f + (cam_r * u + cam_u * v));
            r.depth = 0;
            float* pix = img + 3 * ((size_t)py * width + px);
            for (;;) {
                ++traced;
                const Hit hit = trace(r, sph, pln);
                F3 color;
                bool cont = false;
                Ray refl;
                if (hit.did_hit) {
                    const float NdotL = fmaxf(0.f, dot(hit.n, light_dir));
                    color = ambient + hit.albedo * NdotL;
                    if (hit.refl > 0.f && r.depth < max_bounces) {
                        refl.o = hit.p + hit.n * 1e-4f;
                        refl.d = norm(reflect(r.d, hit.n));
                        refl.depth = r.depth + 1;
                        cont = true;
                    }
                } else {
                    const float t = 0.5f * (r.d.y + 1.f);
                    color = f3(1, 1, 1) * (1.f - t) + f3(0.5f, 0.7f, 1.f) * t;
                }
                const float w = r.depth == 0 ? 1.0f : 0.5f;
                color = clamp01(color) * w;
                if (r.depth == 0) { pix[0] = color.x; pix[1] = color.y; pix[2] = color.z; }
                else { pix[0] += color.x; pix[1] += color.y; pix[2] += color.z; }
                if (!cont) break;
                r = refl;
            }
        }
    return traced;
}

// ---------------------------------------------------------------------------------
// The benchmark scenes at one sample per pixel (the reference has no such renderer;
// this restates gcq_rt_bounce_render of the library so the GPU image can be checked
// bit for bit).  Per pixel: a PCG stream seeded by splitmix64(seed ^ pixel << 20) | 1,
// one path of at most max_bounces scattering events, the contribution written once.
// Every float operation is written in the device code's order.
namespace bounce {

enum { DIFFUSE = 0, METAL = 1, GLASS = 2, LIGHT = 3 };
struct Ball { F3 c; float r; F3 albedo; float param; int mat; };
struct Rect { int axis; float k, a0, a1, b0, b1; F3 albedo; int mat; };
struct Cam { F3 o, ll, horiz, vert; };
struct BHit { float t; F3 p, n, albedo; float param; int mat; bool front, did_hit; };
struct Scene { std::vector<Ball> balls; std::vector<Rect> rects; Cam cam; bool sky; };

uint64_t splitmix64(uint64_t x) {
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}
// scene randomness: splitmix64 of a counter stepping by the golden ratio
struct SceneRng {
    uint64_t s;
    float u01() {
        const uint64_t r = splitmix64(s);
        s += 0x9e3779b97f4a7c15ULL;
        return (float)(r >> 40) * (1.0f / 16777216.0f);
    }
};
// PCG-RXS-M-XS 32-bit (O'Neill, "PCG: A Family of Simple Fast Space-Efficient
// Statistically Good Algorithms for Random Number Generation", 2014)
uint32_t pcg(uint32_t& s) {
    s = s * 747796405u + 2891336453u;
    const uint32_t w = ((s >> ((s >> 28u) + 4u)) ^ s) * 277803737u;
    return (w >> 22u) ^ w;
}
float rand01(uint32_t& s) { return (float)(pcg(s) >> 8) * (1.0f / 16777216.0f); }
F3 in_unit_sphere(uint32_t& s) {
    for (int k = 0; k < 64; ++k) {
        const float x = 2.f * rand01(s) - 1.f;
        const float y = 2.f * rand01(s) - 1.f;
        const float z = 2.f * rand01(s) - 1.f;
        const F3 p = f3(x, y, z);
        if (dot(p, p) < 1.f) return p;
    }
    return f3(0.f, 0.f, 0.f);
}
float comp(F3 v, int i) { return i == 0 ? v.x : i == 1 ? v.y : v.z; }
F3 cross(F3 a, F3 b) { return f3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x); }

Cam look_at(F3 from, F3 at, float half_h, float aspect) {
    const F3 w = norm(from - at);
    const F3 u = norm(cross(f3(0.f, 1.f, 0.f), w));
    const F3 v = cross(w, u);
    Cam c;
    c.o = from;
    c.horiz = u * (2.f * half_h * aspect);
    c.vert = v * (2.f * half_h);
    c.ll = ((from - c.horiz * 0.5f) - c.vert * 0.5f) - w;
    return c;
}
void box(std::vector<Rect>& q, F3 lo, F3 hi, F3 a) {
    q.push_back({0, lo.x, lo.y, hi.y, lo.z, hi.z, a, DIFFUSE});
    q.push_back({0, hi.x, lo.y, hi.y, lo.z, hi.z, a, DIFFUSE});
    q.push_back({1, lo.y, lo.x, hi.x, lo.z, hi.z, a, DIFFUSE});
    q.push_back({1, hi.y, lo.x, hi.x, lo.z, hi.z, a, DIFFUSE});
    q.push_back({2, lo.z, lo.x, hi.x, lo.y, hi.y, a, DIFFUSE});
    q.push_back({2, hi.z, lo.x, hi.x, lo.y, hi.y, a, DIFFUSE});
}
// scene 0: 512 seeded spheres (60 % diffuse, 30 % metal, 10 % glass) on a 40 x 40
// ground under a sky; scene 1: box room, two boxes, emitting ceiling rectangle
Scene make_scene(int scene, uint64_t seed, float aspect) {
    Scene S;
    if (scene == 0) {
        S.rects.push_back({1, 0.f, -20.f, 20.f, -20.f, 20.f, f3(0.5f, 0.5f, 0.5f), DIFFUSE});
        SceneRng g{seed};
        for (int i = 0; i < 512; ++i) {
            const float r = 0.2f + 0.8f * g.u01();
            const float x = -20.f + 40.f * g.u01();
            const float z = -20.f + 40.f * g.u01();
            const float m = g.u01();
            Ball b;
            b.c = f3(x, r, z);
            b.r = r;
            b.param = 0.f;
            if (m < 0.6f) {
                const float a0 = g.u01(), a1 = g.u01(), a2 = g.u01();
                b.albedo = f3(a0 * a0, a1 * a1, a2 * a2);
                b.mat = DIFFUSE;
            } else if (m < 0.9f) {
                const float a0 = g.u01(), a1 = g.u01(), a2 = g.u01(), f = g.u01();
                b.albedo = f3(0.5f + 0.5f * a0, 0.5f + 0.5f * a1, 0.5f + 0.5f * a2);
                b.param = 0.5f * f;
                b.mat = METAL;
            } else {
                b.albedo = f3(1.f, 1.f, 1.f);
                b.param = 1.5f;
                b.mat = GLASS;
            }
            S.balls.push_back(b);
        }
        S.sky = true;
        S.cam = look_at(f3(13.f, 2.f, 3.f), f3(0.f, 0.f, 0.f), 0.17632698f, aspect);   // tan 10 degrees
    } else {
        const F3 white = f3(0.73f, 0.73f, 0.73f);
        S.rects.push_back({1, 0.f, -1.f, 1.f, -1.f, 1.f, white, DIFFUSE});
        S.rects.push_back({1, 2.f, -1.f, 1.f, -1.f, 1.f, white, DIFFUSE});
        S.rects.push_back({2, -1.f, -1.f, 1.f, 0.f, 2.f, white, DIFFUSE});
        S.rects.push_back({0, -1.f, 0.f, 2.f, -1.f, 1.f, f3(0.65f, 0.05f, 0.05f), DIFFUSE});
        S.rects.push_back({0, 1.f, 0.f, 2.f, -1.f, 1.f, f3(0.12f, 0.45f, 0.15f), DIFFUSE});
        S.rects.push_back({1, 1.999f, -0.3f, 0.3f, -0.3f, 0.3f, f3(15.f, 15.f, 15.f), LIGHT});
        box(S.rects, f3(-0.6f, 0.f, -0.6f), f3(-0.1f, 1.2f, -0.1f), white);
        box(S.rects, f3(0.15f, 0.f, 0.f), f3(0.65f, 0.6f, 0.5f), white);
        S.sky = false;
        S.cam = look_at(f3(0.f, 1.f, 3.4f), f3(0.f, 1.f, 0.f), 0.36397023f, aspect);   // tan 20 degrees
    }
    return S;
}

bool hit_ball(F3 o, F3 d, const Ball& b, float tmax, BHit& h) {
    const F3 oc = o - b.c;
    const float a = dot(d, d);
    const float half_b = dot(oc, d);
    const float c = dot(oc, oc) - b.r * b.r;
    const float disc = half_b * half_b - a * c;
    if (disc < 0.f) return false;
    const float sq = sqrtf(disc);
    float root = (-half_b - sq) / a;
    if (root <= 1e-3f || root >= tmax) {
        root = (-half_b + sq) / a;
        if (root <= 1e-3f || root >= tmax) return false;
    }
    h.t = root;
    h.p = o + d * root;
    const F3 outward = (h.p - b.c) * (1.f / b.r);
    h.front = dot(d, outward) < 0.f;
    h.n = h.front ? outward : outward * -1.f;
    h.albedo = b.albedo;
    h.param = b.param;
    h.mat = b.mat;
    h.did_hit = true;
    return true;
}
bool hit_rect(F3 o, F3 d, const Rect& q, float tmax, BHit& h) {
    const float da = comp(d, q.axis);
    if (fabsf(da) < 1e-8f) return false;
    const float t = (q.k - comp(o, q.axis)) / da;
    if (t <= 1e-3f || t >= tmax) return false;
    const F3 p = o + d * t;
    const float u = q.axis == 0 ? p.y : p.x;
    const float w = q.axis == 2 ? p.y : p.z;
    if (u < q.a0 || u > q.a1 || w < q.b0 || w > q.b1) return false;
    h.t = t;
    h.p = p;
    const F3 outward = f3(q.axis == 0 ? 1.f : 0.f, q.axis == 1 ? 1.f : 0.f, q.axis == 2 ? 1.f : 0.f);
    h.front = da < 0.f;
    h.n = h.front ? outward : outward * -1.f;
    h.albedo = q.albedo;
    h.param = 0.f;
    h.mat = q.mat;
    h.did_hit = true;
    return true;
}

// one path; returns the rays traced, the pixel colour in *out
int64_t path(const Scene& S, F3 o, F3 d, uint32_t rng, int max_bounces, F3* out) {
    F3 tp = f3(1.f, 1.f, 1.f);
    int64_t traced = 0;
    for (int depth = 0;; ++depth) {
        BHit best;
        best.did_hit = false;
        best.t = 1e30f;
        for (const Ball& b : S.balls) { BHit h; if (hit_ball(o, d, b, best.t, h)) best = h; }
        for (const Rect& q : S.rects) { BHit h; if (hit_rect(o, d, q, best.t, h)) best = h; }
        ++traced;
        if (!best.did_hit) {
            if (S.sky) {
                const F3 unit = norm(d);
                const float t = 0.5f * (unit.y + 1.f);
                const F3 sky = f3(1.f, 1.f, 1.f) * (1.f - t) + f3(0.5f, 0.7f, 1.f) * t;
                *out = mul(tp, sky);
            } else {
                *out = f3(0.f, 0.f, 0.f);
            }
            return traced;
        }
        if (best.mat == LIGHT) { *out = mul(tp, best.albedo); return traced; }
        if (depth >= max_bounces) { *out = f3(0.f, 0.f, 0.f); return traced; }
        F3 dir;
        F3 att = best.albedo;
        if (best.mat == DIFFUSE) {
            dir = best.n + norm(in_unit_sphere(rng));
            if (fabsf(dir.x) < 1e-8f && fabsf(dir.y) < 1e-8f && fabsf(dir.z) < 1e-8f) dir = best.n;
        } else if (best.mat == METAL) {
            const F3 refl = reflect(norm(d), best.n);
            dir = refl + in_unit_sphere(rng) * best.param;
            if (dot(dir, best.n) <= 0.f) { *out = f3(0.f, 0.f, 0.f); return traced; }
        } else {
            const float ratio = best.front ? 1.f / best.param : best.param;
            const F3 unit = norm(d);
            const float cos_t = fminf(dot(unit * -1.f, best.n), 1.f);
            const float sin_t = sqrtf(1.f - cos_t * cos_t);
            float r0 = (1.f - ratio) / (1.f + ratio);
            r0 = r0 * r0;
            const float x = 1.f - cos_t;
            const float schlick = r0 + (1.f - r0) * (x * x * x * x * x);
            const float u = rand01(rng);
            if (ratio * sin_t > 1.f || schlick > u) {
                dir = reflect(unit, best.n);
            } else {
                const F3 perp = (unit + best.n * cos_t) * ratio;
                const F3 par = best.n * -sqrtf(fabsf(1.f - dot(perp, perp)));
                dir = perp + par;
            }
            att = f3(1.f, 1.f, 1.f);
        }
        o = best.p;
        d = norm(dir);
        tp = mul(tp, att);
    }
}

}  // namespace bounce

// Returns the rays traced (primary + secondary); img receives width*height RGB.
// threads > 1 splits the rows over std::threads (the image does not depend on it).
extern "C" int64_t oracle_rt_bounce_render(int scene, int width, int height, int max_bounces, uint64_t seed,
                                           int threads, float* img) {
    if (width <= 0 || height <= 0 || scene < 0 || scene > 1 || max_bounces < 0) return -1;
    const bounce::Scene S = bounce::make_scene(scene, seed, (float)width / (float)height);
    if (threads < 1) threads = 1;
    std::vector<int64_t> counts((size_t)threads, 0);
    auto rows = [&](int t) {
        int64_t n = 0;
        for (int py = t; py < height; py += threads)
            for (int px = 0; px < width; ++px) {
                const uint32_t g = (uint32_t)(py * width + px);
                const float s = ((float)px + 0.5f) / (float)width;
                const float tt = 1.0f - ((float)py + 0.5f) / (float)height;
                const F3 d = norm(((S.cam.ll + S.cam.horiz * s) + S.cam.vert * tt) - S.cam.o);
                const uint32_t rng = (uint32_t)bounce::splitmix64(seed ^ ((uint64_t)g << 20)) | 1u;
                F3 c;
                n += bounce::path(S, S.cam.o, d, rng, max_bounces, &c);
                float* o = img + 3 * (size_t)g;
                o[0] = c.x; o[1] = c.y; o[2] = c.z;
            }
        counts[(size_t)t] = n;
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < threads; ++t) pool.emplace_back(rows, t);
    rows(0);
    for (auto& th : pool) th.join();
    int64_t total = 0;
    for (int64_t n : counts) total += n;
    return total;
}
