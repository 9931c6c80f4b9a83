// Serial CPU render of the reference ray tracer: test infrastructure (the oracle for
// images).  Restates concurrent_rt/rt_final.cpp: the vector helpers (:329-345), scene
// structures (:350-366), intersection (:371-419), primary rays (:485-499), shading of
// k_trace (:568-639), scenes (:650-684) and cameras (:849-859).  Each pixel's bounces
// run in order and add into the pixel in that order, with the same float operations
// as the device code; built with -ffp-contract=off so no multiply-add is fused.
#include <cmath>
#include <cstdint>
#include <cstring>
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
