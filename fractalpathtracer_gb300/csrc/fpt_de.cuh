// fpt_de.cuh -- distance estimators, materials and environment on sm_103a.
//
// Every estimator here restates a function of FPT Metal's shader library
// (shaders/Shaders.metal) or of the Mandelbulber FP64 orbit code
// (src/mandelbulber/orbit.rs) in CUDA; the line ranges are cited per
// function.  The extension formulas are templates over float and D4 (dual
// numbers) so the same code yields distances and analytic gradients.
#pragma once

#include <cuda_fp16.h>

#include "fpt_math.cuh"
#include "fpt_scene.h"

namespace fpt {

struct Material {
    float3 rgb;
    float roughness, specular, translucency, ior, emission;
    int surface;  // extension shading: 0 fractal lobe, 1 ground plane
};
__device__ __forceinline__ Material default_material() {
    Material m;
    m.rgb = mk3(1.0f);
    m.roughness = 1.0f; m.specular = 0.0f; m.translucency = 0.0f; m.ior = 1.5f; m.emission = 0.0f; m.surface = 0;
    return m;
}
__device__ __forceinline__ Material mat(float r, float g, float b, float rough, float spec, float trans, float ior, float em) {
    Material m;
    m.rgb = mk3(r, g, b);
    m.roughness = rough; m.specular = spec; m.translucency = trans; m.ior = ior; m.emission = em; m.surface = 0;
    return m;
}

// Result of one scene evaluation: distance, orbit value (or analytic-scene
// material id) and which surface of an extension scene is nearest.
struct Eval {
    float d;
    float orbit;
    int id;
    int iters;   // orbit iterations of an extension-formula evaluation (profile counters), else 0
};

// ---------------------------------------------------------------- analytic scenes
__device__ __forceinline__ float sd_box(float3 p, float3 b) {                       // :578-581
    float3 q = abs3(p) - b;
    return len3(max3(q, mk3(0.0f))) + fminf(fmaxf(q.x, fmaxf(q.y, q.z)), 0.0f);
}
__device__ __forceinline__ float sd_sphere(float3 p, float r) { return len3(p) - r; }
__device__ __forceinline__ float sd_capped_cylinder(float3 p, float hh, float r) {   // :587-590
    float dx = fabsf(sqrtf(p.x * p.x + p.z * p.z)) - r, dy = fabsf(p.y) - hh;
    float ox = fmaxf(dx, 0.0f), oy = fmaxf(dy, 0.0f);
    return fminf(fmaxf(dx, dy), 0.0f) + sqrtf(ox * ox + oy * oy);
}
__device__ __forceinline__ void hit_union(float &d, int &id, float nd, int nid) { if (nd < d) { d = nd; id = nid; } }  // opUnion :603
__device__ __forceinline__ float room_sdf(float3 p, int &id) {                     // :607-621
    float d = 1000.0f; id = 0;
    float v = p.y + 1.0f; if (v < d) { d = v; id = 0; }
    v = 1.0f - p.y; if (v < d) { d = v; id = 0; }
    v = 1.0f - p.z; if (v < d) { d = v; id = 0; }
    v = p.x + 1.0f; if (v < d) { d = v; id = 1; }
    v = 1.0f - p.x; if (v < d) { d = v; id = 2; }
    return d;
}
static __device__ Eval cornell_scene(float3 p) {                                           // :623-634
    int id; float d = room_sdf(p, id);
    hit_union(d, id, sd_box(p - mk3(0.0f, 0.985f, 0.15f), mk3(0.34f, 0.012f, 0.24f)), 3);
    float3 bp = p - mk3(-0.36f, -0.68f, 0.20f);
    float2 r = rot2a(bp.x, bp.z, 0.28f); bp.x = r.x; bp.z = r.y;
    hit_union(d, id, sd_box(bp, mk3(0.28f, 0.32f, 0.28f)), 5);
    float3 tp = p - mk3(0.36f, -0.48f, -0.16f);
    r = rot2a(tp.x, tp.z, -0.34f); tp.x = r.x; tp.z = r.y;
    hit_union(d, id, sd_box(tp, mk3(0.25f, 0.52f, 0.25f)), 4);
    return {d, 0.0f, id};
}
static __device__ Eval glass_ball_scene(float3 p) {                                        // :636-642
    float d = p.y + 0.72f; int id = 0;
    hit_union(d, id, 1.8f - p.z, 2);
    hit_union(d, id, sd_sphere(p - mk3(0.0f, -0.22f, 0.35f), 0.50f), 1);
    hit_union(d, id, sd_box(p - mk3(-0.58f, 1.05f, -0.28f), mk3(0.32f, 0.04f, 0.32f)), 3);
    return {d, 0.0f, id};
}
static __device__ Eval readme_scene(float3 p, bool glass) {                               // :644-659
    int id; float d = room_sdf(p, id);
    if (glass) {
        hit_union(d, id, sd_capped_cylinder(p - mk3(0.0f, -0.52f, 0.28f), 0.40f, 0.31f), 7);
        hit_union(d, id, sd_sphere(p - mk3(0.0f, 0.17f, 0.28f), 0.30f), 6);
    } else {
        hit_union(d, id, sd_sphere(p - mk3(0.0f, 0.02f, 0.28f), 0.31f), 6);
    }
    hit_union(d, id, sd_box(p - mk3(0.0f, 0.985f, 0.16f), mk3(0.30f, 0.010f, 0.20f)), 3);
    return {d, 0.0f, id};
}

// ---------------------------------------------------------------- built-in fractals
static __device__ Eval de_ball(float3 p0, const DeviceScene &S) {                          // :661-679
    const float *sv = S.set_values;
    float px = p0.x, py = p0.y, pz = p0.z, pw = 1.0f, orbit = 0.0f;
    float a = sv[2] * 2.0f + 2.0f, b = sv[3] * 2.0f + 2.680f, c = sv[4] * 2.0f + 2.0f;
    float hx = a * 0.5f, hy = b * 0.5f, hz = c * 0.5f, fs = 1.4f + sv[5];
    for (int i = 0; i < 12; i++) {
        px = mod1f(px - hx, a) - hx;
        py = mod1f(py - hy, b) - hy;
        pz = mod1f(pz - hz, c) - hz;
        float k = fs / fmaxf(px * px + py * py + pz * pz, 0.0001f);
        px *= k; py *= k; pz *= k; pw *= k;
        orbit += fabsf(py / pw) * 0.25f;
    }
    float d = fmaxf(fabsf(py / pw) * 0.25f * 0.7f, len3(p0) - sv[6]);
    d = fmaxf(d, fabsf(p0.y) - 1.0f);
    return {d, orbit * 2.0f, 0};
}
static __device__ Eval de_cage(float3 p0, const DeviceScene &S) {                          // :681-700
    const float *sv = S.set_values;
    float3 p = p0; float w = 3.0f;
    float k = 2.0f / fminf(dot(p, p), 30.0f);
    p = p * k; w *= k;
    float3 fold = mk3(1.0f + sv[2] * 4.0f, 12.0f + (sv[3] * 4.0f) / 3.0f, 2.0f + sv[4] * 4.0f);
    float sdf = 0.0f, col = 0.0f;
    for (int i = 0; i < 12; i++) {
        p = mk3(2.0f, 4.0f, 2.0f) - (abs3(p) - fold);
        p = mod3f(p - 4.0f, 8.0f) - 4.0f;
        float s = 9.0f / fminf(dot(p, p), 12.0f);
        p = p * s; w *= s;
        sdf = len3(p - clamp3(p, -1.2f, 1.2f)) / w;
        col += sdf;
    }
    return {fmaxf(sdf, len3(p0) - sv[5]), col, 0};
}
static __device__ Eval de_ifs(float3 p, const DeviceScene &S) {                           // :702-728
    const float *sv = S.set_values;
    const float scale = 1.34f, fy = 1.025709f, fx = 1.025709f, fz = 0.035271f;
    float3 julia = mk3(-1.763517f + sv[5], 0.392486f + sv[6], -1.734913f + sv[7]);
    const float *r = S.ifs_rot;  // sxy cxy syz cyz sxz cxz
    p = abs3(p) + (-3.036726f);
    float sdf = 0.0f, col = 0.0f;
    for (int i = 0; i < 50; i++) {
        float zx = p.x, zy = p.y, zz = p.z, t = zx;
        zx = r[1] * t - r[0] * zy; zy = r[0] * t + r[1] * zy;
        t = zx; zx = r[5] * t + r[4] * zz; zz = -r[4] * t + r[5] * zz;
        t = zy; zy = r[3] * t - r[2] * zz; zz = r[2] * t + r[3] * zz;
        p = mk3(fabsf(zx + fx) - fx, fabsf(zy + fy) - fy, fabsf(zz + fz) - fz);
        p = p * scale + julia;
        sdf = len3(p) * powf(scale, -float(i));
        col += sdf;
    }
    return {sdf * 0.7f, col, 0};
}
static __device__ Eval de_mandelbox_ref(float3 pos, const DeviceScene &S) {                // :730-754
    const float *b = S.box_ref;  // s, s, s, |s| over minRad; minRad2; absScalem1; AbsScale
    const float *sv = S.set_values;
    float ox = sv[4], oy = sv[5], oz = sv[6];
    float px = pos.x, py = pos.y, pz = pos.z, pw = 1.0f;
    float sdf = 0.0f, col = 0.0f;
    for (int i = 0; i < 12; i++) {
        px = clampf(px, -1.0f, 1.0f) * 2.0f - px;
        py = clampf(py, -1.0f, 1.0f) * 2.0f - py;
        pz = clampf(pz, -1.0f, 1.0f) * 2.0f - pz;
        float r2 = px * px + py * py + pz * pz;
        float k = clampf(fmaxf(b[4] / fmaxf(r2, 0.00001f), b[4]), 0.0f, 1.0f);
        px *= k; py *= k; pz *= k; pw *= k;
        px = px * b[0] + pos.x + ox;
        py = py * b[1] + pos.y + oy;
        pz = pz * b[2] + pos.z + oz;
        pw = pw * b[3] + 1.0f;
        sdf = (sqrtf(px * px + py * py + pz * pz) - b[5]) / pw - b[6];
        col += sdf;
    }
    return {sdf, col, 0};
}
__device__ __forceinline__ float menger_cut(float3 p, float s) {                    // :761-768
    s *= 2.0f;
    p = mod3f(p - s / 2.0f, s) - s / 2.0f;
    float da = fmaxf(fabsf(p.x), fabsf(p.y)), db = fmaxf(fabsf(p.y), fabsf(p.z)), dc = fmaxf(fabsf(p.z), fabsf(p.x));
    return fminf(da, fminf(db, dc)) - s / 6.0f;
}
static __device__ Eval de_menger_ref(float3 p, const DeviceScene &S) {                    // :770-784
    const float *sv = S.set_values;
    float3 d = abs3(p) - 1.0f;
    float sdf = fmaxf(fmaxf(d.x, d.y), d.z);
    float scale = fmaxf(sv[0], 0.0001f), div = fmaxf(sv[1], 0.0001f);
    for (int i = 0; i < 12; i++) {
        sdf = fmaxf(sdf, -menger_cut(p, scale));
        scale /= div;
        p = rotate_camera(p, sv[2], sv[3]);
    }
    return {sdf, 1.0f, 0};
}
static __device__ Eval de_tower(float3 p, const DeviceScene &S) {                         // :1011-1035
    const float *sv = S.set_values;
    float3 p0 = p;
    p = mod3f(p, 2.0f) - 1.0f;
    p = abs3(p) - 1.0f;
    float t;
    if (p.x < p.z) { t = p.x; p.x = p.z; p.z = t; }
    if (p.y < p.z) { t = p.y; p.y = p.z; p.z = t; }
    if (p.x < p.y) { t = p.x; p.x = p.y; p.y = t; }
    float s = 1.0f, sdf = 0.0f, col = 0.0f;
    float3 shift = mk3(0.6f * (sv[5] * 2.0f + 1.0f), 0.6f * (sv[4] * 2.0f + 1.0f), 3.5f * (sv[3] * 2.0f + 1.0f));
    for (int i = 0; i < 14; i++) {
        float r2 = 2.0f / clampf(dot(p, p), 0.1f, 1.0f);
        p = abs3(p) * r2 - shift;
        s *= r2;
        sdf = len3(p) / s;
        col += sdf;
    }
    return {fmaxf(sdf, len3(p0) - sv[2]), col, 0};
}
static __device__ Eval de_tree(float3 p, const DeviceScene &S) {                          // :1037-1063
    const float *sv = S.set_values;
    float a1 = -9.83f + sv[2] / 2.0f, a2 = -1.16f + sv[3] / 2.0f;
    float3 shift = mk3(-3.508f, -3.593f, 3.295f) + mk3(sv[4], sv[5], sv[6]) * 7.0f;
    float s1, c1, s2, c2;
    sincosf(-a1, &s1, &c1);
    sincosf(-a2, &s2, &c2);
    float s = 1.0f, sdf = 0.0f, orbit = 0.0f;
    for (int i = 0; i < 20; ++i) {
        p = abs3(p);
        float2 r = rot2sc(p.x, p.y, s1, c1); p.x = r.x; p.y = r.y;
        float m = fminf(p.x - p.y, 0.0f); p.x -= m; p.y += m;
        m = fminf(p.x - p.z, 0.0f); p.x -= m; p.z += m;
        m = fminf(p.y - p.z, 0.0f); p.y -= m; p.z += m;
        r = rot2sc(p.y, p.z, s2, c2); p.y = r.x; p.z = r.y;
        p = p * 1.9f; s *= 1.9f;
        p = p + shift;
        float3 d = abs3(p) - 6.0f;
        sdf = (fminf(fmaxf(d.x, fmaxf(d.y, d.z)), 0.0f) + len3(max3(d, mk3(0.0f)))) / s;
        orbit += sdf;
    }
    return {sdf, orbit, 0};
}

// ---------------------------------------------------------------- Mandelbulber field
// Global transform (shaders/Shaders.metal:827-843): world (x, z, y) / scale,
// minus position, SetRotation2, periodic repeat, back to world.
template <class T> __device__ __forceinline__ void global_point(const DeviceScene &S, T &x, T &y, T &z) {
    float ws = fmaxf(S.set_values[0], 1.0f);
    if (S.global_identity) return;
    T qx = x / T(ws), qy = z / T(ws), qz = y / T(ws);
    qx = qx - T(S.vset_values[120]); qy = qy - T(S.vset_values[121]); qz = qz - T(S.vset_values[122]);
    const float *g = S.global_rot;  // sx cx sy cy sz cz
    T ny = qy * T(g[1]) - qz * T(g[0]), nz = qy * T(g[0]) + qz * T(g[1]); qy = ny; qz = nz;
    T nx = qx * T(g[3]) + qz * T(g[2]); nz = -qx * T(g[2]) + qz * T(g[3]); qx = nx; qz = nz;
    nx = qx * T(g[5]) - qy * T(g[4]); ny = qx * T(g[4]) + qy * T(g[5]); qx = nx; qy = ny;
    const float *rep = S.vset_values + 126;
    if (rep[0] > 0.0f) qx = qx - T(rep[0]) * T(floorf((s_val(qx) + 0.5f * rep[0]) / rep[0]));
    if (rep[1] > 0.0f) qy = qy - T(rep[1]) * T(floorf((s_val(qy) + 0.5f * rep[1]) / rep[1]));
    if (rep[2] > 0.0f) qz = qz - T(rep[2]) * T(floorf((s_val(qz) + 0.5f * rep[2]) / rep[2]));
    x = qx * T(ws); y = qz * T(ws); z = qy * T(ws);
}

// screen-space iteration budget (shaders/Shaders.metal:864-887).
__device__ __forceinline__ int screen_iteration_budget(float3 wp, const DeviceScene &S, int mult) {
    int configured = min(max(int(S.set_values[1]) * max(mult, 1), 1), 4096);
    float rate = S.vset_values[130];
    if (!(rate > 0.0f) || !isfinite(rate)) return configured;
    float fp = S.vset_values[115] > 0.5f ? len3(mk3(S.cam_pos[0], S.cam_pos[1], S.cam_pos[2]) - wp) * S.vset_values[116]
                                          : S.vset_values[117];
    fp = clampf(fp, S.vset_values[118], S.vset_values[119]);
    float minimum = fmaxf(S.vset_values[118], 1.0e-12f);
    float oct = fmaxf(log2f(fmaxf(fp / minimum, 1.0f)), 0.0f);
    int red = int(floorf(oct * rate));
    int fb = max(int(ceilf(float(configured) * 0.75f)), 1);
    return max(configured - red, fb);
}

struct Field4 { float d, r, dr, state; };

// Kaleidoscopic IFS built into the Metal library (shaders/Shaders.metal:901-954).
static __device__ Field4 field_ifs(float3 p, const DeviceScene &S, int mult) {
    int budget = screen_iteration_budget(p, S, mult);
    float gx = p.x, gy = p.y, gz = p.z;
    global_point(S, gx, gy, gz);
    const float *sv = S.set_values;
    float ws = fmaxf(sv[0], 1.0f);
    float3 z = mk3(gx / ws, gz / ws, gy / ws);
    float dr = 1.0f, radius = len3(z);
    int completed = 0;
    bool escaped = false;
    float bailout = fmaxf(sv[2], 1.0f), sc = fmaxf(sv[3], 1.000001f);
    uint32_t abs_mask = uint32_t(rintf(sv[4])), enabled = uint32_t(rintf(sv[5]));
    float3 off = mk3(sv[6], sv[7], sv[8]);
    const float *rr = S.mb_rot;  // rotation3: sin/cos of (z-angle, y-angle, x-angle)
    for (int it = 0; it < budget; ++it) {
        if (abs_mask & 1u) z.x = fabsf(z.x);
        if (abs_mask & 2u) z.y = fabsf(z.y);
        if (abs_mask & 4u) z.z = fabsf(z.z);
        for (uint32_t plane = 0; plane < 9u; ++plane) {
            if ((enabled & (1u << plane)) == 0u) continue;
            uint32_t base = 12u + plane * 3u;
            float3 dir = mk3(sv[base], sv[base + 1], sv[base + 2]);
            float proj = dot(z, dir);
            if (proj < 0.0f) z = z - dir * (2.0f * proj);
        }
        float3 v = z - off;
        float ny = v.y * rr[1] - v.z * rr[0], nz = v.y * rr[0] + v.z * rr[1]; v.y = ny; v.z = nz;
        float nx = v.x * rr[3] + v.z * rr[2]; nz = -v.x * rr[2] + v.z * rr[3]; v.x = nx; v.z = nz;
        nx = v.x * rr[5] - v.y * rr[4]; ny = v.x * rr[4] + v.y * rr[5]; v.x = nx; v.y = ny;
        z = v + off;
        z = z * sc - off * (sc - 1.0f);
        dr *= fabsf(sc);
        radius = len3(z);
        completed = it + 1;
        if (radius > bailout) { escaped = true; break; }
    }
    float d = (radius - 2.0f) / fmaxf(fabsf(dr), 1.0e-30f) * ws;
    return {d, radius, dr, escaped ? -float(completed) : float(completed)};
}

// ---------------------------------------------------------------- extension orbit formulas
// Orbit loop of src/mandelbulber/orbit.rs:529-585 with the formula steps of
// orbit.rs:766-778 (Mandelbulb), 1636-1693 (Mandelbox) and the Menger fold;
// finalizers orbit.rs:638-683.  T is float (distance) or D4 (gradient).
template <class T> struct OrbitResult { T d; T r; T dr; int iterations; bool escaped; };

// Power-8 Mandelbulb step in algebraic form: with rho = |z.xy| and
// r = |z|, r^8 (cos 8t, sin 8t) = (rho + i z)^8 and (cos 8p, sin 8p) =
// ((x + i y) / rho)^8, equal to the trigonometric step of orbit.rs:766-778
// (theta = asin(z/r), phi = atan2(y, x)) without any transcendental call.
template <class T> __device__ __forceinline__ void bulb8_step(T &x, T &y, T &z, T &dr, T r) {
    T rho2 = x * x + y * y;
    T rho = s_sqrt(rho2);
    // (rho + i z)^8 by three squarings.
    T a = rho, b = z;
    T a2 = a * a - b * b, b2 = T(2.0f) * a * b;
    T a4 = a2 * a2 - b2 * b2, b4 = T(2.0f) * a2 * b2;
    T a8 = a4 * a4 - b4 * b4, b8 = T(2.0f) * a4 * b4;
    // ((x + i y) / rho)^8, or (1, 0) on the polar axis where atan2(0, 0) = 0.
    T c8, s8;
    if (s_val(rho2) > 0.0f) {
        T inv = T(1.0f) / rho;
        T u = x * inv, v = y * inv;
        T u2 = u * u - v * v, v2 = T(2.0f) * u * v;
        T u4 = u2 * u2 - v2 * v2, v4 = T(2.0f) * u2 * v2;
        c8 = u4 * u4 - v4 * v4; s8 = T(2.0f) * u4 * v4;
    } else {
        c8 = T(1.0f); s8 = T(0.0f);
    }
    T r2 = r * r;
    T r7 = r2 * r2 * r2 * r;
    dr = r7 * dr * T(8.0f) + T(1.0f);
    x = a8 * c8;
    y = a8 * s8;
    z = b8;
}
// Trigonometric step for any power (orbit.rs:766-778).
template <class T> __device__ __forceinline__ void bulb_step(T &x, T &y, T &z, T &dr, T r, float power) {
    T theta0 = s_asin(z / r);
    T phi0 = s_atan2(y, x);
    T rp = s_pow(r, power - 1.0f);
    T theta = theta0 * T(power), phi = phi0 * T(power);
    dr = rp * dr * T(power) + T(1.0f);
    rp = rp * r;
    T st, ct, sp, cp;
    s_sincos(theta, &st, &ct);
    s_sincos(phi, &sp, &cp);
    x = ct * cp * rp;
    y = ct * sp * rp;
    z = st * rp;
}
// The same step in FP32 with cheaper calls: the angles times power/pi go to
// sincospif (no large-argument range reduction), and r^(power-1) is
// exp2((power-1) log2 r).  Against the FP64 oracle the field stays within the
// 5e-5 gate (tests/test_gpu_field.py, powers 2.3-10.6).
__device__ __forceinline__ void bulb_step(float &x, float &y, float &z, float &dr, float r, float power) {
    const float k = power * 0.318309886183790672f;   // power / pi
    const float th = asinf(z / r) * k, ph = atan2f(y, x) * k;
    float rp = exp2f((power - 1.0f) * log2f(r));
    dr = rp * dr * power + 1.0f;
    rp = rp * r;
    float st, ct, sp, cp;
    sincospif(th, &st, &ct);
    sincospif(ph, &sp, &cp);
    x = ct * cp * rp;
    y = ct * sp * rp;
    z = st * rp;
}
// Quadratic triplex, Mandelbulber formula 3 (orbit.rs:752-764): the
// derivative doubles by r with no +1.  On the z axis the division makes the
// point non-finite and the orbit loop rolls the step back.
template <class T> __device__ __forceinline__ void triplex2_step(T &x, T &y, T &z, T &dr, T r) {
    dr = dr * (T(2.0f) * r);
    const T x2 = x * x, y2 = y * y, z2 = z * z;
    const T rho2 = x2 + y2;
    const T temp = T(1.0f) - z2 / rho2;
    const T nx = (x2 - y2) * temp;
    const T ny = T(2.0f) * x * y * temp;
    z = T(-2.0f) * z * s_sqrt(rho2);
    x = nx;
    y = ny;
}
// Mandelbox step (orbit.rs:1636-1693, no rotations, zero offset).
template <class T> __device__ __forceinline__ void box_step(T &x, T &y, T &z, T &dr, const DeviceScene &S) {
    const float lim = S.box_fold_limit, val = S.box_fold_value;
    if (s_val(s_abs(x)) > lim) x = T(signf(s_val(x)) * val) - x;
    if (s_val(s_abs(y)) > lim) y = T(signf(s_val(y)) * val) - y;
    if (s_val(s_abs(z)) > lim) z = T(signf(s_val(z)) * val) - z;
    T r2 = x * x + y * y + z * z;
    if (s_val(r2) < S.box_min2) {
        T f = T(S.box_min_factor);
        x = x * f; y = y * f; z = z * f; dr = dr * f;
    } else if (s_val(r2) < S.box_fixed2) {
        T f = T(S.box_fixed2) / r2;
        x = x * f; y = y * f; z = z * f; dr = dr * f;
    }
    T s = T(S.box_scale);
    x = x * s; y = y * s; z = z * s;
    dr = dr * T(fabsf(S.box_scale)) + T(1.0f);
}
// Menger fold step: abs, descending sort, scale about (1, 1, 1) with the
// Menger-sponge z offset of orbit.rs:734-745.
template <class T> __device__ __forceinline__ void menger_step(T &x, T &y, T &z, T &dr, float s) {
    x = s_abs(x); y = s_abs(y); z = s_abs(z);
    T t;
    if (x < z) { t = x; x = z; z = t; }
    if (y < z) { t = y; y = z; z = t; }
    if (x < y) { t = x; x = y; y = t; }
    float o = s - 1.0f;
    x = x * T(s) - T(o);
    y = y * T(s) - T(o);
    z = z * T(s);
    if (s_val(z) > 0.5f * o) z = z - T(o);
    dr = dr * T(s);
}

// The orbit loop as start / step / finish (orbit_eval runs it to
// completion).
template <class T> struct Orbit {
    T x, y, z, dr, r;
    T cx, cy, cz;   // the constant added after each step
    int i;          // completed iterations
    bool escaped;
};

template <class T> __device__ __forceinline__ void orbit_start(Orbit<T> &o, T px, T py, T pz) {
    o.x = px; o.y = py; o.z = pz;
    o.cx = px; o.cy = py; o.cz = pz;
    o.dr = T(1.0f);
    o.r = s_sqrt(px * px + py * py + pz * pz);
    o.i = 0;
    o.escaped = false;
}

// One iteration; returns false once the orbit is finished (escaped, not
// finite -- the step is rolled back -- or max_iter iterations done).
template <int KIND, class T>
__device__ __forceinline__ bool orbit_step(Orbit<T> &o, const DeviceScene &S, int max_iter, float bailout) {
    const T ox = o.x, oy = o.y, oz = o.z;
    const int i = o.i;
    bool add_c = true;
    if (KIND == KIND_BULB8) bulb8_step(o.x, o.y, o.z, o.dr, o.r);
    else if (KIND == KIND_BULB) {
        if (S.formula == FPT_CUDA_FORMULA_MANDELBULB_POWER2) triplex2_step(o.x, o.y, o.z, o.dr, o.r);
        else bulb_step(o.x, o.y, o.z, o.dr, o.r, S.power);
    } else if (KIND == KIND_BOX) box_step(o.x, o.y, o.z, o.dr, S);
    else if (KIND == KIND_MENGER) { menger_step(o.x, o.y, o.z, o.dr, S.menger_scale); add_c = false; }
    else {  // KIND_HYBRID
        const int period = S.hybrid_period > 1u ? int(S.hybrid_period) : 3;
        if (i % period == period - 1) { menger_step(o.x, o.y, o.z, o.dr, S.menger_scale); add_c = false; }
        else if (S.power == 8.0f) bulb8_step(o.x, o.y, o.z, o.dr, o.r);
        else bulb_step(o.x, o.y, o.z, o.dr, o.r, S.power);
    }
    if (add_c) { o.x = o.x + o.cx; o.y = o.y + o.cy; o.z = o.z + o.cz; }
    o.r = s_sqrt(o.x * o.x + o.y * o.y + o.z * o.z);
    o.i = i + 1;
    if (!isfinite(s_val(o.r))) {
        o.x = ox; o.y = oy; o.z = oz;
        o.r = s_sqrt(o.x * o.x + o.y * o.y + o.z * o.z);
        return false;
    }
    if (s_val(o.r) > bailout) { o.escaped = true; return false; }
    return o.i < max_iter;
}

template <int KIND, class T> __device__ __forceinline__ OrbitResult<T> orbit_finish(const Orbit<T> &ob) {
    OrbitResult<T> o;
    o.r = ob.r; o.dr = ob.dr; o.iterations = ob.i; o.escaped = ob.escaped;
    if (KIND == KIND_MENGER) {
        T qx = s_abs(ob.x) - T(1.0f), qy = s_abs(ob.y) - T(1.0f), qz = s_abs(ob.z) - T(1.0f);
        T mx = s_max(qx, T(0.0f)), my = s_max(qy, T(0.0f)), mz = s_max(qz, T(0.0f));
        T outside = s_sqrt(mx * mx + my * my + mz * mz);
        o.d = (outside + s_min(s_max(qx, s_max(qy, qz)), T(0.0f))) / ob.dr;
    } else if (!(s_val(ob.dr) > 0.0f)) {
        o.d = ob.r;
    } else if (KIND == KIND_BOX) {
        o.d = ob.r / ob.dr;
    } else {
        o.d = s_val(ob.r) > 1.0f ? T(0.5f) * ob.r * s_log(ob.r) / ob.dr : T(0.0f);
    }
    return o;
}

template <int KIND, class T>
__device__ __forceinline__ OrbitResult<T> orbit_eval(const DeviceScene &S, T px, T py, T pz, int max_iter, float bailout) {
    Orbit<T> o;
    orbit_start(o, px, py, pz);
    if (max_iter > 0)
        while (orbit_step<KIND>(o, S, max_iter, bailout)) {
        }
    return orbit_finish<KIND>(o);
}

__device__ __forceinline__ int ext_iterations(const DeviceScene &S) {
    return S.iterations > 0u ? int(S.iterations) : max(int(S.set_values[1]), 1);
}
__device__ __forceinline__ float ext_bailout(const DeviceScene &S) {
    return S.bailout > 0.0f ? S.bailout : fmaxf(S.set_values[2], 1.0f);
}

// Extension formula as a Mandelbulber field (global transform, swizzle,
// distance times world scale) or directly at p for the other scene ids.
template <int KIND, class T>
__device__ __forceinline__ OrbitResult<T> ext_field(const DeviceScene &S, T x, T y, T z, int mult) {
    if (S.sdf_id == FPT_SDF_MANDELBULBER) {
        float ws = fmaxf(S.set_values[0], 1.0f);
        global_point(S, x, y, z);
        T inv = T(1.0f / ws);
        OrbitResult<T> o = orbit_eval<KIND, T>(S, x / T(ws), z / T(ws), y / T(ws), ext_iterations(S) * max(mult, 1), ext_bailout(S));
        (void)inv;
        o.d = o.d * T(ws);
        return o;
    }
    return orbit_eval<KIND, T>(S, x, y, z, ext_iterations(S) * max(mult, 1), ext_bailout(S));
}

// deMandelbulber's iteration-threshold handling (shaders/Shaders.metal:970-994).
__device__ __forceinline__ float mandel_threshold(float3 p, const DeviceScene &S) {                // :3635-3641
    float th = S.vset_values[115] > 0.5f ? len3(mk3(S.cam_pos[0], S.cam_pos[1], S.cam_pos[2]) - p) * S.vset_values[116]
                                         : S.vset_values[117];
    return clampf(th, S.vset_values[118], S.vset_values[119]);
}
__device__ __forceinline__ Eval mandel_finish(const DeviceScene &S, float3 p, Field4 f) {
    Eval e{f.d, 0.0f, 0};
    if (S.vset_values[115] > 1.5f) {
        float th = clampf(len3(mk3(S.cam_pos[0], S.cam_pos[1], S.cam_pos[2]) - p) * S.vset_values[116], S.vset_values[118],
                          S.vset_values[119]);
        if (f.state > 0.0f) e.d = 0.0f;
        else if (e.d < th) e.d = th * 1.01f;
    }
    e.orbit = fabsf(f.state) / fmaxf(S.set_values[1], 1.0f);
    e.iters = int(fabsf(f.state));
    return e;
}

// Field sample (d, r, dr, +-iterations) of a Mandelbulber scene.
template <int KIND> __device__ Field4 mandel_field(float3 p, const DeviceScene &S, int mult) {
    if (KIND == KIND_GENERIC && S.formula == 0) return field_ifs(p, S, mult);
    OrbitResult<float> o;
    if (runtime_kind(KIND)) {
        switch (S.kind) {
            case KIND_BULB8: o = ext_field<KIND_BULB8, float>(S, p.x, p.y, p.z, mult); break;
            case KIND_BULB: o = ext_field<KIND_BULB, float>(S, p.x, p.y, p.z, mult); break;
            case KIND_BOX: o = ext_field<KIND_BOX, float>(S, p.x, p.y, p.z, mult); break;
            case KIND_MENGER: o = ext_field<KIND_MENGER, float>(S, p.x, p.y, p.z, mult); break;
            default: o = ext_field<KIND_HYBRID, float>(S, p.x, p.y, p.z, mult); break;
        }
    } else {
        o = ext_field<KIND, float>(S, p.x, p.y, p.z, mult);
    }
    return {o.d, o.r, o.dr, o.escaped ? -float(o.iterations) : float(o.iterations)};
}

// ---------------------------------------------------------------- typed programs
__device__ __forceinline__ float combine(float cur, float cand, uint32_t mode) {     // :1065-1069
    if (mode == 1u) return fmaxf(cur, cand);
    if (mode == 2u) return fmaxf(cur, -cand);
    return fminf(cur, cand);
}
// deProgramDistance (:1961-2036) / deShadingProgram (:1882-1959).
static __device__ Eval program_distance(float3 p, const DeviceScene &S, bool shading) {
    float scale_acc = 1.0f, distance = kInf, orbit = 0.0f;
    bool has = false;
    uint32_t count = min(shading ? S.shading_count : S.program_count, (uint32_t)FPT_SDF_PROGRAM_MAX_OPS);
    const FptSdfInstruction *prog = shading ? S.shading : S.program;
    for (uint32_t i = 0; i < count; ++i) {
        const FptSdfInstruction op = prog[i];
        float d0 = op.data[0], d1 = op.data[1], d2 = op.data[2], d3 = op.data[3];
        switch (op.opcode) {
            case FPT_SDF_OP_ABS: p = abs3(p); break;
            case FPT_SDF_OP_TRANSLATE: p = p - mk3(d0, d1, d2); break;
            case FPT_SDF_OP_SCALE: { float s = fabsf(d0) > 1.0e-6f ? d0 : 1.0f; p = p * s; scale_acc *= fabsf(s); break; }
            case FPT_SDF_OP_ROTATE_X: { float2 r = rot2a(p.y, p.z, d0); p.y = r.x; p.z = r.y; break; }
            case FPT_SDF_OP_ROTATE_Y: { float2 r = rot2a(p.x, p.z, d0); p.x = r.x; p.z = r.y; break; }
            case FPT_SDF_OP_ROTATE_Z: { float2 r = rot2a(p.x, p.y, d0); p.x = r.x; p.y = r.y; break; }
            case FPT_SDF_OP_REPEAT: {
                float3 per = max3(abs3(mk3(d0, d1, d2)), mk3(1.0e-5f));
                p = p - per * mk3(floorf(p.x / per.x + 0.5f), floorf(p.y / per.y + 0.5f), floorf(p.z / per.z + 0.5f));
                break;
            }
            case FPT_SDF_OP_SORT_DESC: {
                float t;
                if (p.x < p.z) { t = p.x; p.x = p.z; p.z = t; }
                if (p.y < p.z) { t = p.y; p.y = p.z; p.z = t; }
                if (p.x < p.y) { t = p.x; p.x = p.y; p.y = t; }
                break;
            }
            case FPT_SDF_OP_SPHERE: {
                float cand = (len3(p) - d0) / fmaxf(scale_acc, 1.0e-6f);
                distance = has ? combine(distance, cand, op.flags) : cand;
                has = true;
                if (shading) orbit += fabsf(cand) * d3;
                break;
            }
            case FPT_SDF_OP_BOX: {
                float3 q = abs3(p) - abs3(mk3(d0, d1, d2));
                float cand = (fminf(fmaxf(q.x, fmaxf(q.y, q.z)), 0.0f) + len3(max3(q, mk3(0.0f)))) / fmaxf(scale_acc, 1.0e-6f);
                distance = has ? combine(distance, cand, op.flags) : cand;
                has = true;
                if (shading) orbit += fabsf(cand) * d3;
                break;
            }
            case FPT_SDF_OP_PLANE: {
                float3 n = mk3(d0, d1, d2);
                n = n / len3(n);
                float cand = (dot(p, n) + d3) / fmaxf(scale_acc, 1.0e-6f);
                distance = has ? combine(distance, cand, op.flags) : cand;
                has = true;
                break;
            }
            case FPT_SDF_OP_ORBIT_ADD:
                if (shading) orbit += len3(p * mk3(d0, d1, d2)) * d3;
                break;
            default: break;
        }
    }
    return {distance, orbit, 0};
}
// Typed SoA direct evaluation (deTypedSoADistance / typedSoASurface,
// :2857-2960): the union of the lowered spheres, boxes and planes without the
// interpreter.  The surface form also returns the winner's gradient; equal
// distances go to the primitive with the lower source instruction.
__device__ __forceinline__ float soa_distance(float3 p, const DeviceScene &S) {
    const FptTypedSoAProgram &T = S.soa;
    float d = kInf;
    for (uint32_t i = 0; i < T.sphere_count; ++i)
        d = fminf(d, len3(p - mk3(T.sphere_x[i], T.sphere_y[i], T.sphere_z[i])) - T.sphere_radius[i]);
    for (uint32_t i = 0; i < T.box_count; ++i) {
        float3 q = abs3(p - mk3(T.box_x[i], T.box_y[i], T.box_z[i])) - mk3(T.box_half_x[i], T.box_half_y[i], T.box_half_z[i]);
        d = fminf(d, fminf(fmaxf(q.x, fmaxf(q.y, q.z)), 0.0f) + len3(max3(q, mk3(0.0f))));
    }
    for (uint32_t i = 0; i < T.plane_count; ++i) {
        float3 n = normalize3(mk3(T.plane_x[i], T.plane_y[i], T.plane_z[i]));
        d = fminf(d, dot(p - mk3(T.plane_center_x[i], T.plane_center_y[i], T.plane_center_z[i]), n) + T.plane_offset[i]);
    }
    return d;
}
__device__ __forceinline__ float soa_surface(float3 p, const DeviceScene &S, float3 &g) {
    const FptTypedSoAProgram &T = S.soa;
    float best = kInf;
    uint32_t src = 0xffffffffu;
    g = mk3(0.0f);
    auto take = [&](float cand, uint32_t s, float3 grad) {
        if (cand < best || (cand == best && s < src)) { best = cand; src = s; g = grad; }
    };
    for (uint32_t i = 0; i < T.sphere_count; ++i) {
        float3 l = p - mk3(T.sphere_x[i], T.sphere_y[i], T.sphere_z[i]);
        float r = len3(l);
        take(r - T.sphere_radius[i], T.sphere_source[i], r > 1.0e-8f ? l / r : mk3(0.f, 1.f, 0.f));
    }
    for (uint32_t i = 0; i < T.box_count; ++i) {
        float3 l = p - mk3(T.box_x[i], T.box_y[i], T.box_z[i]);
        float3 q = abs3(l) - mk3(T.box_half_x[i], T.box_half_y[i], T.box_half_z[i]);
        float3 o = max3(q, mk3(0.0f));
        float ol = len3(o);
        float cand = fminf(fmaxf(q.x, fmaxf(q.y, q.z)), 0.0f) + ol;
        float3 grad;
        if (ol > 1.0e-8f) grad = mk3(signf(l.x) * o.x, signf(l.y) * o.y, signf(l.z) * o.z) / ol;
        else if (q.x >= q.y && q.x >= q.z) grad = mk3(signf(l.x), 0.f, 0.f);
        else if (q.y >= q.z) grad = mk3(0.f, signf(l.y), 0.f);
        else grad = mk3(0.f, 0.f, signf(l.z));
        take(cand, T.box_source[i], grad);
    }
    for (uint32_t i = 0; i < T.plane_count; ++i) {
        float3 n = normalize3(mk3(T.plane_x[i], T.plane_y[i], T.plane_z[i]));
        take(dot(p - mk3(T.plane_center_x[i], T.plane_center_y[i], T.plane_center_z[i]), n) + T.plane_offset[i],
             T.plane_source[i], n);
    }
    return best;
}

// programSurfaceInterpreted: Jacobian-propagated gradient (:3266-3369).
static __device__ float3 program_gradient(float3 p, const DeviceScene &S, float *dist_out) {
    float3 jx = mk3(1.f, 0.f, 0.f), jy = mk3(0.f, 1.f, 0.f), jz = mk3(0.f, 0.f, 1.f);
    float scale_acc = 1.0f, sd = kInf;
    float3 sg = mk3(0.0f);
    bool has = false;
    uint32_t count = min(S.program_count, (uint32_t)FPT_SDF_PROGRAM_MAX_OPS);
    for (uint32_t i = 0; i < count; ++i) {
        const FptSdfInstruction op = S.program[i];
        float d0 = op.data[0], d1 = op.data[1], d2 = op.data[2], d3 = op.data[3];
        switch (op.opcode) {
            case FPT_SDF_OP_ABS:
                jx = jx * signf(p.x); jy = jy * signf(p.y); jz = jz * signf(p.z); p = abs3(p); break;
            case FPT_SDF_OP_TRANSLATE: p = p - mk3(d0, d1, d2); break;
            case FPT_SDF_OP_SCALE: {
                float sc = fabsf(d0) > 1.0e-6f ? d0 : 1.0f;
                p = p * sc; jx = jx * sc; jy = jy * sc; jz = jz * sc; scale_acc *= fabsf(sc); break;
            }
            case FPT_SDF_OP_ROTATE_X: {
                float sn, cs; sincosf(d0, &sn, &cs);
                float py = p.y; float3 oy = jy;
                p.y = cs * py - sn * p.z; p.z = sn * py + cs * p.z;
                jy = oy * cs - jz * sn; jz = oy * sn + jz * cs; break;
            }
            case FPT_SDF_OP_ROTATE_Y: {
                float sn, cs; sincosf(d0, &sn, &cs);
                float px = p.x; float3 ox = jx;
                p.x = cs * px - sn * p.z; p.z = sn * px + cs * p.z;
                jx = ox * cs - jz * sn; jz = ox * sn + jz * cs; break;
            }
            case FPT_SDF_OP_ROTATE_Z: {
                float sn, cs; sincosf(d0, &sn, &cs);
                float px = p.x; float3 ox = jx;
                p.x = cs * px - sn * p.y; p.y = sn * px + cs * p.y;
                jx = ox * cs - jy * sn; jy = ox * sn + jy * cs; break;
            }
            case FPT_SDF_OP_REPEAT: {
                float3 per = max3(abs3(mk3(d0, d1, d2)), mk3(1.0e-5f));
                p = p - per * mk3(floorf(p.x / per.x + 0.5f), floorf(p.y / per.y + 0.5f), floorf(p.z / per.z + 0.5f));
                break;
            }
            case FPT_SDF_OP_SORT_DESC: {
                float t; float3 tv;
                if (p.x < p.z) { t = p.x; p.x = p.z; p.z = t; tv = jx; jx = jz; jz = tv; }
                if (p.y < p.z) { t = p.y; p.y = p.z; p.z = t; tv = jy; jy = jz; jz = tv; }
                if (p.x < p.y) { t = p.x; p.x = p.y; p.y = t; tv = jx; jx = jy; jy = tv; }
                break;
            }
            case FPT_SDF_OP_SPHERE:
            case FPT_SDF_OP_BOX:
            case FPT_SDF_OP_PLANE: {
                float scale = fmaxf(scale_acc, 1.0e-6f);
                float cand; float3 lg;
                if (op.opcode == FPT_SDF_OP_SPHERE) {
                    float radius = len3(p);
                    cand = (radius - d0) / scale;
                    lg = radius > 1.0e-8f ? p / radius : mk3(0.f, 1.f, 0.f);
                } else if (op.opcode == FPT_SDF_OP_BOX) {
                    float3 q = abs3(p) - abs3(mk3(d0, d1, d2));
                    float3 outside = max3(q, mk3(0.0f));
                    float ol = len3(outside);
                    cand = (fminf(fmaxf(q.x, fmaxf(q.y, q.z)), 0.0f) + ol) / scale;
                    if (ol > 1.0e-8f) lg = mk3(signf(p.x), signf(p.y), signf(p.z)) * outside / ol;
                    else if (q.x >= q.y && q.x >= q.z) lg = mk3(signf(p.x), 0.f, 0.f);
                    else if (q.y >= q.z) lg = mk3(0.f, signf(p.y), 0.f);
                    else lg = mk3(0.f, 0.f, signf(p.z));
                } else {
                    lg = mk3(d0, d1, d2);
                    lg = lg / len3(lg);
                    cand = (dot(p, lg) + d3) / scale;
                }
                float3 cg = (jx * lg.x + jy * lg.y + jz * lg.z) / scale;
                bool choose = !has || (op.flags == 1u ? cand > sd : (op.flags == 2u ? -cand > sd : cand < sd));
                if (choose) {
                    sd = (op.flags == 2u && has) ? -cand : cand;
                    sg = (op.flags == 2u && has) ? -cg : cg;
                }
                has = true;
                break;
            }
            default: break;
        }
    }
    if (dist_out) *dist_out = sd;
    return sg;
}

// ---------------------------------------------------------------- materials
__device__ __forceinline__ float3 hsv2rgb(float3 c) {                              // :535-539
    float k0 = 1.0f, k1 = 2.0f / 3.0f, k2 = 1.0f / 3.0f, k3 = 3.0f;
    float3 p = mk3(fabsf(fractf(c.x + k0) * 6.0f - k3), fabsf(fractf(c.x + k1) * 6.0f - k3), fabsf(fractf(c.x + k2) * 6.0f - k3));
    float3 q = clamp3(p - k0, 0.0f, 1.0f);
    return mk3(c.z * mixf(k0, q.x, c.y), c.z * mixf(k0, q.y, c.y), c.z * mixf(k0, q.z, c.y));
}
static __device__ float3 program_gradient_color(float value, const DeviceScene &S) {       // :3370-3384
    uint32_t count = min(S.gradient_count, 16u);
    if (count == 0u) return mk3(S.program_material[0], S.program_material[1], S.program_material[2]);
    if (count == 1u) return mk3(S.gradient_stops[0][1], S.gradient_stops[0][2], S.gradient_stops[0][3]);
    float t = fractf(value);
    const float *prev = S.gradient_stops[0];
    for (uint32_t i = 1; i < count; ++i) {
        const float *cur = S.gradient_stops[i];
        if (t <= cur[0]) {
            float f = clampf((t - prev[0]) / fmaxf(cur[0] - prev[0], 1.0e-6f), 0.0f, 1.0f);
            return mix3(mk3(prev[1], prev[2], prev[3]), mk3(cur[1], cur[2], cur[3]), f);
        }
        prev = cur;
    }
    return mk3(prev[1], prev[2], prev[3]);
}
static __device__ Material program_material(float orbit, const DeviceScene &S) {          // :3386-3402
    Material m = default_material();
    const float *sv = S.set_values;
    if (S.material_mode == 1u) m.rgb = hsv2rgb(mk3(orbit * (1.0f + sv[1]) + sv[0], 0.5f, 1.0f));
    else if (S.material_mode == 2u) m.rgb = program_gradient_color(orbit * (1.0f + sv[1]) + sv[0], S);
    else m.rgb = mk3(S.program_material[0], S.program_material[1], S.program_material[2]);
    m.roughness = S.program_material[3]; m.specular = S.program_material[4]; m.translucency = S.program_material[5];
    m.ior = S.program_material[6]; m.emission = S.program_material[7];
    return m;
}
static __device__ Material fractal_material(float orbit, const DeviceScene &S, bool menger) { // :3404-3434
    Material m = default_material();
    const float *fs = S.fractal_style;
    if (S.fractal_style_mode != 0u) {
        float o = orbit * fs[1] + fs[0];
        if (S.fractal_style_mode == 1u) m.rgb = hsv2rgb(mk3(o, fs[2], fs[3]));
        else if (S.fractal_style_mode == 2u) m.rgb = mk3(fs[8], fs[9], fs[10]) * fs[3];
        else m.rgb = program_gradient_color(o, S) * fs[3];
        m.rgb = mix3(m.rgb, mk3(fs[8], fs[9], fs[10]), clampf(fs[7], 0.0f, 1.0f));
        m.roughness = fs[4]; m.specular = fs[5]; m.emission = fs[6];
        return m;
    }
    if (menger) return m;
    const float *sv = S.set_values;
    float o = orbit * (1.0f + sv[1]) + sv[0];
    if (S.sdf_id == FPT_SDF_CAGE_FRACTAL || S.sdf_id == FPT_SDF_IFS_FRACTAL || S.sdf_id == FPT_SDF_TREE_FRACTAL)
        o = orbit * (1.0f + sv[1]) / 5.0f + 0.3f + sv[0];
    if (S.sdf_id == FPT_SDF_TOWER_FRACTAL) o = orbit * (1.0f + sv[1]) + 0.3f + sv[0];
    m.rgb = hsv2rgb(mk3(o, 0.5f, 1.0f));
    return m;
}
// Materials of the analytic scenes by hit id (userSdf, :3499-3535).
static __device__ Material analytic_material(const DeviceScene &S, int id) {
    if (S.sdf_id == FPT_SDF_README_CORNELL || S.sdf_id == FPT_SDF_README_GLASS) {
        if (id == 1) return mat(0.62f, 0.055f, 0.030f, 0.95f, 0, 0, 1.5f, 0.010f);
        if (id == 2) return mat(0.035f, 0.82f, 0.09f, 0.92f, 0, 0, 1.5f, 0.010f);
        if (id == 3) return mat(1.0f, 0.94f, 0.82f, 1.0f, 0, 0, 1.5f, 12.0f);
        if (id == 6) {
            if (S.sdf_id == FPT_SDF_README_GLASS) return mat(0.42f, 0.68f, 0.52f, 0.025f, 1.0f, 0.90f, 1.45f, 0);
            return mat(0.72f, 0.78f, 0.74f, 0.24f, 0.72f, 0, 1.5f, 0.012f);
        }
        if (id == 7) return mat(0.84f, 0.88f, 0.86f, 0.45f, 0.24f, 0, 1.5f, 0.018f);
        return mat(0.78f, 0.80f, 0.75f, 0.92f, 0, 0, 1.5f, 0.015f);
    }
    if (S.sdf_id == FPT_SDF_CORNELL_BOX) {
        if (id == 1) return mat(0.82f, 0.12f, 0.08f, 1, 0, 0, 1.5f, 0);
        if (id == 2) return mat(0.10f, 0.55f, 0.18f, 1, 0, 0, 1.5f, 0);
        if (id == 3) return mat(1.0f, 0.88f, 0.64f, 1, 0, 0, 1.5f, 7.0f);
        if (id == 4) return mat(0.72f, 0.70f, 0.64f, 0.82f, 0, 0, 1.5f, 0);
        if (id == 5) return mat(0.70f, 0.68f, 0.62f, 0.92f, 0, 0, 1.5f, 0);
        return mat(0.82f, 0.80f, 0.74f, 1, 0, 0, 1.5f, 0);
    }
    // glass ball scene
    if (id == 1) return mat(0.92f, 0.97f, 1.0f, 0.02f, 1.0f, 1.0f, 1.5f, 0);
    if (id == 2) return mat(0.48f, 0.58f, 0.72f, 0.85f, 0, 0, 1.5f, 0);
    if (id == 3) return mat(1.0f, 0.92f, 0.78f, 1, 0, 0, 1.5f, 5.5f);
    return mat(0.70f, 0.68f, 0.62f, 0.72f, 0.08f, 0, 1.5f, 0);
}

// ---------------------------------------------------------------- scene evaluation
enum EvalMode : int {
    EV_MAP = 0,        // mapSdf (distanceSdf + render[6] halving), :3612-3615
    EV_MATERIAL = 1,   // userSdf (distance + material inputs), :3485-3562
    EV_NORMAL = 2,     // Mandelbulber normal field (mandelbulberNormalDistance, :956-960)
    EV_RAW = 3,        // distanceSdf without the render[6] halving (:3564-3610)
};

template <int KIND>
__device__ __forceinline__ Eval ext_eval(const DeviceScene &S, float3 p) {
    Eval e;
    if (S.sdf_id == FPT_SDF_MANDELBULBER) {
        e = mandel_finish(S, p, mandel_field<KIND>(p, S, 1));
    } else {
        OrbitResult<float> o;
        switch (runtime_kind(KIND) ? S.kind : (uint32_t)KIND) {
            case KIND_BULB8: o = orbit_eval<KIND_BULB8, float>(S, p.x, p.y, p.z, ext_iterations(S), ext_bailout(S)); break;
            case KIND_BULB: o = orbit_eval<KIND_BULB, float>(S, p.x, p.y, p.z, ext_iterations(S), ext_bailout(S)); break;
            case KIND_BOX: o = orbit_eval<KIND_BOX, float>(S, p.x, p.y, p.z, ext_iterations(S), ext_bailout(S)); break;
            case KIND_MENGER: o = orbit_eval<KIND_MENGER, float>(S, p.x, p.y, p.z, ext_iterations(S), ext_bailout(S)); break;
            default: o = orbit_eval<KIND_HYBRID, float>(S, p.x, p.y, p.z, ext_iterations(S), ext_bailout(S)); break;
        }
        e = {o.d, float(o.iterations) / float(max(ext_iterations(S), 1)), 0, o.iterations};
    }
    if (S.ground_plane) {
        float plane = p.y - S.plane_height;
        if (plane < e.d) { e.d = plane; e.id = 1; }
    }
    return e;
}

// One evaluation of the scene at p.  KIND selects a specialised estimator;
// KIND_GENERIC dispatches on the scene at run time.
template <int KIND>
__device__ __forceinline__ Eval scene_eval(const DeviceScene &S, float3 p, int mode) {
    Eval e;
    if (KIND != KIND_GENERIC || S.formula != 0) {
        if (mode == EV_NORMAL && S.sdf_id == FPT_SDF_MANDELBULBER) {
            int mult = S.vset_values[115] > 1.5f ? 5 : 1;
            Field4 f = mandel_field<KIND>(p, S, mult);
            return {f.d, 0.0f, 0};
        }
        e = ext_eval<KIND>(S, p);
    } else {
        switch (S.sdf_id) {
            case FPT_SDF_PROGRAM:
                if (S.soa_count > 0u && mode != EV_MATERIAL) { e = {soa_distance(p, S), 0.0f, 0}; break; }   // :3576-3578
                if (S.program_count > 0u) { e = program_distance(p, S, mode == EV_MATERIAL); break; }
                e = {1000.0f, 0.0f, 0}; break;
            case FPT_SDF_README_CORNELL: e = readme_scene(p, false); break;
            case FPT_SDF_README_GLASS: e = readme_scene(p, true); break;
            case FPT_SDF_CORNELL_BOX: e = cornell_scene(p); break;
            case FPT_SDF_GLASS_BALL: e = glass_ball_scene(p); break;
            case FPT_SDF_BALL_FRACTAL: e = de_ball(p, S); break;
            case FPT_SDF_CAGE_FRACTAL: e = de_cage(p, S); break;
            case FPT_SDF_IFS_FRACTAL: e = de_ifs(p, S); break;
            case FPT_SDF_MANDELBOX_FRACTAL: e = de_mandelbox_ref(p, S); break;
            case FPT_SDF_MENGER_SPONGE: e = de_menger_ref(p, S); break;
            case FPT_SDF_TOWER_FRACTAL: e = de_tower(p, S); break;
            case FPT_SDF_TREE_FRACTAL: e = de_tree(p, S); break;
            case FPT_SDF_MANDELBULBER:
                if (mode == EV_NORMAL) {
                    int mult = S.vset_values[115] > 1.5f ? 5 : 1;
                    Field4 f = field_ifs(p, S, mult);
                    return {f.d, 0.0f, 0};
                }
                e = mandel_finish(S, p, field_ifs(p, S, 1));
                break;
            default: e = {1000.0f, 0.0f, 0}; break;
        }
    }
    if (mode == EV_MAP) e.d = mixf(e.d, e.d / 2.0f, S.render[6]);
    return e;
}

// Material of an evaluation taken with EV_MATERIAL.
static __device__ Material material_of(const DeviceScene &S, const Eval &e) {
    if (S.formula != 0) {
        Material m = fractal_material(e.orbit, S, false);
        if (S.brdf == FPT_CUDA_BRDF_LAMBERT_GGX) m.rgb = mk3(e.id ? S.plane_albedo : S.albedo);
        m.surface = e.id;
        return m;
    }
    switch (S.sdf_id) {
        case FPT_SDF_PROGRAM: return program_material(e.orbit, S);
        case FPT_SDF_README_CORNELL:
        case FPT_SDF_README_GLASS:
        case FPT_SDF_CORNELL_BOX:
        case FPT_SDF_GLASS_BALL: return analytic_material(S, e.id);
        case FPT_SDF_MENGER_SPONGE: return fractal_material(e.orbit, S, true);
        default: return fractal_material(e.orbit, S, false);
    }
}

// Analytic gradient of the extension distance (dual numbers), or the typed
// program's Jacobian gradient.  Returns false when no analytic form applies.
template <int KIND>
static __device__ bool analytic_gradient(const DeviceScene &S, float3 p, float3 &g, uint32_t *orbit_iters = nullptr) {
    if (S.formula != 0) {
        D4 x(p.x, 1.f, 0.f, 0.f), y(p.y, 0.f, 1.f, 0.f), z(p.z, 0.f, 0.f, 1.f);
        OrbitResult<D4> o;
        uint32_t k = runtime_kind(KIND) ? S.kind : (uint32_t)KIND;
        switch (k) {
            case KIND_BULB8: o = ext_field<KIND_BULB8, D4>(S, x, y, z, 1); break;
            case KIND_BULB: o = ext_field<KIND_BULB, D4>(S, x, y, z, 1); break;
            case KIND_BOX: o = ext_field<KIND_BOX, D4>(S, x, y, z, 1); break;
            case KIND_MENGER: o = ext_field<KIND_MENGER, D4>(S, x, y, z, 1); break;
            default: o = ext_field<KIND_HYBRID, D4>(S, x, y, z, 1); break;
        }
        g = mk3(o.d.x, o.d.y, o.d.z);
        if (S.ground_plane && p.y - S.plane_height < o.d.v) g = mk3(0.f, 1.f, 0.f);
        if (orbit_iters) *orbit_iters += uint32_t(o.iterations);
        return true;
    }
    if (S.sdf_id == FPT_SDF_PROGRAM && S.program_count > 0u && (S.normal_mode == 0u || S.normal_mode == 2u)) {
        if (S.soa_count > 0u) soa_surface(p, S, g);   // programSurface uses the lowered form (:3403-3405)
        else g = program_gradient(p, S, nullptr);
        return dot(g, g) >= 1.0e-12f && finite3(g);
    }
    return false;
}

// ---------------------------------------------------------------- environment
static __device__ float preetham(float3 dr, float3 sun) {                                  // :5764-5774
    const float T = 2.0f;
    float A = 0.1787f * T - 1.4630f, B = -0.3554f * T + 0.4275f, C = -0.0227f * T + 5.3251f;
    float D = 0.1206f * T - 2.5771f, E = -0.0670f * T + 0.3703f;
    float theta = acosf(clampf(dr.y, -1.0f, 1.0f));
    float gamma = acosf(clampf(dot(dr, sun), -1.0f, 1.0f));
    float cg = cosf(gamma);
    return (1.0f + A * expf(B / fmaxf(0.1f, cosf(theta)))) * (1.0f + C * expf(D * gamma) + E * cg * cg);
}
static __device__ float3 sky_color(float3 dr, float3 sun) {                                 // :5776-5787
    float sk = preetham(dr, sun);
    float3 col = mix3(mk3(0.004f, 0.048f, 0.253f), mk3(0.8f, 0.9f, 1.0f), sk);
    float hd = (dr.y + 1.0f) / 2.0f, hs = (sun.y + 1.0f) / 2.0f;
    col = mix3(mk3(1.0f, 0.85f, 0.53f) / 4.0f, col * 1.2f, hd) * hs;
    col = (col - 0.5f) * 1.2f + 0.5f;
    float disk = fmaxf((dot(dr, sun) - 1.0f) / (1.0f - cosf(0.05f)) + 1.0f, 0.0f);
    disk *= powf(hd, 10.0f);
    return col * 0.8f + mk3(disk * 100.0f);
}
__device__ __forceinline__ float3 background_gradient(float3 d, const DeviceScene &S) {     // :5789-5794
    float t = clampf((d.y + 1.0f) / 2.0f, 0.0f, 1.0f);
    const float *g = S.background_gradient;
    return mix3(mk3(g[3], g[4], g[5]), mk3(g[0], g[1], g[2]), t);
}
__device__ __forceinline__ float half_bits_to_float(uint16_t h) { return __half2float(__ushort_as_half(h)); }
static __device__ float3 sample_hdri_lut(float3 direction, const DeviceScene &S) {          // :5796-5821
    uint32_t w = min(max(S.hdri_width, 1u), 32u), h = min(max(S.hdri_height, 1u), 16u);
    float3 d = normalize3(direction);
    float u = fractf(atan2f(d.z, d.x) / (2.0f * kPi) + 0.5f);
    float v = clampf(acosf(clampf(d.y, -1.0f, 1.0f)) / kPi, 0.0f, 1.0f);
    float x = u * float(w) - 0.5f, y = v * float(h - 1u);
    int x0i = int(floorf(x));
    uint32_t x0 = uint32_t((x0i % int(w) + int(w)) % int(w)), x1 = (x0 + 1u) % w;
    uint32_t y0 = uint32_t(min(max(int(floorf(y)), 0), int(h - 1u))), y1 = min(y0 + 1u, h - 1u);
    float fx = fractf(x), fy = fractf(y);
    auto px = [&](uint32_t X, uint32_t Y) {
        uint32_t i = (min(Y, h - 1u) * w + min(X, w - 1u)) * 3u;
        return mk3(half_bits_to_float(S.hdri_lut[i]), half_bits_to_float(S.hdri_lut[i + 1]), half_bits_to_float(S.hdri_lut[i + 2]));
    };
    return mix3(mix3(px(x0, y0), px(x1, y0), fx), mix3(px(x0, y1), px(x1, y1), fx), fy);
}
// Full-resolution equirect sky of the extension (texel-centre bilinear).
static __device__ float3 sample_equirect(float3 direction, const DeviceScene &S) {
    uint32_t w = S.sky_width, h = S.sky_height;
    float3 d = normalize3(direction);
    float u = fractf(atan2f(d.z, d.x) / (2.0f * kPi) + 0.5f);
    float v = clampf(acosf(clampf(d.y, -1.0f, 1.0f)) / kPi, 0.0f, 1.0f);
    float x = u * float(w) - 0.5f, y = v * float(h) - 0.5f;
    int x0i = int(floorf(x));
    uint32_t x0 = uint32_t((x0i % int(w) + int(w)) % int(w)), x1 = (x0 + 1u) % w;
    uint32_t y0 = uint32_t(min(max(int(floorf(y)), 0), int(h) - 1)), y1 = min(y0 + 1u, h - 1u);
    float fx = fractf(x), fy = y < 0.0f ? 0.0f : fractf(y);
    auto px = [&](uint32_t X, uint32_t Y) {
        const float *s = S.sky_rgb + (size_t(Y) * w + X) * 3u;
        return mk3(__ldg(s), __ldg(s + 1), __ldg(s + 2));
    };
    return mix3(mix3(px(x0, y0), px(x1, y0), fx), mix3(px(x0, y1), px(x1, y1), fx), fy);
}
static __device__ float3 environment(float3 view, const DeviceScene &S) {                  // :5823-5844
    if (S.sky_width > 0u && S.sky_rgb) return sample_equirect(view, S) * S.world[4];
    if (S.world[4] < 0.00001f) return mk3(0.0f);
    float3 ld = mk3(S.env_light_dir[0], S.env_light_dir[1], S.env_light_dir[2]);
    float3 env;
    if (S.world[0] == 0.0f) {
        float ls = fmaxf(S.world[1], 0.0001f);
        env = mk3(fmaxf((dot(view, ld) - 1.0f) / (1.0f - S.world_cos_size) + 1.0f, 0.0f) / ls * 3.0f);
    } else if (S.world[0] == 1.0f) {
        env = sky_color(view, ld);
    } else if (S.world[0] == 2.0f && S.hdri_enabled != 0u && S.hdri_width > 0u) {
        env = sample_hdri_lut(rotate_camera(view, S.world[2] * kPi / 180.0f, 0.0f), S);
    } else if (S.world[0] == 3.0f) {
        env = mk3(S.world_one_color[0], S.world_one_color[1], S.world_one_color[2]);
    } else {
        env = mk3(1.0f);
    }
    float contrast = S.world[0] == 3.0f ? 1.0f : S.world[5];
    return max3(env * S.world[4] - mk3(0.5f) * contrast + mk3(0.5f), mk3(0.0f));
}

// ---------------------------------------------------------------- path RNG
enum Slot : uint32_t {
    SLOT_LENS0 = 0, SLOT_LENS1 = 1, SLOT_SUN0 = 2, SLOT_SUN1 = 3, SLOT_SCATTER = 4, SLOT_FRESNEL = 5,
    SLOT_DIR0 = 6, SLOT_DIR1 = 7, SLOT_RR = 8, SLOT_LOBE = 9,
};
// Random numbers of one path.  hash13 mode reproduces the reference's seed
// expressions bit for bit (no fused multiply-add, so the float seeds match);
// PCG mode keys each draw by (seed, pixel, sample, bounce, slot).
struct PathRng {
    float x, y, frame;
    uint32_t key;   // PCG: hash of (seed, pixel, sample); 0 in hash13 mode
    bool pcg;
    __device__ void init(bool use_pcg, uint32_t seed, uint32_t pixel, uint32_t sample, float ux, float uy) {
        pcg = use_pcg; x = ux; y = uy; frame = float(sample);
        key = use_pcg ? pcg_hash(seed ^ pcg_hash(pixel ^ pcg_hash(sample))) : 0u;
    }
    __device__ float uniform(uint32_t slot, int bounce) const {
        if (pcg) return float(pcg_hash(key + uint32_t(bounce) * 16u + slot) >> 8) * (1.0f / 16777216.0f);
        float fb = float(bounce);
        switch (slot) {
            case SLOT_LENS0: return hash13(x, y, __fmul_rn(frame, 2.0f));
            case SLOT_LENS1: return hash13(x, y, __fadd_rn(__fmul_rn(frame, 2.0f), 1.0f));
            case SLOT_SUN0: return hash13(x, y, __fadd_rn(__fmul_rn(frame, 5.0f), 1.0f));
            case SLOT_SUN1: return hash13(x, y, __fadd_rn(__fmul_rn(frame, 3.0f), 5.0f));
            case SLOT_SCATTER: return hash13(x, y, __fadd_rn(__fmul_rn(frame, 1.37f), fb));
            case SLOT_FRESNEL: return hash13(x, y, __fadd_rn(__fmul_rn(frame, 7.91f), fb));
            case SLOT_DIR0: { float s = __fadd_rn(__fmul_rn(frame, 13.37f), fb); return hash13(x, y, __fmul_rn(s, 2.0f)); }
            case SLOT_DIR1: { float s = __fadd_rn(__fmul_rn(frame, 13.37f), fb); return hash13(x, y, __fadd_rn(__fmul_rn(s, 2.0f), 1.0f)); }
            case SLOT_RR: return hash13(x, y, __fadd_rn(__fmul_rn(frame, 19.19f), __fmul_rn(fb, 3.17f)));
            default: return hash13(x, y, __fadd_rn(__fmul_rn(frame, 23.71f), __fmul_rn(fb, 5.13f)));
        }
    }
};

// sdfScreenUv (shaders/Shaders.metal:6847-6855) in correctly rounded
// arithmetic: its bits seed hash13.
__device__ __forceinline__ float2 screen_uv(uint32_t gx, uint32_t gy, const DeviceScene &S) {
    float ox = S.sdf_id == FPT_SDF_MANDELBULBER ? 0.0f : 0.5f;
    float oy = S.sdf_id == FPT_SDF_MANDELBULBER ? 1.0f : 0.5f;
    float u = __fsub_rn(__fdiv_rn(__fadd_rn(float(gx), ox), float(S.width)), 0.5f);
    float v = __fsub_rn(__fdiv_rn(__fadd_rn(float(gy), oy), float(S.height)), 0.5f);
    u = __fmul_rn(u, __fdiv_rn(float(S.width), float(S.height)));
    return make_float2(u, v);
}

// ---------------------------------------------------------------- camera
__device__ __forceinline__ bool mandel_visible(float x, float y, const DeviceScene &S) {      // :438-445
    if (S.vset_values[107] < 2.5f || S.vset_values[107] > 3.5f) return true;
    float fov = S.camera_fov * kPi / 180.0f;
    return sqrtf(x * x + y * y) <= (0.5f * kPi / fmaxf(fov, 1.0e-6f));
}
static __device__ float3 mandel_camera_ray(float x, float y, const DeviceScene &S) {                 // :447-471
    float proj = S.vset_values[107];
    float fov = S.camera_fov * kPi / 180.0f;
    float3 ld;
    if ((proj > 0.5f && proj < 1.5f) || (proj > 2.5f && proj < 3.5f)) {
        float radius = sqrtf(x * x + y * y);
        if (radius <= 1.0e-8f) ld = mk3(0.0f, 0.0f, 1.0f);
        else { float rs = sinf(radius * fov) / radius; ld = mk3(x * rs, y * rs, cosf(radius * fov)); }
    } else if (proj > 1.5f && proj < 2.5f) {
        float aspect = float(S.width) / float(S.height);
        float ax = x * (2.0f / aspect) * (0.5f * fov), ay = y * (0.5f * fov);
        ld = mk3(sinf(ax) * cosf(ay), sinf(ay), cosf(ax) * cosf(ay));
    } else {
        ld = normalize3(mk3(x, y, 1.0f / tanf(0.5f * fov)));
    }
    return rotate_camera(normalize3(ld), S.yaw, S.pitch, S.roll);
}
// renderPath's camera ray (shaders/Shaders.metal:5926-5956).
static __device__ bool camera_ray(const DeviceScene &S, float2 uv, const PathRng &rng, bool jitter, float3 &rp, float3 &dr) {
    rp = mk3(S.cam_pos[0], S.cam_pos[1], S.cam_pos[2]);
    float cx = uv.x, cy = uv.y;
    if (jitter) {
        float h1 = rng.uniform(SLOT_LENS0, 0), h2 = rng.uniform(SLOT_LENS1, 0);
        float sr, cr;
        sincosf(2.0f * h1 * kPi, &sr, &cr);
        float s = sqrtf(2.0f * h2 * kPi) * S.aa_strength;
        cx += cr * s; cy += sr * s;
    }
    if (S.sdf_id == FPT_SDF_MANDELBULBER) {
        if (!mandel_visible(cx, cy, S)) return false;
        dr = mandel_camera_ray(cx, cy, S);
    } else {
        dr = rotate_camera(normalize3(mk3(cx, cy, S.focal)), S.yaw, S.pitch, S.roll);
    }
    if (jitter && S.camera_dof > 0.0f) {
        float3 fp = rp + dr * S.focus_distance;
        float h1 = rng.uniform(SLOT_LENS0, 0), h2 = rng.uniform(SLOT_LENS1, 0);
        float sr, cr;
        sincosf(2.0f * h1 * kPi, &sr, &cr);
        float s = sqrtf(2.0f * h2 * kPi) * S.camera_dof;
        rp = rp + rotate_camera(mk3(cr * s, sr * s, 0.0f), S.yaw, S.pitch, S.roll);
        dr = normalize3(fp - rp);
    }
    return true;
}

}  // namespace fpt
