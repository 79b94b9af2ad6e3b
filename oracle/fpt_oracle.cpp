// fpt_oracle.cpp -- CPU oracle for the GB300 sphere-tracing path.
//
// TEST INFRASTRUCTURE ONLY.  This is a scalar C++ restatement of FPT Metal's
// hot path (shaders/Shaders.metal, src/metal_bridge.mm) and of the FP64 orbit
// formulas in src/mandelbulber/orbit.rs.  It is used by tests/, by
// __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker;
// the CUDA library never links, loads or calls it.  Each function cites the
// reference lines it follows.  Every routine is a template over the scalar
// type: float reproduces the reference's FP32 arithmetic (compiled with
// -ffp-contract=off so no fused multiply-add changes rounding), double is the
// FP64 oracle, and oracle::Dual carries analytic gradients.
//
// Parity pins: tests/test_oracle.py checks this file against the reference's
// own known-answer tests (src/mandelbulber/orbit.rs:1866-1960) and the voxel
// DDA contract cases (shaders/Shaders.metal:5164-5211).
#include "fpt_math.h"
#include "../include/fpt_cuda.h"

#include <cstdio>
#include <cstdlib>
#include <type_traits>
#include <fstream>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

using Cfg = FptRenderConfig;
using Ext = FptCudaSceneExt;

// ------------------------------------------------------------------ material
template <class T> struct Material {
    V3<T> rgb{T(1), T(1), T(1)};
    T roughness = T(1), specular = T(0), translucency = T(0), ior = T(1.5f), emission = T(0);
    int surface = 0;  // extension shading: 0 fractal lobe, 1 ground plane
};

template <class T> struct DeResult { T d; T orbit; };

// ------------------------------------------------------------------ RNG
// shaders/Shaders.metal:541-555
inline uint32_t hash13bits(float x, float y, float z) {
    uint32_t h = 1190494759u;
    h = (h ^ float_bits(x)) * 0x5bd1e995u;
    h = (h ^ float_bits(y)) * 0x5bd1e995u;
    h = (h ^ float_bits(z)) * 0x5bd1e995u;
    h ^= h >> 13u;
    h *= 0x5bd1e995u;
    h ^= h >> 15u;
    return h;
}
// shaders/Shaders.metal:553-555
inline float hash13(float x, float y, float z) {
    return float(hash13bits(x, y, z) & 0x00ffffffu) / float(0x01000000u);
}

// PCG hash (O'Neill's PCG-RXS-M-XS output permutation applied to one LCG
// step, as tabulated by Jarzynski & Olano, "Hash Functions for GPU
// Rendering", JCGT 2020).  The counter-based stream keys every draw by
// (seed, pixel, sample, bounce, slot), so any sample is reproducible alone.
inline uint32_t pcg_hash(uint32_t v) {
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}
inline float pcg_uniform(uint32_t seed, uint32_t pixel, uint32_t sample, uint32_t dim) {
    uint32_t key = pcg_hash(seed ^ pcg_hash(pixel ^ pcg_hash(sample)));
    return float(pcg_hash(key + dim) >> 8) * (1.0f / 16777216.0f);
}

// Random-number slots of one path (PCG mode); hash13 mode reproduces the
// reference's seed expressions instead (see PathRng::uniform).
enum Slot : uint32_t {
    SLOT_LENS0 = 0, SLOT_LENS1 = 1,          // AA jitter and DOF (reference shares them)
    SLOT_SUN0 = 2, SLOT_SUN1 = 3,            // sun divergence
    SLOT_SCATTER = 4, SLOT_FRESNEL = 5,      // r1, r2
    SLOT_DIR0 = 6, SLOT_DIR1 = 7,            // scatter direction
    SLOT_RR = 8,                             // Russian roulette
    SLOT_LOBE = 9,                           // extension BRDF lobe choice
};

struct PathRng {
    bool pcg;
    uint32_t seed, pixel, sample;
    float x, y, frame;  // uv (bit-exact inputs of hash13) and float(sample)
    float uniform(uint32_t slot, int bounce) const {
        if (pcg) return pcg_uniform(seed, pixel, sample, uint32_t(bounce) * 16u + slot);
        float fb = float(bounce);
        switch (slot) {
            case SLOT_LENS0: return hash13(x, y, frame * 2.0f + 0.0f);
            case SLOT_LENS1: return hash13(x, y, frame * 2.0f + 1.0f);
            case SLOT_SUN0: return hash13(x, y, frame * 5.0f + 1.0f);
            case SLOT_SUN1: return hash13(x, y, frame * 3.0f + 5.0f);
            case SLOT_SCATTER: return hash13(x, y, frame * 1.37f + fb);
            case SLOT_FRESNEL: return hash13(x, y, frame * 7.91f + fb);
            case SLOT_DIR0: { float s = frame * 13.37f + fb; return hash13(x, y, s * 2.0f + 0.0f); }
            case SLOT_DIR1: { float s = frame * 13.37f + fb; return hash13(x, y, s * 2.0f + 1.0f); }
            case SLOT_RR: return hash13(x, y, frame * 19.19f + fb * 3.17f);
            default: return hash13(x, y, frame * 23.71f + fb * 5.13f);
        }
    }
};

// ------------------------------------------------------------------ helpers
template <class T> inline T mod1(T x, T y) { return x - y * std::floor(x / y); }   // :393-395
template <class T> inline V3<T> mod3(V3<T> x, T y) { return {mod1(x.x, y), mod1(x.y, y), mod1(x.z, y)}; }
template <class T> inline T pow5(T x) { T x2 = x * x; return x2 * x2 * x; }      // :401-404

template <class T> inline V2<T> rot2(T px, T py, T a) {                          // :419-423
    T s = std::sin(a), c = std::cos(a);
    return {c * px - s * py, s * px + c * py};
}
// shaders/Shaders.metal:425-431
template <class T> inline V3<T> rotateCamera(V3<T> v, T yaw, T pitch) {
    v = V3<T>(v.x, v.z * std::sin(pitch) + v.y * std::cos(pitch), v.z * std::cos(pitch) - v.y * std::sin(pitch));
    v = V3<T>(v.x * std::cos(yaw) + v.z * std::sin(yaw), v.y, -v.x * std::sin(yaw) + v.z * std::cos(yaw));
    return v;
}
// shaders/Shaders.metal:433-436
template <class T> inline V3<T> rotateCamera(V3<T> v, T yaw, T pitch, T roll) {
    V2<T> r = rot2(v.x, v.y, roll);
    return rotateCamera(V3<T>(r.x, r.y, v.z), yaw, pitch);
}
// shaders/Shaders.metal:535-539
template <class T> inline V3<T> hsv2rgb(V3<T> c) {
    T k[4] = {T(1), T(2) / T(3), T(1) / T(3), T(3)};
    V3<T> p(std::fabs(fractv(c.x + k[0]) * T(6) - k[3]), std::fabs(fractv(c.x + k[1]) * T(6) - k[3]),
            std::fabs(fractv(c.x + k[2]) * T(6) - k[3]));
    V3<T> q = vclamp(p - V3<T>(k[0]), T(0), T(1));
    return V3<T>(c.z * mixv(k[0], q.x, c.y), c.z * mixv(k[0], q.y, c.y), c.z * mixv(k[0], q.z, c.y));
}
// shaders/Shaders.metal:557-569
template <class T> inline V3<T> randomVector(V3<T> normal, T h1, T h2) {
    V3<T> n = normalize(normal);
    V3<T> uu = normalize(cross(n, V3<T>(T(0), T(1), T(1))));
    V3<T> vv = cross(uu, n);
    T ra = std::sqrt(h2);
    T rx = ra * std::cos(T(kPi) * T(2) * h1);
    T ry = ra * std::sin(T(kPi) * T(2) * h1);
    T rz = std::sqrt(std::max(T(1) - h2, T(0)));
    return normalize(uu * rx + vv * ry + n * rz);
}
// shaders/Shaders.metal:571-576
template <class T> inline V2<T> randomPoint(T power, T h1, T h2) {
    T r = T(2) * h1 * T(kPi);
    T r2 = T(2) * h2 * T(kPi);
    T s = std::sqrt(r2) * power;
    return {std::cos(r) * s, std::sin(r) * s};
}
template <class T> inline T sdBox(V3<T> p, V3<T> b) {                             // :578-581
    V3<T> q = vabs(p) - b;
    return length(vmax(q, V3<T>(T(0)))) + std::min(std::max(q.x, std::max(q.y, q.z)), T(0));
}
template <class T> inline T sdSphere(V3<T> p, T r) { return length(p) - r; }      // :583-585
template <class T> inline T sdCappedCylinder(V3<T> p, T hh, T r) {                // :587-590
    T dx = std::fabs(std::sqrt(p.x * p.x + p.z * p.z)) - r;
    T dy = std::fabs(p.y) - hh;
    T ox = std::max(dx, T(0)), oy = std::max(dy, T(0));
    return std::min(std::max(dx, dy), T(0)) + std::sqrt(ox * ox + oy * oy);
}

template <class T> inline T setv(const Cfg &c, int i) { return T(c.set_values[i]); }
template <class T> inline V3<T> cameraPos(const Cfg &c) {
    return {T(c.camera_position[0]), T(c.camera_position[1]), T(c.camera_position[2])};
}

// ------------------------------------------------------------------ analytic scenes
struct SceneHit { float d; int id; };
template <class T> struct HitT { T d; int id; };
template <class T> inline HitT<T> opUnion(HitT<T> a, HitT<T> b) { return (a.d < b.d) ? a : b; }   // :603-605

template <class T> inline T roomSDF(V3<T> p, int &id) {                          // :607-621
    T d = T(1000); id = 0;
    T v = p.y + T(1); if (v < d) { d = v; id = 0; }
    v = T(1) - p.y; if (v < d) { d = v; id = 0; }
    v = T(1) - p.z; if (v < d) { d = v; id = 0; }
    v = p.x + T(1); if (v < d) { d = v; id = 1; }
    v = T(1) - p.x; if (v < d) { d = v; id = 2; }
    return d;
}
template <class T> inline HitT<T> cornellScene(V3<T> p) {                        // :623-634
    int rid = 0;
    HitT<T> s{roomSDF(p, rid), rid};
    s = opUnion(s, HitT<T>{sdBox(p - V3<T>(T(0), T(0.985f), T(0.15f)), V3<T>(T(0.34f), T(0.012f), T(0.24f))), 3});
    V3<T> bp = p - V3<T>(T(-0.36f), T(-0.68f), T(0.20f));
    V2<T> r = rot2(bp.x, bp.z, T(0.28f)); bp.x = r.x; bp.z = r.y;
    s = opUnion(s, HitT<T>{sdBox(bp, V3<T>(T(0.28f), T(0.32f), T(0.28f))), 5});
    V3<T> tp = p - V3<T>(T(0.36f), T(-0.48f), T(-0.16f));
    r = rot2(tp.x, tp.z, T(-0.34f)); tp.x = r.x; tp.z = r.y;
    s = opUnion(s, HitT<T>{sdBox(tp, V3<T>(T(0.25f), T(0.52f), T(0.25f))), 4});
    return s;
}
template <class T> inline HitT<T> glassBallScene(V3<T> p) {                      // :636-642
    HitT<T> s{p.y + T(0.72f), 0};
    s = opUnion(s, HitT<T>{T(1.8f) - p.z, 2});
    s = opUnion(s, HitT<T>{sdSphere(p - V3<T>(T(0), T(-0.22f), T(0.35f)), T(0.50f)), 1});
    s = opUnion(s, HitT<T>{sdBox(p - V3<T>(T(-0.58f), T(1.05f), T(-0.28f)), V3<T>(T(0.32f), T(0.04f), T(0.32f))), 3});
    return s;
}
template <class T> inline HitT<T> readmeCornellScene(V3<T> p) {                  // :644-650
    int rid = 0;
    HitT<T> s{roomSDF(p, rid), rid};
    s = opUnion(s, HitT<T>{sdSphere(p - V3<T>(T(0), T(0.02f), T(0.28f)), T(0.31f)), 6});
    s = opUnion(s, HitT<T>{sdBox(p - V3<T>(T(0), T(0.985f), T(0.16f)), V3<T>(T(0.30f), T(0.010f), T(0.20f))), 3});
    return s;
}
template <class T> inline HitT<T> readmeGlassScene(V3<T> p) {                    // :652-659
    int rid = 0;
    HitT<T> s{roomSDF(p, rid), rid};
    s = opUnion(s, HitT<T>{sdCappedCylinder(p - V3<T>(T(0), T(-0.52f), T(0.28f)), T(0.40f), T(0.31f)), 7});
    s = opUnion(s, HitT<T>{sdSphere(p - V3<T>(T(0), T(0.17f), T(0.28f)), T(0.30f)), 6});
    s = opUnion(s, HitT<T>{sdBox(p - V3<T>(T(0), T(0.985f), T(0.16f)), V3<T>(T(0.30f), T(0.010f), T(0.20f))), 3});
    return s;
}

// ------------------------------------------------------------------ built-in fractals
template <class T> DeResult<T> deBall(V3<T> p0, const Cfg &c) {                  // :661-679
    T p[4] = {p0.x, p0.y, p0.z, T(1)};
    T sdf = 0, orbit = 0;
    T a = setv<T>(c, 2) * T(2) + T(2);
    T b = setv<T>(c, 3) * T(2) + T(2.680f);
    T cc = setv<T>(c, 4) * T(2) + T(2);
    T hx = a * T(0.5f), hy = b * T(0.5f), hz = cc * T(0.5f);
    T fs = T(1.4f) + setv<T>(c, 5);
    for (int i = 0; i < 12; i++) {
        p[0] = mod1(p[0] - hx, a) - hx;
        p[1] = mod1(p[1] - hy, b) - hy;
        p[2] = mod1(p[2] - hz, cc) - hz;
        T k = fs / std::max(p[0] * p[0] + p[1] * p[1] + p[2] * p[2], T(0.0001f));
        for (int j = 0; j < 4; ++j) p[j] *= k;
        sdf = std::fabs(p[1] / p[3]) * T(0.25f);
        orbit += sdf;
    }
    DeResult<T> r;
    r.d = std::max(std::fabs(p[1] / p[3]) * T(0.25f) * T(0.7f), length(p0) - setv<T>(c, 6));
    r.d = std::max(r.d, std::fabs(p0.y) - T(1));
    r.orbit = orbit * T(2);
    return r;
}

template <class T> DeResult<T> deCage(V3<T> p0, const Cfg &c) {                  // :681-700
    T sdf = 0, col = 0;
    V3<T> p = p0; T w = T(3);
    T k = T(2) / std::min(dot(p, p), T(30));
    p = p * k; w *= k;
    V3<T> fold(T(1) + setv<T>(c, 2) * T(4), T(12) + (setv<T>(c, 3) * T(4)) / T(3), T(2) + setv<T>(c, 4) * T(4));
    for (int i = 0; i < 12; i++) {
        p = V3<T>(T(2), T(4), T(2)) - (vabs(p) - fold);
        p = mod3(p - T(4), T(8)) - T(4);
        T s = T(9) / std::min(dot(p, p), T(12));
        p = p * s; w *= s;
        sdf = length(p - vclamp(p, T(-1.2f), T(1.2f))) / w;
        col += sdf;
    }
    return {std::max(sdf, length(p0) - setv<T>(c, 5)), col};
}

template <class T> V3<T> rotateIFS(V3<T> z, T axy, T ayz, T axz) {               // :473-493
    T sxy = std::sin(axy * T(kPi) / T(180)), cxy = std::cos(axy * T(kPi) / T(180));
    T syz = std::sin(ayz * T(kPi) / T(180)), cyz = std::cos(ayz * T(kPi) / T(180));
    T sxz = std::sin(axz * T(kPi) / T(180)), cxz = std::cos(axz * T(kPi) / T(180));
    T zx = z.x, zy = z.y, zz = z.z, t = zx;
    zx = cxy * t - sxy * zy; zy = sxy * t + cxy * zy;
    t = zx; zx = cxz * t + sxz * zz; zz = -sxz * t + cxz * zz;
    t = zy; zy = cyz * t - syz * zz; zz = syz * t + cyz * zz;
    return {zx, zy, zz};
}

template <class T> DeResult<T> deIFS(V3<T> p, const Cfg &c) {                    // :702-728
    T scale = T(1.34f), fy = T(1.025709f), fx = T(1.025709f), fz = T(0.035271f);
    V3<T> julia(T(-1.763517f) + setv<T>(c, 5), T(0.392486f) + setv<T>(c, 6), T(-1.734913f) + setv<T>(c, 7));
    T ax = T(-51.080209f) + setv<T>(c, 2) * T(90);
    T ay = setv<T>(c, 3) * T(90);
    T az = T(-29.096322f) + setv<T>(c, 4) * T(90);
    p = vabs(p) + T(-3.036726f);
    T sdf = 0, col = 0;
    for (int i = 0; i < 50; i++) {
        p = rotateIFS(p, ax, ay, az);
        p.x = std::fabs(p.x + fx) - fx;
        p.y = std::fabs(p.y + fy) - fy;
        p.z = std::fabs(p.z + fz) - fz;
        p = p * scale + julia;
        sdf = length(p) * std::pow(scale, -T(i));
        col += sdf;
    }
    return {sdf * T(0.7f), col};
}

template <class T> DeResult<T> deMandelbox(V3<T> pos, const Cfg &c) {            // :730-754
    T S = T(2.8f) + setv<T>(c, 2);
    T M = T(0.25f) + setv<T>(c, 3);
    T sc[4] = {S / M, S / M, S / M, std::fabs(S) / M};
    T minRad2 = clampv(M, T(1.0e-9f), T(1));
    T absScalem1 = std::fabs(S - T(1));
    T absScale = std::pow(std::fabs(S), T(-9));
    T off[4] = {setv<T>(c, 4), setv<T>(c, 5), setv<T>(c, 6), T(0)};
    T p[4] = {pos.x, pos.y, pos.z, T(1)};
    T p0[4] = {p[0], p[1], p[2], p[3]};
    T sdf = 0, col = 0;
    for (int i = 0; i < 12; i++) {
        for (int j = 0; j < 3; ++j) p[j] = clampv(p[j], T(-1), T(1)) * T(2) - p[j];
        T r2 = p[0] * p[0] + p[1] * p[1] + p[2] * p[2];
        T k = clampv(std::max(minRad2 / std::max(r2, T(0.00001f)), minRad2), T(0), T(1));
        for (int j = 0; j < 4; ++j) p[j] *= k;
        for (int j = 0; j < 4; ++j) p[j] = p[j] * sc[j] + p0[j] + off[j];
        sdf = (std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]) - absScalem1) / p[3] - absScale;
        col += sdf;
    }
    return {sdf, col};
}

template <class T> inline T cubeSdf(V3<T> p) { V3<T> d = vabs(p) - T(1); return std::max(std::max(d.x, d.y), d.z); }  // :756-759
template <class T> inline T mengerCut(V3<T> p, T s) {                            // :761-768
    s *= T(2);
    p = mod3(p - s / T(2), s) - s / T(2);
    T da = std::max(std::fabs(p.x), std::fabs(p.y));
    T db = std::max(std::fabs(p.y), std::fabs(p.z));
    T dc = std::max(std::fabs(p.z), std::fabs(p.x));
    return std::min(da, std::min(db, dc)) - s / T(6);
}
template <class T> DeResult<T> deMenger(V3<T> p, const Cfg &c) {                 // :770-784
    T sdf = cubeSdf(p);
    T scale = std::max(setv<T>(c, 0), T(0.0001f));
    T div = std::max(setv<T>(c, 1), T(0.0001f));
    T ry = setv<T>(c, 2), rp = setv<T>(c, 3);
    for (int i = 0; i < 12; i++) {
        sdf = std::max(sdf, -mengerCut(p, scale));
        scale /= div;
        p = rotateCamera(p, ry, rp);
    }
    return {sdf, T(1)};
}

template <class T> DeResult<T> deTower(V3<T> p, const Cfg &c) {                  // :1011-1035
    T sdf = 0, col = 0;
    V3<T> p0 = p;
    p = mod3(p, T(2)) - T(1);
    p = vabs(p) - T(1);
    if (p.x < p.z) std::swap(p.x, p.z);
    if (p.y < p.z) std::swap(p.y, p.z);
    if (p.x < p.y) std::swap(p.x, p.y);
    T s = T(1);
    V3<T> shift(T(0.6f) * (setv<T>(c, 5) * T(2) + T(1)), T(0.6f) * (setv<T>(c, 4) * T(2) + T(1)),
                T(3.5f) * (setv<T>(c, 3) * T(2) + T(1)));
    for (int i = 0; i < 14; i++) {
        T r2 = T(2) / clampv(dot(p, p), T(0.1f), T(1));
        p = vabs(p) * r2 - shift;
        s *= r2;
        sdf = length(p) / s;
        col += sdf;
    }
    return {std::max(sdf, length(p0) - setv<T>(c, 2)), col};
}

template <class T> DeResult<T> deTree(V3<T> p, const Cfg &c) {                   // :1037-1063
    T orbit = 0, sdf = 0, scale = T(1.9f);
    T a1 = T(-9.83f) + setv<T>(c, 2) / T(2);
    T a2 = T(-1.16f) + setv<T>(c, 3) / T(2);
    V3<T> shift = V3<T>(T(-3.508f), T(-3.593f), T(3.295f)) + V3<T>(setv<T>(c, 4), setv<T>(c, 5), setv<T>(c, 6)) * T(7);
    T s = T(1);
    for (int i = 0; i < 20; ++i) {
        p = vabs(p);
        V2<T> r = rot2(p.x, p.y, -a1); p.x = r.x; p.y = r.y;
        T m = std::min(p.x - p.y, T(0)); p.x += m * T(-1); p.y += m;
        m = std::min(p.x - p.z, T(0)); p.x += m * T(-1); p.z += m;
        m = std::min(p.y - p.z, T(0)); p.y += m * T(-1); p.z += m;
        r = rot2(p.y, p.z, -a2); p.y = r.x; p.z = r.y;
        p = p * scale;
        s *= scale;
        p = p + shift;
        V3<T> d = vabs(p) - T(6);
        sdf = (std::min(std::max(d.x, std::max(d.y, d.z)), T(0)) + length(vmax(d, V3<T>(T(0))))) / s;
        orbit += sdf;
    }
    return {sdf, orbit};
}

// ------------------------------------------------------------------ Mandelbulber field
// Rotation order of Mandelbulber's SetRotation2 (shaders/Shaders.metal:803-820).
template <class T> V3<T> rotation2(V3<T> v, T rx, T ry, T rz) {
    T sx = std::sin(rx), cx = std::cos(rx);
    T y = v.y * cx - v.z * sx, z = v.y * sx + v.z * cx; v.y = y; v.z = z;
    T sy = std::sin(ry), cy = std::cos(ry);
    T x = v.x * cy + v.z * sy; z = -v.x * sy + v.z * cy; v.x = x; v.z = z;
    T sz = std::sin(rz), cz = std::cos(rz);
    x = v.x * cz - v.y * sz; y = v.x * sz + v.y * cz; v.x = x; v.y = y;
    return v;
}
// Rotation order of SetRotation3 (shaders/Shaders.metal:786-801).
template <class T> V3<T> rotation3(V3<T> v, T ax, T ay, T az) {
    T sx = std::sin(az), cx = std::cos(az);
    T y = v.y * cx - v.z * sx, z = v.y * sx + v.z * cx; v.y = y; v.z = z;
    T sy = std::sin(ay), cy = std::cos(ay);
    T x = v.x * cy + v.z * sy; z = -v.x * sy + v.z * cy; v.x = x; v.z = z;
    T sz = std::sin(ax), cz = std::cos(ax);
    x = v.x * cz - v.y * sz; y = v.x * sz + v.y * cz; v.x = x; v.y = y;
    return v;
}
template <class T> inline T repeatCoord(T v, T period) {                         // :822-825
    if (!(period > T(0))) return v;
    return v - period * std::floor((v + T(0.5f) * period) / period);
}
// shaders/Shaders.metal:827-843
template <class T> V3<T> globalPoint(V3<T> p, const Cfg &c) {
    T ws = std::max(setv<T>(c, 0), T(1));
    V3<T> q = V3<T>(p.x, p.z, p.y) / ws;
    q = q - V3<T>(T(c.vset_values[120]), T(c.vset_values[121]), T(c.vset_values[122]));
    q = rotation2(q, T(c.vset_values[123]), T(c.vset_values[124]), T(c.vset_values[125]));
    q = V3<T>(repeatCoord(q.x, T(c.vset_values[126])), repeatCoord(q.y, T(c.vset_values[127])),
              repeatCoord(q.z, T(c.vset_values[128])));
    return V3<T>(q.x, q.z, q.y) * ws;
}
// shaders/Shaders.metal:864-887
template <class T> int screenIterationBudget(V3<T> wp, const Cfg &c, int mult) {
    int configured = std::min(std::max(int(c.set_values[1]) * std::max(mult, 1), 1), 4096);
    float rate = c.vset_values[130];
    if (!(rate > 0.0f) || !std::isfinite(rate)) return configured;
    float footprint = c.vset_values[115] > 0.5f
        ? float(length(cameraPos<T>(c) - wp)) * c.vset_values[116] : c.vset_values[117];
    footprint = clampv(footprint, c.vset_values[118], c.vset_values[119]);
    float minimum = std::max(c.vset_values[118], 1.0e-12f);
    float octaves = std::max(std::log2(std::max(footprint / minimum, 1.0f)), 0.0f);
    int reduction = int(std::floor(octaves * rate));
    int floor_budget = std::max(int(std::ceil(float(configured) * 0.75f)), 1);
    return std::max(configured - reduction, floor_budget);
}

template <class T> struct Field4 { T d, r, dr, state; };  // state = +-completed iterations

// ---------------------------------------------------------------- extension orbit formulas
// FP64 orbit semantics of src/mandelbulber/orbit.rs:529-585 (loop, constant
// addition, bailout, non-finite rollback) with the formulas it names.
template <class T> struct OrbitOut { T d, r, dr; int iterations; bool escaped; T color; };

template <class T> inline T powc(T r, double p) { return std::pow(r, T(p)); }
inline Dual powc(Dual r, double p) { return std::pow(r, p); }

template <class T> inline T len4(const T z[4]) { return std::sqrt(z[0] * z[0] + z[1] * z[1] + z[2] * z[2] + z[3] * z[3]); }

// orbit.rs:766-778 (Mandelbulb, trigonometric form).
template <class T> inline void stepMandelbulb(T z[4], T &dr, T r, double power) {
    T theta0 = std::asin(z[2] / r);
    T phi0 = std::atan2(z[1], z[0]);
    T rp = powc(r, power - 1.0);
    T theta = theta0 * T(power);
    T phi = phi0 * T(power);
    dr = rp * dr * T(power) + T(1);
    rp = rp * r;
    T ct = std::cos(theta);
    z[0] = ct * std::cos(phi) * rp;
    z[1] = ct * std::sin(phi) * rp;
    z[2] = std::sin(theta) * rp;
}
// orbit.rs:752-764 (quadratic triplex, Mandelbulber formula 3): no +1 in the
// derivative; on the z axis the division gives a non-finite point, which the
// orbit loop rolls back.
template <class T> inline void stepMandelbulbPower2(T z[4], T &dr, T r) {
    dr = dr * (T(2) * r);
    T x2 = z[0] * z[0], y2 = z[1] * z[1], z2 = z[2] * z[2];
    T temp = T(1) - z2 / (x2 + y2);
    T x = (x2 - y2) * temp;
    T y = T(2) * z[0] * z[1] * temp;
    T zz = T(-2) * z[2] * std::sqrt(x2 + y2);
    z[0] = x; z[1] = y; z[2] = zz;
}
// Colour increments of the Mandelbox: per folded axis, and for the minimum /
// fixed radius spheres (Mandelbulber's defaults, the parameters of the
// reference's own test at orbit.rs:1946-1948).
constexpr double kBoxColorFactor[3] = {0.03, 0.05, 0.07};
constexpr double kBoxColorSphereMin = 0.2, kBoxColorSphereFixed = 0.2;
// orbit.rs:1636-1693 (full Mandelbox, rotations disabled, zero offset).
template <class T> inline void stepMandelbox(T z[4], T &dr, T &color, const Ext &e) {
    T limit = T(e.box_fold_limit), value = T(e.box_fold_value);
    for (int a = 0; a < 3; ++a) {
        if (std::fabs(z[a]) > limit) {
            z[a] = signv(z[a]) * value - z[a];
            color += T(kBoxColorFactor[a]);
        }
    }
    T r2 = z[0] * z[0] + z[1] * z[1] + z[2] * z[2] + z[3] * z[3];
    T fixed2 = T(double(e.box_fixed_radius) * double(e.box_fixed_radius));
    T min2 = T(double(e.box_min_radius) * double(e.box_min_radius));
    if (r2 < min2) {
        T f = fixed2 / min2;
        for (int k = 0; k < 4; ++k) z[k] = z[k] * f;
        dr = dr * f;
        color += T(kBoxColorSphereMin);
    } else if (r2 < fixed2) {
        T f = fixed2 / r2;
        for (int k = 0; k < 4; ++k) z[k] = z[k] * f;
        dr = dr * f;
        color += T(kBoxColorSphereFixed);
    }
    T s = T(e.box_scale);
    for (int k = 0; k < 4; ++k) z[k] = z[k] * s;
    dr = dr * std::fabs(s) + T(1);
}
// Menger fold: abs, descending sort (the SORT_DESC swaps of
// shaders/Shaders.metal:1918-1922) and the scale/offset step of orbit.rs's
// Kaleidoscopic IFS in Menger-sponge mode (orbit.rs:734-745, offset (1,1,1)).
template <class T> inline void stepMenger(T z[4], T &dr, T s) {
    z[0] = std::fabs(z[0]); z[1] = std::fabs(z[1]); z[2] = std::fabs(z[2]);
    if (z[0] < z[2]) std::swap(z[0], z[2]);
    if (z[1] < z[2]) std::swap(z[1], z[2]);
    if (z[0] < z[1]) std::swap(z[0], z[1]);
    T o = s - T(1);
    z[0] = z[0] * s - o;
    z[1] = z[1] * s - o;
    z[2] = z[2] * s;
    if (z[2] > T(0.5f) * o) z[2] = z[2] - o;
    dr = dr * s;
}

template <class T> OrbitOut<T> orbitEval(const Ext &e, int max_iter, double bailout, V3<T> p) {
    T z[4] = {p.x, p.y, p.z, T(0)};
    T c[4] = {p.x, p.y, p.z, T(0)};
    T dr = T(1), color = T(1);
    T r = len4(z);
    int iterations = 0;
    bool escaped = false;
    const int period = e.hybrid_period > 1 ? int(e.hybrid_period) : 3;
    for (int i = 0; i < max_iter; ++i) {
        T old[4] = {z[0], z[1], z[2], z[3]};
        bool add_c = true;
        switch (e.formula) {
            case FPT_CUDA_FORMULA_MANDELBULB: stepMandelbulb(z, dr, r, double(e.power)); break;
            case FPT_CUDA_FORMULA_MANDELBULB_POWER2: stepMandelbulbPower2(z, dr, r); break;
            case FPT_CUDA_FORMULA_MANDELBOX: stepMandelbox(z, dr, color, e); break;
            case FPT_CUDA_FORMULA_MENGER_FOLD: stepMenger(z, dr, T(e.menger_scale)); add_c = false; break;
            case FPT_CUDA_FORMULA_BULB_MENGER_HYBRID:
                if (i % period == period - 1) { stepMenger(z, dr, T(e.menger_scale)); add_c = false; }
                else stepMandelbulb(z, dr, r, double(e.power));
                break;
            default: break;
        }
        if (add_c) for (int k = 0; k < 4; ++k) z[k] = z[k] + c[k];
        r = len4(z);
        iterations = i + 1;
        if (!std::isfinite(r)) {
            for (int k = 0; k < 4; ++k) z[k] = old[k];
            r = len4(z);
            break;
        }
        if (r > T(bailout)) { escaped = true; break; }
    }
    OrbitOut<T> out;
    out.r = r; out.dr = dr; out.iterations = iterations; out.escaped = escaped; out.color = color;
    // Finalizers: orbit.rs:638-683.
    if (e.formula == FPT_CUDA_FORMULA_MENGER_FOLD) {
        // Box distance of the folded point over the accumulated scale.
        V3<T> q = vabs(V3<T>(z[0], z[1], z[2])) - T(1);
        T outside = length(vmax(q, V3<T>(T(0))));
        out.d = (outside + std::min(std::max(q.x, std::max(q.y, q.z)), T(0))) / dr;
    } else if (!(dr > T(0))) {
        out.d = r;
    } else if (e.formula == FPT_CUDA_FORMULA_MANDELBOX) {
        out.d = r / dr;                         // Linear, offset1 = 0
    } else {
        out.d = r > T(1) ? T(0.5) * r * std::log(r) / dr : T(0);   // Logarithmic
    }
    return out;
}

inline int extIterations(const Ext &e, const Cfg &c) {
    if (e.iterations > 0) return int(e.iterations);
    return std::max(int(c.set_values[1]), 1);
}
inline double extBailout(const Ext &e, const Cfg &c) {
    if (e.bailout > 0.0f) return double(e.bailout);
    return double(std::max(c.set_values[2], 1.0f));
}

// shaders/Shaders.metal:901-954 (Kaleidoscopic IFS built into the Metal
// library) or the extension formula through the same world transform.
template <class T> Field4<T> fieldSample(V3<T> p, const Cfg &c, const Ext &e, int mult) {
    if (e.formula != 0) {
        T ws = std::max(setv<T>(c, 0), T(1));
        V3<T> g = globalPoint(p, c) / ws;
        V3<T> z(g.x, g.z, g.y);
        int iters = extIterations(e, c) * std::max(mult, 1);
        OrbitOut<T> o = orbitEval(e, iters, extBailout(e, c), z);
        return {o.d * ws, o.r, o.dr, o.escaped ? T(-o.iterations) : T(o.iterations)};
    }
    if constexpr (std::is_same<T, Dual>::value) {
        return {T(0), T(0), T(0), T(0)};
    } else {
    int budget = screenIterationBudget(p, c, mult);
    p = globalPoint(p, c);
    T ws = std::max(setv<T>(c, 0), T(1));
    V3<T> sc = p / ws;
    V3<T> z(sc.x, sc.z, sc.y);
    T dr = T(1);
    T radius = length(z);
    int completed = 0;
    bool escaped = false;
    T bailout = std::max(setv<T>(c, 2), T(1));
    T ifs_scale = std::max(setv<T>(c, 3), T(1.000001f));
    uint32_t abs_mask = uint32_t(std::lround(c.set_values[4]));
    uint32_t enabled = uint32_t(std::lround(c.set_values[5]));
    V3<T> off(setv<T>(c, 6), setv<T>(c, 7), setv<T>(c, 8));
    T rx = setv<T>(c, 9), ry = setv<T>(c, 10), rz = setv<T>(c, 11);
    for (int it = 0; it < budget; ++it) {
        if (abs_mask & 1u) z.x = std::fabs(z.x);
        if (abs_mask & 2u) z.y = std::fabs(z.y);
        if (abs_mask & 4u) z.z = std::fabs(z.z);
        for (uint32_t plane = 0; plane < 9; ++plane) {
            if ((enabled & (1u << plane)) == 0u) continue;
            uint32_t base = 12u + plane * 3u;
            V3<T> dir(setv<T>(c, base), setv<T>(c, base + 1), setv<T>(c, base + 2));
            T proj = dot(z, dir);
            if (proj < T(0)) z = z - dir * (T(2) * proj);
        }
        z = rotation3(z - off, rx, ry, rz) + off;
        z = z * ifs_scale - off * (ifs_scale - T(1));
        dr = dr * std::fabs(ifs_scale);
        radius = length(z);
        completed = it + 1;
        if (radius > bailout) { escaped = true; break; }
    }
    T d = (radius - T(2)) / std::max(std::fabs(dr), T(1.0e-30f)) * ws;
    return {d, radius, dr, escaped ? T(-completed) : T(completed)};
    }
}

// shaders/Shaders.metal:970-994
template <class T> DeResult<T> deMandelbulber(V3<T> p, const Cfg &c, const Ext &e) {
    Field4<T> s = fieldSample(p, c, e, 1);
    DeResult<T> r{s.d, T(0)};
    if (c.vset_values[115] > 1.5f) {
        T th = clampv(length(cameraPos<T>(c) - p) * T(c.vset_values[116]), T(c.vset_values[118]), T(c.vset_values[119]));
        if (s.state > T(0)) r.d = T(0);
        else if (r.d < th) r.d = th * T(1.01f);
    }
    r.orbit = std::fabs(s.state) / std::max(setv<T>(c, 1), T(1));
    return r;
}

// ------------------------------------------------------------------ typed programs
template <class T> inline T combine(T cur, T cand, uint32_t mode) {              // :1065-1069
    if (mode == 1u) return std::max(cur, cand);
    if (mode == 2u) return std::max(cur, -cand);
    return std::min(cur, cand);
}

// Distance of one program (deProgramDistance :1961-2036, or deShadingProgram
// :1882-1959 when `shading` is set, which also accumulates the orbit value).
template <class T> DeResult<T> programDistance(V3<T> p, const Cfg &c, bool shading) {
    T scale_acc = T(1), distance = T(kInf), orbit = T(0);
    bool has = false;
    uint32_t count = std::min<uint32_t>(shading ? c.sdf_shading_program_count : c.sdf_program_count, FPT_SDF_PROGRAM_MAX_OPS);
    const FptSdfInstruction *prog = shading ? c.sdf_shading_program : c.sdf_program;
    for (uint32_t i = 0; i < count; ++i) {
        const FptSdfInstruction &op = prog[i];
        T d0 = T(op.data[0]), d1 = T(op.data[1]), d2 = T(op.data[2]), d3 = T(op.data[3]);
        switch (op.opcode) {
            case FPT_SDF_OP_ABS: p = vabs(p); break;
            case FPT_SDF_OP_TRANSLATE: p = p - V3<T>(d0, d1, d2); break;
            case FPT_SDF_OP_SCALE: {
                T s = std::fabs(d0) > T(1.0e-6f) ? d0 : T(1);
                p = p * s; scale_acc *= std::fabs(s); break;
            }
            case FPT_SDF_OP_ROTATE_X: { V2<T> r = rot2(p.y, p.z, d0); p.y = r.x; p.z = r.y; break; }
            case FPT_SDF_OP_ROTATE_Y: { V2<T> r = rot2(p.x, p.z, d0); p.x = r.x; p.z = r.y; break; }
            case FPT_SDF_OP_ROTATE_Z: { V2<T> r = rot2(p.x, p.y, d0); p.x = r.x; p.y = r.y; break; }
            case FPT_SDF_OP_REPEAT: {
                V3<T> per = vmax(vabs(V3<T>(d0, d1, d2)), V3<T>(T(1.0e-5f)));
                p = p - per * vfloor(p / per + T(0.5f));
                break;
            }
            case FPT_SDF_OP_SORT_DESC:
                if (p.x < p.z) std::swap(p.x, p.z);
                if (p.y < p.z) std::swap(p.y, p.z);
                if (p.x < p.y) std::swap(p.x, p.y);
                break;
            case FPT_SDF_OP_SPHERE: {
                T cand = (length(p) - d0) / std::max(scale_acc, T(1.0e-6f));
                distance = has ? combine(distance, cand, op.flags) : cand;
                has = true;
                if (shading) orbit += std::fabs(cand) * d3;
                break;
            }
            case FPT_SDF_OP_BOX: {
                V3<T> q = vabs(p) - vabs(V3<T>(d0, d1, d2));
                T cand = (std::min(std::max(q.x, std::max(q.y, q.z)), T(0)) + length(vmax(q, V3<T>(T(0))))) /
                         std::max(scale_acc, T(1.0e-6f));
                distance = has ? combine(distance, cand, op.flags) : cand;
                has = true;
                if (shading) orbit += std::fabs(cand) * d3;
                break;
            }
            case FPT_SDF_OP_PLANE: {
                T cand = (dot(p, normalize(V3<T>(d0, d1, d2))) + d3) / std::max(scale_acc, T(1.0e-6f));
                distance = has ? combine(distance, cand, op.flags) : cand;
                has = true;
                break;
            }
            case FPT_SDF_OP_ORBIT_ADD:
                if (shading) orbit += length(p * V3<T>(d0, d1, d2)) * d3;
                break;
            default: break;
        }
    }
    return {distance, orbit};
}

// Analytic gradient by Jacobian propagation: programSurfaceInterpreted,
// shaders/Shaders.metal:3266-3369.
template <class T> struct ProgramSurface { T distance; V3<T> gradient; };
template <class T> ProgramSurface<T> programSurface(V3<T> p, const Cfg &c) {
    V3<T> jx(T(1), T(0), T(0)), jy(T(0), T(1), T(0)), jz(T(0), T(0), T(1));
    T scale_acc = T(1);
    ProgramSurface<T> s{T(kInf), V3<T>(T(0))};
    bool has = false;
    uint32_t count = std::min<uint32_t>(c.sdf_program_count, FPT_SDF_PROGRAM_MAX_OPS);
    for (uint32_t i = 0; i < count; ++i) {
        const FptSdfInstruction &op = c.sdf_program[i];
        T d0 = T(op.data[0]), d1 = T(op.data[1]), d2 = T(op.data[2]), d3 = T(op.data[3]);
        switch (op.opcode) {
            case FPT_SDF_OP_ABS:
                jx = jx * signv(p.x); jy = jy * signv(p.y); jz = jz * signv(p.z);
                p = vabs(p); break;
            case FPT_SDF_OP_TRANSLATE: p = p - V3<T>(d0, d1, d2); break;
            case FPT_SDF_OP_SCALE: {
                T sc = std::fabs(d0) > T(1.0e-6f) ? d0 : T(1);
                p = p * sc; jx = jx * sc; jy = jy * sc; jz = jz * sc; scale_acc *= std::fabs(sc); break;
            }
            case FPT_SDF_OP_ROTATE_X: {
                T sn = std::sin(d0), cs = std::cos(d0);
                T py = p.y; V3<T> oy = jy;
                p.y = cs * py - sn * p.z; p.z = sn * py + cs * p.z;
                jy = oy * cs - jz * sn; jz = oy * sn + jz * cs; break;
            }
            case FPT_SDF_OP_ROTATE_Y: {
                T sn = std::sin(d0), cs = std::cos(d0);
                T px = p.x; V3<T> ox = jx;
                p.x = cs * px - sn * p.z; p.z = sn * px + cs * p.z;
                jx = ox * cs - jz * sn; jz = ox * sn + jz * cs; break;
            }
            case FPT_SDF_OP_ROTATE_Z: {
                T sn = std::sin(d0), cs = std::cos(d0);
                T px = p.x; V3<T> ox = jx;
                p.x = cs * px - sn * p.y; p.y = sn * px + cs * p.y;
                jx = ox * cs - jy * sn; jy = ox * sn + jy * cs; break;
            }
            case FPT_SDF_OP_REPEAT: {
                V3<T> per = vmax(vabs(V3<T>(d0, d1, d2)), V3<T>(T(1.0e-5f)));
                p = p - per * vfloor(p / per + T(0.5f));
                break;
            }
            case FPT_SDF_OP_SORT_DESC:
                if (p.x < p.z) { std::swap(p.x, p.z); std::swap(jx, jz); }
                if (p.y < p.z) { std::swap(p.y, p.z); std::swap(jy, jz); }
                if (p.x < p.y) { std::swap(p.x, p.y); std::swap(jx, jy); }
                break;
            case FPT_SDF_OP_SPHERE:
            case FPT_SDF_OP_BOX:
            case FPT_SDF_OP_PLANE: {
                T scale = std::max(scale_acc, T(1.0e-6f));
                T cand; V3<T> lg;
                if (op.opcode == FPT_SDF_OP_SPHERE) {
                    T radius = length(p);
                    cand = (radius - d0) / scale;
                    lg = radius > T(1.0e-8f) ? p / radius : V3<T>(T(0), T(1), T(0));
                } else if (op.opcode == FPT_SDF_OP_BOX) {
                    V3<T> q = vabs(p) - vabs(V3<T>(d0, d1, d2));
                    V3<T> outside = vmax(q, V3<T>(T(0)));
                    T ol = length(outside);
                    cand = (std::min(std::max(q.x, std::max(q.y, q.z)), T(0)) + ol) / scale;
                    if (ol > T(1.0e-8f)) lg = V3<T>(signv(p.x), signv(p.y), signv(p.z)) * outside / ol;
                    else if (q.x >= q.y && q.x >= q.z) lg = V3<T>(signv(p.x), T(0), T(0));
                    else if (q.y >= q.z) lg = V3<T>(T(0), signv(p.y), T(0));
                    else lg = V3<T>(T(0), T(0), signv(p.z));
                } else {
                    lg = normalize(V3<T>(d0, d1, d2));
                    cand = (dot(p, lg) + d3) / scale;
                }
                V3<T> cg = (jx * lg.x + jy * lg.y + jz * lg.z) / scale;
                bool choose = !has || (op.flags == 1u ? cand > s.distance
                                      : (op.flags == 2u ? -cand > s.distance : cand < s.distance));
                if (choose) {
                    s.distance = (op.flags == 2u && has) ? -cand : cand;
                    s.gradient = (op.flags == 2u && has) ? -cg : cg;
                }
                has = true;
                break;
            }
            default: break;
        }
    }
    return s;
}

// shaders/Shaders.metal:3370-3384
template <class T> V3<T> programGradient(T value, const Cfg &c) {
    uint32_t count = std::min<uint32_t>(c.gradient_count, FPT_SDF_GRADIENT_MAX_STOPS);
    if (count == 0u) return V3<T>(T(c.program_material[0]), T(c.program_material[1]), T(c.program_material[2]));
    if (count == 1u) return V3<T>(T(c.gradient_stops[0][1]), T(c.gradient_stops[0][2]), T(c.gradient_stops[0][3]));
    T t = fractv(value);
    const float *prev = c.gradient_stops[0];
    for (uint32_t i = 1; i < count; ++i) {
        const float *cur = c.gradient_stops[i];
        if (t <= T(cur[0])) {
            T f = clampv((t - T(prev[0])) / std::max(T(cur[0]) - T(prev[0]), T(1.0e-6f)), T(0), T(1));
            return vmix(V3<T>(T(prev[1]), T(prev[2]), T(prev[3])), V3<T>(T(cur[1]), T(cur[2]), T(cur[3])), f);
        }
        prev = cur;
    }
    return V3<T>(T(prev[1]), T(prev[2]), T(prev[3]));
}

template <class T> Material<T> programMaterial(T orbit, const Cfg &c) {          // :3386-3402
    Material<T> m;
    if (c.material_mode == 1u) m.rgb = hsv2rgb(V3<T>(orbit * (T(1) + setv<T>(c, 1)) + setv<T>(c, 0), T(0.5f), T(1)));
    else if (c.material_mode == 2u) m.rgb = programGradient(orbit * (T(1) + setv<T>(c, 1)) + setv<T>(c, 0), c);
    else m.rgb = V3<T>(T(c.program_material[0]), T(c.program_material[1]), T(c.program_material[2]));
    m.roughness = T(c.program_material[3]);
    m.specular = T(c.program_material[4]);
    m.translucency = T(c.program_material[5]);
    m.ior = T(c.program_material[6]);
    m.emission = T(c.program_material[7]);
    return m;
}

template <class T> Material<T> fractalMaterial(T orbit, const Cfg &c, bool menger) {   // :3404-3434
    Material<T> m;
    if (c.fractal_style_mode != 0u) {
        T o = orbit * T(c.fractal_style[1]) + T(c.fractal_style[0]);
        if (c.fractal_style_mode == 1u) m.rgb = hsv2rgb(V3<T>(o, T(c.fractal_style[2]), T(c.fractal_style[3])));
        else if (c.fractal_style_mode == 2u)
            m.rgb = V3<T>(T(c.fractal_style[8]), T(c.fractal_style[9]), T(c.fractal_style[10])) * T(c.fractal_style[3]);
        else m.rgb = programGradient(o, c) * T(c.fractal_style[3]);
        V3<T> solid(T(c.fractal_style[8]), T(c.fractal_style[9]), T(c.fractal_style[10]));
        m.rgb = vmix(m.rgb, solid, clampv(T(c.fractal_style[7]), T(0), T(1)));
        m.roughness = T(c.fractal_style[4]);
        m.specular = T(c.fractal_style[5]);
        m.emission = T(c.fractal_style[6]);
        return m;
    }
    if (menger) { m.rgb = V3<T>(T(1)); return m; }
    T o = orbit * (T(1) + setv<T>(c, 1)) + setv<T>(c, 0);
    if (c.sdf_id == FPT_SDF_CAGE_FRACTAL || c.sdf_id == FPT_SDF_IFS_FRACTAL || c.sdf_id == FPT_SDF_TREE_FRACTAL)
        o = orbit * (T(1) + setv<T>(c, 1)) / T(5) + T(0.3f) + setv<T>(c, 0);
    if (c.sdf_id == FPT_SDF_TOWER_FRACTAL) o = orbit * (T(1) + setv<T>(c, 1)) + T(0.3f) + setv<T>(c, 0);
    m.rgb = hsv2rgb(V3<T>(o, T(0.5f), T(1)));
    return m;
}

template <class T> Material<T> mk_mat(float r, float g, float b, float rough, float spec, float trans, float ior, float em) {
    Material<T> m;
    m.rgb = V3<T>(T(r), T(g), T(b));
    m.roughness = T(rough); m.specular = T(spec); m.translucency = T(trans); m.ior = T(ior); m.emission = T(em);
    return m;
}

// ------------------------------------------------------------------ scene dispatch
// Extension field (formula, optionally unioned with the ground plane).
template <class T> DeResult<T> extDistance(V3<T> p, const Cfg &c, const Ext &e, int *surface) {
    DeResult<T> r;
    if (c.sdf_id == FPT_SDF_MANDELBULBER) {
        r = deMandelbulber(p, c, e);
    } else {
        OrbitOut<T> o = orbitEval(e, extIterations(e, c), extBailout(e, c), p);
        r = {o.d, T(o.iterations) / T(std::max(extIterations(e, c), 1))};
    }
    if (surface) *surface = 0;
    if (e.ground_plane) {
        T plane = p.y - T(e.plane_height);
        if (plane < r.d) { r.d = plane; if (surface) *surface = 1; }
    }
    return r;
}

// userSdf: shaders/Shaders.metal:3485-3562
template <class T> Material<T> userMaterial(V3<T> p, const Cfg &c, const Ext &e, T *dist_out = nullptr) {
    if (e.formula != 0) {
        int surface = 0;
        DeResult<T> r = extDistance(p, c, e, &surface);
        if (dist_out) *dist_out = r.d;
        Material<T> m = fractalMaterial(r.orbit, c, false);
        if (e.brdf == FPT_CUDA_BRDF_LAMBERT_GGX) {
            m.rgb = V3<T>(T(surface ? e.plane_albedo : e.albedo));
        }
        m.surface = surface;
        return m;
    }
    if (c.sdf_id == FPT_SDF_PROGRAM && c.sdf_program_count > 0u) {
        DeResult<T> pr = programDistance(p, c, true);
        if (dist_out) *dist_out = pr.d;
        return programMaterial(pr.orbit, c);
    }
    if (c.sdf_id == FPT_SDF_README_CORNELL || c.sdf_id == FPT_SDF_README_GLASS) {
        HitT<T> h = c.sdf_id == FPT_SDF_README_CORNELL ? readmeCornellScene(p) : readmeGlassScene(p);
        if (dist_out) *dist_out = h.d;
        if (h.id == 1) return mk_mat<T>(0.62f, 0.055f, 0.030f, 0.95f, 0, 0, 1.5f, 0.010f);
        if (h.id == 2) return mk_mat<T>(0.035f, 0.82f, 0.09f, 0.92f, 0, 0, 1.5f, 0.010f);
        if (h.id == 3) return mk_mat<T>(1.0f, 0.94f, 0.82f, 1.0f, 0, 0, 1.5f, 12.0f);
        if (h.id == 6) {
            if (c.sdf_id == FPT_SDF_README_GLASS) return mk_mat<T>(0.42f, 0.68f, 0.52f, 0.025f, 1.0f, 0.90f, 1.45f, 0);
            return mk_mat<T>(0.72f, 0.78f, 0.74f, 0.24f, 0.72f, 0, 1.5f, 0.012f);
        }
        if (h.id == 7) return mk_mat<T>(0.84f, 0.88f, 0.86f, 0.45f, 0.24f, 0, 1.5f, 0.018f);
        return mk_mat<T>(0.78f, 0.80f, 0.75f, 0.92f, 0, 0, 1.5f, 0.015f);
    }
    if (c.sdf_id == FPT_SDF_CORNELL_BOX) {
        HitT<T> h = cornellScene(p);
        if (dist_out) *dist_out = h.d;
        if (h.id == 1) return mk_mat<T>(0.82f, 0.12f, 0.08f, 1, 0, 0, 1.5f, 0);
        if (h.id == 2) return mk_mat<T>(0.10f, 0.55f, 0.18f, 1, 0, 0, 1.5f, 0);
        if (h.id == 3) return mk_mat<T>(1.0f, 0.88f, 0.64f, 1, 0, 0, 1.5f, 7.0f);
        if (h.id == 4) return mk_mat<T>(0.72f, 0.70f, 0.64f, 0.82f, 0, 0, 1.5f, 0);
        if (h.id == 5) return mk_mat<T>(0.70f, 0.68f, 0.62f, 0.92f, 0, 0, 1.5f, 0);
        return mk_mat<T>(0.82f, 0.80f, 0.74f, 1, 0, 0, 1.5f, 0);
    }
    if (c.sdf_id == FPT_SDF_GLASS_BALL) {
        HitT<T> h = glassBallScene(p);
        if (dist_out) *dist_out = h.d;
        if (h.id == 1) return mk_mat<T>(0.92f, 0.97f, 1.0f, 0.02f, 1.0f, 1.0f, 1.5f, 0);
        if (h.id == 2) return mk_mat<T>(0.48f, 0.58f, 0.72f, 0.85f, 0, 0, 1.5f, 0);
        if (h.id == 3) return mk_mat<T>(1.0f, 0.92f, 0.78f, 1, 0, 0, 1.5f, 5.5f);
        return mk_mat<T>(0.70f, 0.68f, 0.62f, 0.72f, 0.08f, 0, 1.5f, 0);
    }
    DeResult<T> de{T(1000), T(0)};
    bool menger = false;
    switch (c.sdf_id) {
        case FPT_SDF_BALL_FRACTAL: de = deBall(p, c); break;
        case FPT_SDF_CAGE_FRACTAL: de = deCage(p, c); break;
        case FPT_SDF_IFS_FRACTAL: de = deIFS(p, c); break;
        case FPT_SDF_MANDELBOX_FRACTAL: de = deMandelbox(p, c); break;
        case FPT_SDF_MENGER_SPONGE: de = deMenger(p, c); menger = true; break;
        case FPT_SDF_TOWER_FRACTAL: de = deTower(p, c); break;
        case FPT_SDF_TREE_FRACTAL: de = deTree(p, c); break;
        case FPT_SDF_MANDELBULBER: de = deMandelbulber(p, c, e); break;
        default: break;
    }
    if (dist_out) *dist_out = de.d;
    return fractalMaterial(de.orbit, c, menger);
}

// distanceSdf: shaders/Shaders.metal:3564-3610 (interpreted program path).
template <class T> T distanceSdf(V3<T> p, const Cfg &c, const Ext &e) {
    if (e.formula != 0) return extDistance(p, c, e, nullptr).d;
    if (c.sdf_id == FPT_SDF_PROGRAM && c.sdf_program_count > 0u) return programDistance(p, c, false).d;
    if (c.sdf_id == FPT_SDF_README_CORNELL) return readmeCornellScene(p).d;
    if (c.sdf_id == FPT_SDF_README_GLASS) return readmeGlassScene(p).d;
    if (c.sdf_id == FPT_SDF_CORNELL_BOX) return cornellScene(p).d;
    if (c.sdf_id == FPT_SDF_GLASS_BALL) return glassBallScene(p).d;
    switch (c.sdf_id) {
        case FPT_SDF_BALL_FRACTAL: return deBall(p, c).d;
        case FPT_SDF_CAGE_FRACTAL: return deCage(p, c).d;
        case FPT_SDF_IFS_FRACTAL: return deIFS(p, c).d;
        case FPT_SDF_MANDELBOX_FRACTAL: return deMandelbox(p, c).d;
        case FPT_SDF_MENGER_SPONGE: return deMenger(p, c).d;
        case FPT_SDF_TOWER_FRACTAL: return deTower(p, c).d;
        case FPT_SDF_TREE_FRACTAL: return deTree(p, c).d;
        case FPT_SDF_MANDELBULBER: return deMandelbulber(p, c, e).d;
        default: return T(1000);
    }
}
template <class T> inline T mapSdf(V3<T> p, const Cfg &c, const Ext &e) {         // :3612-3615
    T d = distanceSdf(p, c, e);
    return mixv(d, d / T(2), T(c.render[6]));
}
inline bool hasTranslucent(const Cfg &c, const Ext &e) {                           // :3617-3624
    if (e.formula != 0) return false;
    return c.sdf_id == FPT_SDF_GLASS_BALL || c.sdf_id == FPT_SDF_README_GLASS ||
           (c.sdf_id == FPT_SDF_PROGRAM && c.program_material[5] > 0.0f);
}
inline int iterationLimit(int req, const Cfg &c) {                                 // :3626-3633
    return std::min(req, c.sdf_id == FPT_SDF_MANDELBULBER ? 10000 : 360);
}
template <class T> T mandelbulberThreshold(V3<T> p, const Cfg &c) {               // :3635-3641
    T th = c.vset_values[115] > 0.5f ? length(cameraPos<T>(c) - p) * T(c.vset_values[116]) : T(c.vset_values[117]);
    return clampv(th, T(c.vset_values[118]), T(c.vset_values[119]));
}
template <class T> T marchStep(T d, T th, const Cfg &c) {                          // :3643-3681
    if (c.sdf_id == FPT_SDF_MANDELBULBER) {
        T step = std::max(d - T(0.5f) * th, T(0)) * T(c.vset_values[113]);
        if (c.vset_values[108] > 0.5f) {
            step = clampv(step, T(c.vset_values[109]), T(c.vset_values[110]));
            if (th > T(c.vset_values[109])) step = clampv(step, T(c.vset_values[111]) * th, T(c.vset_values[112]) * th);
        } else {
            step = std::min(step, T(c.vset_values[110]));
        }
        return step;
    }
    return std::fabs(d) * T(0.99f);
}

template <class T> struct MarchOut { V3<T> pos; bool found; int steps; };

// marchMandelbulber: shaders/Shaders.metal:3700-3751.  With fp64 set, the
// refinement bisects in double precision (extension (1): FP64 at the
// representable-position stop).
template <class T> MarchOut<T> marchMandelbulber(V3<T> dir, V3<T> pos, int iters, const Cfg &c, const Ext &e) {
    V3<T> start = pos;
    T distance = T(0), th = mandelbulberThreshold(pos, c), step = T(0);
    bool found = false;
    int steps = 0;
    int maxi = iterationLimit(iters, c);
    for (int it = 0; it < maxi; ++it) {
        th = mandelbulberThreshold(pos, c);
        distance = mapSdf(pos, c, e);
        ++steps;
        if (!std::isfinite(distance)) break;
        if (distance < th) { found = true; break; }
        step = marchStep(distance, th, c);
        V3<T> next = pos + dir * step;
        if (next.x == pos.x && next.y == pos.y && next.z == pos.z) break;
        pos = next;
        if (length(pos - start) >= T(c.render[4])) break;
    }
    if (!found) return {pos, false, steps};
    T limit = T(1) - T(0.001f) * std::max(T(c.vset_values[129]), T(0));
    step = step * T(0.5f);
    for (int r = 0; r < 30; ++r) {
        if (distance < th && distance > th * limit) break;
        if (distance > th) {
            V3<T> next = pos + dir * step;
            if (next.x == pos.x && next.y == pos.y && next.z == pos.z) break;
            pos = next;
        } else if (distance < th * limit) {
            V3<T> next = pos - dir * step;
            if (next.x == pos.x && next.y == pos.y && next.z == pos.z) break;
            pos = next;
        }
        distance = mapSdf(pos, c, e);
        ++steps;
        step = step * T(0.5f);
    }
    return {pos, true, steps};
}

// march: shaders/Shaders.metal:3753-3783.  `found` reports convergence.
template <class T> MarchOut<T> march(V3<T> dr, V3<T> rp, int ni, T min_dist, T lod_falloff, const Cfg &c, const Ext &e) {
    if (c.sdf_id == FPT_SDF_MANDELBULBER) return marchMandelbulber(dr, rp, ni, c, e);
    V3<T> cam = rp;
    int maxi = iterationLimit(ni, c);
    bool translucent = hasTranslucent(c, e);
    int steps = 0;
    bool found = false;
    for (int i = 0; i < maxi; i++) {
        T d = mapSdf(rp, c, e);
        ++steps;
        if (!std::isfinite(d)) break;
        T th = min_dist;
        T o = marchStep(d, th, c);
        rp = rp + dr * o;
        T lod = th;
        if (lod_falloff > T(0.00001f)) {
            T fog = dot(cam - rp, cam - rp);
            lod = mixv(lod, T(0.1f), fog * lod_falloff);
            lod = mixv(th, lod, T(c.render[5]));
        }
        if (translucent && userMaterial(rp, c, e).translucency > T(0)) lod = T(0.0001f);
        if (o < lod) { found = true; break; }
        if (T(c.render[4]) < o) break;
    }
    return {rp, found, steps};
}

// normalizeFiniteDifference: shaders/Shaders.metal:3863-3869
template <class T> V3<T> normalizeFD(V3<T> g) {
    T m = std::max(std::fabs(g.x), std::max(std::fabs(g.y), std::fabs(g.z)));
    if (!(m > T(0)) || !std::isfinite(m)) return V3<T>(T(0), T(1), T(0));
    return normalize(g / m);
}

template <class T> T mandelNormalDistance(V3<T> p, const Cfg &c, const Ext &e) {  // :956-960
    int mult = c.vset_values[115] > 1.5f ? 5 : 1;
    return fieldSample(p, c, e, mult).d;
}
template <class T> T mandelNormalOrbitRadius(V3<T> p, const Cfg &c, const Ext &e) {   // :962-968
    int mult = c.vset_values[115] > 1.5f ? 5 : 1;
    return std::log(std::max(std::fabs(fieldSample(p, c, e, mult).r), T(1.0e-30f)));
}

// Gradient of the extension distance by forward-mode dual numbers (always
// evaluated in FP64): the analytic-derivative normal.
inline V3<double> extGradient(V3<double> p, const Cfg &c, const Ext &e) {
    V3<Dual> q(Dual::var(p.x, 0), Dual::var(p.y, 1), Dual::var(p.z, 2));
    Dual d = extDistance(q, c, e, nullptr).d;
    return V3<double>(d.d[0], d.d[1], d.d[2]);
}

// normalAt: shaders/Shaders.metal:3871-3971 (+ the analytic extension mode).
template <class T> V3<T> normalAt(V3<T> p, const Cfg &c, const Ext &e) {
    bool mandel = c.sdf_id == FPT_SDF_MANDELBULBER;
    if (e.formula != 0 && e.normal_mode == FPT_CUDA_NORMAL_ANALYTIC) {
        V3<double> g = extGradient(V3<double>(double(p.x), double(p.y), double(p.z)), c, e);
        V3<T> gt(T(g.x), T(g.y), T(g.z));
        if (finite3(gt) && dot(gt, gt) > T(0)) return normalize(gt);
        return V3<T>(T(0), T(1), T(0));
    }
    if (mandel && c.render[7] > 0.0f) {
        T delta = length(cameraPos<T>(c) - p) * T(c.render[7]) * T(c.vset_values[114]);
        T maxit = T(c.set_values[1]);
        V3<T> sn(T(0));
        for (int ix = -5; ix <= 5; ++ix)
            for (int iy = -5; iy <= 5; ++iy)
                for (int iz = -5; iz <= 5; ++iz) {
                    V3<T> sd = V3<T>(T(ix), T(iy), T(iz)) * T(0.2f);
                    Field4<T> s = fieldSample(p + sd * delta, c, e, 1);
                    T pd = T(1) + maxit - std::fabs(s.state);
                    sn = sn + sd * pd;
                }
        T m = std::max(std::fabs(sn.x), std::max(std::fabs(sn.y), std::fabs(sn.z)));
        if (!(m > T(0)) || !std::isfinite(m)) return V3<T>(T(1), T(0), T(0));
        return normalize(sn / m);
    }
    T eps = mandel ? mandelbulberThreshold(p, c) * T(c.vset_values[114]) : std::max(T(c.render[2]), T(0.0002f));
    if ((c.sdf_normal_mode == 0u || c.sdf_normal_mode == 2u) && c.sdf_id == FPT_SDF_PROGRAM && c.sdf_program_count > 0u &&
        e.formula == 0) {
        V3<T> g = programSurface(p, c).gradient;
        if (dot(g, g) >= T(1.0e-12f) && finite3(g)) return normalize(g);
    }
    auto D = [&](V3<T> q) { return mandel ? mandelNormalDistance(q, c, e) : mapSdf(q, c, e); };
    if (c.sdf_normal_mode == 1u) {
        T te = eps * T(0.57735026919f);
        V3<T> k0(T(1), T(-1), T(-1)), k1(T(-1), T(-1), T(1)), k2(T(-1), T(1), T(-1)), k3(T(1), T(1), T(1));
        T d0 = D(p + k0 * te), d1 = D(p + k1 * te), d2 = D(p + k2 * te), d3 = D(p + k3 * te);
        return normalizeFD(k0 * d0 + k1 * d1 + k2 * d2 + k3 * d3);
    }
    V3<T> xo(eps, T(0), T(0)), yo(T(0), eps, T(0)), zo(T(0), T(0), eps);
    V3<T> n(D(p + xo) - D(p - xo), D(p + yo) - D(p - yo), D(p + zo) - D(p - zo));
    if (mandel && !(std::max(std::fabs(n.x), std::max(std::fabs(n.y), std::fabs(n.z))) > T(0))) {
        n = V3<T>(mandelNormalOrbitRadius(p + xo, c, e) - mandelNormalOrbitRadius(p - xo, c, e),
                  mandelNormalOrbitRadius(p + yo, c, e) - mandelNormalOrbitRadius(p - yo, c, e),
                  mandelNormalOrbitRadius(p + zo, c, e) - mandelNormalOrbitRadius(p - zo, c, e));
    }
    return normalizeFD(n);
}

// ------------------------------------------------------------------ environment
template <class T> T preetham(V3<T> dr, V3<T> sun) {                             // :5764-5774
    T Tt = T(2);
    T A = T(0.1787f) * Tt - T(1.4630f), B = T(-0.3554f) * Tt + T(0.4275f), C = T(-0.0227f) * Tt + T(5.3251f);
    T D = T(0.1206f) * Tt - T(2.5771f), E = T(-0.0670f) * Tt + T(0.3703f);
    T theta = std::acos(clampv(dr.y, T(-1), T(1)));
    T gamma = std::acos(clampv(dot(dr, sun), T(-1), T(1)));
    return (T(1) + A * std::exp(B / std::max(T(0.1f), std::cos(theta)))) *
           (T(1) + C * std::exp(D * gamma) + E * std::pow(std::cos(gamma), T(2)));
}
template <class T> V3<T> sky(V3<T> dr, V3<T> sun) {                              // :5776-5787
    T sk = preetham(dr, sun);
    V3<T> col = vmix(V3<T>(T(0.004f), T(0.048f), T(0.253f)), V3<T>(T(0.8f), T(0.9f), T(1.0f)), sk);
    T hd = (dr.y + T(1)) / T(2), hs = (sun.y + T(1)) / T(2);
    col = vmix(V3<T>(T(1.0f), T(0.85f), T(0.53f)) / T(4), col * T(1.2f), hd) * hs;
    col = (col - T(0.5f)) * T(1.2f) + T(0.5f);
    T disk = std::max((dot(dr, sun) - T(1)) / (T(1) - std::cos(T(0.05f))) + T(1), T(0));
    disk *= std::pow(hd, T(10));
    return col * T(0.8f) + V3<T>(disk * T(100));
}
template <class T> V3<T> backgroundGradient(V3<T> d, const Cfg &c) {             // :5789-5794
    T t = clampv((d.y + T(1)) / T(2), T(0), T(1));
    V3<T> a(T(c.background_gradient[0]), T(c.background_gradient[1]), T(c.background_gradient[2]));
    V3<T> b(T(c.background_gradient[3]), T(c.background_gradient[4]), T(c.background_gradient[5]));
    return vmix(b, a, t);
}
inline float halfToFloat(uint16_t h) {
    uint32_t sign = uint32_t(h & 0x8000u) << 16, exp = (h >> 10) & 0x1fu, man = h & 0x3ffu;
    uint32_t bits;
    if (exp == 0) {
        if (man == 0) bits = sign;
        else { int e = -1; do { man <<= 1; ++e; } while (!(man & 0x400u)); bits = sign | uint32_t(127 - 15 - e) << 23 | (man & 0x3ffu) << 13; }
    } else if (exp == 31) bits = sign | 0x7f800000u | man << 13;
    else bits = sign | (exp + 112u) << 23 | man << 13;
    return bits_float(bits);
}
template <class T> V3<T> sampleHdriLut(V3<T> direction, const Cfg &c) {          // :5803-5821
    uint32_t w = clampv<uint32_t>(c.hdri_width, 1u, 32u), h = clampv<uint32_t>(c.hdri_height, 1u, 16u);
    auto ch = [&](uint32_t x, uint32_t y, uint32_t k) {
        uint32_t idx = (std::min(y, h - 1u) * w + std::min(x, w - 1u)) * 3u + k;
        return T(halfToFloat(c.hdri_lut[idx]));
    };
    V3<T> d = normalize(direction);
    T u = fractv(std::atan2(d.z, d.x) / (T(2) * T(kPi)) + T(0.5f));
    T v = clampv(std::acos(clampv(d.y, T(-1), T(1))) / T(kPi), T(0), T(1));
    T x = u * T(w) - T(0.5f);
    T y = v * T(h - 1u);
    int x0i = int(std::floor(x));
    uint32_t x0 = uint32_t((x0i % int(w) + int(w)) % int(w));
    uint32_t x1 = (x0 + 1u) % w;
    uint32_t y0 = uint32_t(clampv(int(std::floor(y)), 0, int(h - 1u)));
    uint32_t y1 = std::min(y0 + 1u, h - 1u);
    T fx = fractv(x), fy = fractv(y);
    V3<T> c00(ch(x0, y0, 0), ch(x0, y0, 1), ch(x0, y0, 2)), c10(ch(x1, y0, 0), ch(x1, y0, 1), ch(x1, y0, 2));
    V3<T> c01(ch(x0, y1, 0), ch(x0, y1, 1), ch(x0, y1, 2)), c11(ch(x1, y1, 0), ch(x1, y1, 1), ch(x1, y1, 2));
    return vmix(vmix(c00, c10, fx), vmix(c01, c11, fx), fy);
}
// Full-resolution equirect sky of the extension (same u/v convention as the
// reference LUT, texel-centre bilinear, x wraps, y clamps).
template <class T> V3<T> sampleEquirect(V3<T> direction, const Ext &e) {
    uint32_t w = e.sky_width, h = e.sky_height;
    V3<T> d = normalize(direction);
    T u = fractv(std::atan2(d.z, d.x) / (T(2) * T(kPi)) + T(0.5f));
    T v = clampv(std::acos(clampv(d.y, T(-1), T(1))) / T(kPi), T(0), T(1));
    T x = u * T(w) - T(0.5f), y = v * T(h) - T(0.5f);
    int x0i = int(std::floor(x));
    uint32_t x0 = uint32_t((x0i % int(w) + int(w)) % int(w)), x1 = (x0 + 1u) % w;
    int y0i = clampv(int(std::floor(y)), 0, int(h) - 1);
    uint32_t y0 = uint32_t(y0i), y1 = std::min(y0 + 1u, h - 1u);
    T fx = fractv(x), fy = y < T(0) ? T(0) : fractv(y);
    auto px = [&](uint32_t X, uint32_t Y) {
        const float *s = e.sky_rgb + (size_t(Y) * w + X) * 3u;
        return V3<T>(T(s[0]), T(s[1]), T(s[2]));
    };
    return vmix(vmix(px(x0, y0), px(x1, y0), fx), vmix(px(x0, y1), px(x1, y1), fx), fy);
}
template <class T> V3<T> environment(V3<T> view, const Cfg &c, const Ext &e) {   // :5823-5844
    if (e.sky_width > 0 && e.sky_rgb) return sampleEquirect(view, e) * T(c.world[4]);
    if (c.world[4] < 0.00001f) return V3<T>(T(0));
    V3<T> ld = rotateCamera(V3<T>(T(0), T(0), T(1)), T(c.world[2]) * T(kPi) / T(180), T(c.world[3]) * T(kPi) / T(180));
    V3<T> env(T(0));
    if (c.world[0] == 0.0f) {
        T ls = std::max(T(c.world[1]), T(0.0001f));
        T light = std::max((dot(view, ld) - T(1)) / (T(1) - std::cos(ls)) + T(1), T(0)) / ls * T(3);
        env = V3<T>(light);
    } else if (c.world[0] == 1.0f) {
        env = sky(view, ld);
    } else if (c.world[0] == 2.0f && c.hdri_enabled != 0u && c.hdri_width > 0u) {
        env = sampleHdriLut(rotateCamera(view, T(c.world[2]) * T(kPi) / T(180), T(0)), c);
    } else if (c.world[0] == 3.0f) {
        env = V3<T>(T(c.world_one_color[0]), T(c.world_one_color[1]), T(c.world_one_color[2]));
    } else {
        env = V3<T>(T(1));
    }
    T power = T(c.world[4]);
    T contrast = c.world[0] == 3.0f ? T(1) : T(c.world[5]);
    return vmax(env * power - V3<T>(T(0.5f)) * contrast + V3<T>(T(0.5f)), V3<T>(T(0)));
}

template <class T> V3<T> sunDirection(const PathRng &rng, int bounce, const Cfg &c, const Ext &e) {
    V3<T> ld;
    if (e.sun_intensity > 0.0f) ld = normalize(V3<T>(T(e.sun_direction[0]), T(e.sun_direction[1]), T(e.sun_direction[2])));
    else ld = rotateCamera(V3<T>(T(0), T(0), T(1)), T(c.sun[1]) * T(kPi) / T(180), T(c.sun[2]) * T(kPi) / T(180));
    T h1 = T(rng.uniform(SLOT_SUN0, bounce)), h2 = T(rng.uniform(SLOT_SUN1, bounce));
    T a = h1 * T(2) * T(kPi);
    T s = std::sqrt(h2) * T(c.sun[4]);
    return rotateCamera(ld, std::cos(a) * s, std::sin(a) * s);
}

// sunContributionWithSurface: shaders/Shaders.metal:5846-5861 (visibility part).
template <class T> bool sunVisible(V3<T> rp, V3<T> n, V3<T> ld, const Cfg &c, const Ext &e, int *steps) {
    V3<T> rp0 = rp;
    rp = rp + n * T(0.001f);
    MarchOut<T> m = march(ld, rp, int(c.render[1]), T(c.render[3]), T(0.0002f), c, e);
    if (steps) *steps += m.steps;
    return length(rp0 - m.pos) > T(c.render[4]) * T(0.99f);
}

// estimateFocusDistance: shaders/Shaders.metal:5869-5878
template <class T> T estimateFocus(const Cfg &c, const Ext &e) {
    T f = T(1) / std::tan(T(c.camera_fov) / T(2) * T(kPi) / T(180));
    V3<T> dr = rotateCamera(normalize(V3<T>(T(0), T(0), f)), T(c.camera_yaw_pitch[0]), T(c.camera_yaw_pitch[1]), T(c.camera_roll));
    MarchOut<T> m = march(dr, cameraPos<T>(c), 120, T(0.001f), T(0.001f), c, e);
    T d = length(m.pos - cameraPos<T>(c));
    if (!std::isfinite(d) || d <= T(0.001f) || d > T(c.render[4]) * T(0.99f)) return T(5);
    return d;
}

// Mandelbulber projection helpers: shaders/Shaders.metal:438-471
template <class T> bool mandelVisible(T x, T y, const Cfg &c) {
    if (c.vset_values[107] < 2.5f || c.vset_values[107] > 3.5f) return true;
    T fov = T(c.camera_fov) * T(kPi) / T(180);
    return std::sqrt(x * x + y * y) <= (T(0.5f) * T(kPi) / std::max(fov, T(1.0e-6f)));
}
template <class T> V3<T> mandelCameraRay(T x, T y, const Cfg &c) {
    T proj = T(c.vset_values[107]);
    T fov = T(c.camera_fov) * T(kPi) / T(180);
    V3<T> ld;
    if ((proj > T(0.5f) && proj < T(1.5f)) || (proj > T(2.5f) && proj < T(3.5f))) {
        T radius = std::sqrt(x * x + y * y);
        if (radius <= T(1.0e-8f)) ld = V3<T>(T(0), T(0), T(1));
        else { T rs = std::sin(radius * fov) / radius; ld = V3<T>(x * rs, y * rs, std::cos(radius * fov)); }
    } else if (proj > T(1.5f) && proj < T(2.5f)) {
        T aspect = T(c.width) / T(c.height);
        T ax = x * (T(2) / aspect) * (T(0.5f) * fov), ay = y * (T(0.5f) * fov);
        ld = V3<T>(std::sin(ax) * std::cos(ay), std::sin(ay), std::cos(ax) * std::cos(ay));
    } else {
        T fl = T(1) / std::tan(T(0.5f) * fov);
        ld = normalize(V3<T>(x, y, fl));
    }
    return rotateCamera(normalize(ld), T(c.camera_yaw_pitch[0]), T(c.camera_yaw_pitch[1]), T(c.camera_roll));
}

// sdfScreenUv: shaders/Shaders.metal:6847-6855 (float arithmetic on purpose:
// its bits seed hash13).
inline V2<float> screenUv(uint32_t gx, uint32_t gy, const Cfg &c) {
    float ox = c.sdf_id == FPT_SDF_MANDELBULBER ? 0.0f : 0.5f;
    float oy = c.sdf_id == FPT_SDF_MANDELBULBER ? 1.0f : 0.5f;
    float u = (float(gx) + ox) / float(c.width) - 0.5f;
    float v = (float(gy) + oy) / float(c.height) - 0.5f;
    u *= float(c.width) / float(c.height);
    return {u, v};
}

template <class T> struct PathStats { int primary_steps = 0, shadow_steps = 0, bounces = 0; };

// Camera ray of renderPath: shaders/Shaders.metal:5926-5956.
template <class T> bool cameraRay(V2<float> uv, const PathRng &rng, bool jitter, T focus, const Cfg &c, V3<T> &rp, V3<T> &dr) {
    rp = cameraPos<T>(c);
    T aa = T(0.3f) / std::max(T(c.width), T(c.height));
    V2<T> cs{T(uv.x), T(uv.y)};
    if (jitter) {
        V2<T> j = randomPoint(aa, T(rng.uniform(SLOT_LENS0, 0)), T(rng.uniform(SLOT_LENS1, 0)));
        cs.x = cs.x + j.x; cs.y = cs.y + j.y;
    }
    if (c.sdf_id == FPT_SDF_MANDELBULBER) {
        if (!mandelVisible(cs.x, cs.y, c)) return false;
        dr = mandelCameraRay(cs.x, cs.y, c);
    } else {
        dr = rotateCamera(normalize(V3<T>(cs.x, cs.y, T(1) / std::tan(T(c.camera_fov) / T(2) * T(kPi) / T(180)))),
                          T(c.camera_yaw_pitch[0]), T(c.camera_yaw_pitch[1]), T(c.camera_roll));
    }
    if (jitter && c.camera_dof > 0.0f) {
        V3<T> fp = rp + dr * focus;
        V2<T> lens = randomPoint(T(c.camera_dof), T(rng.uniform(SLOT_LENS0, 0)), T(rng.uniform(SLOT_LENS1, 0)));
        rp = rp + rotateCamera(V3<T>(lens.x, lens.y, T(0)), T(c.camera_yaw_pitch[0]), T(c.camera_yaw_pitch[1]), T(c.camera_roll));
        dr = normalize(fp - rp);
    }
    return true;
}

// ------------------------------------------------------------------ extension BRDF
// Lambert + GGX (Trowbridge-Reitz) microfacet lobe with Schlick Fresnel and
// the height-correlated Smith masking term (Heitz, JCGT 2014); sampling draws
// the lobe with probability 1/2 each and uses the visible-normal sampling of
// Heitz, "Sampling the GGX Distribution of Visible Normals" (JCGT 2018).
template <class T> struct Frame { V3<T> t, b, n; };
template <class T> Frame<T> makeFrame(V3<T> n) {
    // Duff et al., "Building an Orthonormal Basis, Revisited" (JCGT 2017).
    T s = n.z >= T(0) ? T(1) : T(-1);
    T a = T(-1) / (s + n.z);
    T b = n.x * n.y * a;
    return {V3<T>(T(1) + s * n.x * n.x * a, s * b, -s * n.x), V3<T>(b, s + n.y * n.y * a, -n.y), n};
}
template <class T> inline V3<T> toLocal(const Frame<T> &f, V3<T> v) { return {dot(v, f.t), dot(v, f.b), dot(v, f.n)}; }
template <class T> inline V3<T> toWorld(const Frame<T> &f, V3<T> v) { return f.t * v.x + f.b * v.y + f.n * v.z; }
template <class T> inline T ggxD(T nh, T a) { T a2 = a * a; T d = nh * nh * (a2 - T(1)) + T(1); return a2 / (T(kPi) * d * d); }
template <class T> inline T smithLambda(T cosv, T a) {
    T c2 = cosv * cosv; T t2 = std::max(T(1) - c2, T(0)) / std::max(c2, T(1e-12f));
    return (std::sqrt(T(1) + a * a * t2) - T(1)) * T(0.5f);
}
template <class T> inline T schlick(T f0, T c) { return f0 + (T(1) - f0) * pow5(T(1) - c); }

// BRDF value times cos(theta_l), and the mixture pdf of sampling l.
template <class T> void brdfEval(V3<T> v, V3<T> l, T albedo, T alpha, T f0, bool plane, V3<T> &f_cos, T &pdf) {
    T nl = l.z, nv = v.z;
    if (nl <= T(0) || nv <= T(0)) { f_cos = V3<T>(T(0)); pdf = T(0); return; }
    T diffuse = albedo / T(kPi);
    if (plane) { f_cos = V3<T>(diffuse * nl); pdf = nl / T(kPi); return; }
    V3<T> h = normalize(v + l);
    T D = ggxD(h.z, alpha);
    T G = T(1) / (T(1) + smithLambda(nv, alpha) + smithLambda(nl, alpha));
    T F = schlick(f0, std::max(dot(v, h), T(0)));
    T spec = D * G * F / (T(4) * nv * nl);
    f_cos = V3<T>((diffuse * (T(1) - F) + spec) * nl);
    T g1v = T(1) / (T(1) + smithLambda(nv, alpha));
    T pdf_spec = g1v * D / (T(4) * nv);      // VNDF pdf of l = reflect(-v, h)
    pdf = T(0.5f) * nl / T(kPi) + T(0.5f) * pdf_spec;
}
// Heitz 2018 visible-normal sample (isotropic alpha), local frame.
template <class T> V3<T> sampleVndf(V3<T> v, T alpha, T u1, T u2) {
    V3<T> vh = normalize(V3<T>(alpha * v.x, alpha * v.y, v.z));
    T lensq = vh.x * vh.x + vh.y * vh.y;
    V3<T> t1 = lensq > T(0) ? V3<T>(-vh.y, vh.x, T(0)) / std::sqrt(lensq) : V3<T>(T(1), T(0), T(0));
    V3<T> t2 = cross(vh, t1);
    T r = std::sqrt(u1);
    T phi = T(2) * T(kPi) * u2;
    T p1 = r * std::cos(phi), p2 = r * std::sin(phi);
    T s = T(0.5f) * (T(1) + vh.z);
    p2 = (T(1) - s) * std::sqrt(std::max(T(1) - p1 * p1, T(0))) + s * p2;
    V3<T> nh = t1 * p1 + t2 * p2 + vh * std::sqrt(std::max(T(0), T(1) - p1 * p1 - p2 * p2));
    return normalize(V3<T>(alpha * nh.x, alpha * nh.y, std::max(T(0), nh.z)));
}

// ------------------------------------------------------------------ path
// renderPath: shaders/Shaders.metal:5926-6026; with ext.brdf set, the
// Lambert+GGX estimator above with standard throughput weighting.
template <class T> V3<T> renderPath(V2<float> uv, uint32_t pixel, uint32_t sample, T focus, const Cfg &c, const Ext &e,
                                    PathStats<T> *st) {
    PathRng rng{e.rng == FPT_CUDA_RNG_PCG, e.seed, pixel, sample, uv.x, uv.y, float(sample)};
    V3<T> cam = cameraPos<T>(c), rp, dr;
    if (!cameraRay(uv, rng, true, focus, c, rp, dr)) return V3<T>(T(0));
    int local_ni = int(c.render[1]);
    T side = T(1);
    V3<T> light(T(0)), color(T(1));
    T sky_mask = T(0);
    V3<T> grad = backgroundGradient(dr, c);
    int bounces = std::min(int(c.render[0]), 8);
    if (c.sdf_bounce_cap > 0u) bounces = std::min(bounces, int(c.sdf_bounce_cap));
    T maxd = T(c.render[4]), maxd2 = maxd * maxd, far = maxd * T(0.99f), far2 = far * far;
    const bool ggx = e.brdf == FPT_CUDA_BRDF_LAMBERT_GGX;
    for (int i = 0; i < bounces; i++) {
        MarchOut<T> m = march(dr, rp, local_ni, T(c.render[3]), T(0.0002f), c, e);
        rp = m.pos;
        if (st) { st->primary_steps += m.steps; st->bounces = i + 1; }
        T travel2 = dot(rp - cam, rp - cam);
        if (i == 0 && travel2 > maxd2) sky_mask = T(1);
        local_ni = int(c.render[1] / (c.render[5] * 2.0f + 1.0f));
        if (travel2 > far2) {
            V3<T> env = environment(dr, c, e);
            light = light + (ggx ? env * color : env);
            break;
        }
        Material<T> mat = userMaterial(rp, c, e);
        V3<T> n = normalAt(rp, c, e);
        if (ggx) {
            // Extension estimator: emission and sun NEE weighted by throughput.
            if (mat.emission > T(0.001f)) light = light + mat.rgb * mat.emission * color;
            V3<T> v = -dr;
            if (dot(n, v) < T(0)) n = -n;
            Frame<T> fr = makeFrame(n);
            V3<T> vl = toLocal(fr, v);
            T albedo = mat.rgb.x, alpha = T(e.ggx_alpha), f0 = T(e.specular_f0);
            bool plane = mat.surface == 1;
            if (c.sun[0] == 1.0f || e.sun_intensity > 0.0f) {
                V3<T> ld = sunDirection<T>(rng, i, c, e);
                int ss = 0;
                if (dot(ld, n) > T(0) && sunVisible(rp, n, ld, c, e, &ss)) {
                    V3<T> fc; T pdf;
                    brdfEval(vl, toLocal(fr, ld), albedo, alpha, f0, plane, fc, pdf);
                    T power = e.sun_intensity > 0.0f ? T(e.sun_intensity) : T(c.sun[3]);
                    light = light + fc * color * V3<T>(T(c.sun_color[0]), T(c.sun_color[1]), T(c.sun_color[2])) * power;
                }
                if (st) st->shadow_steps += ss;
            }
            T u1 = T(rng.uniform(SLOT_DIR0, i)), u2 = T(rng.uniform(SLOT_DIR1, i));
            V3<T> ll;
            if (plane || T(rng.uniform(SLOT_LOBE, i)) < T(0.5f)) {
                T r = std::sqrt(u1), phi = T(2) * T(kPi) * u2;
                ll = V3<T>(r * std::cos(phi), r * std::sin(phi), std::sqrt(std::max(T(0), T(1) - u1)));
            } else {
                V3<T> h = sampleVndf(vl, alpha, u1, u2);
                ll = vreflect(-vl, h);
            }
            V3<T> fc; T pdf;
            brdfEval(vl, ll, albedo, alpha, f0, plane, fc, pdf);
            if (!(pdf > T(0))) break;
            color = color * (fc / pdf);
            dr = normalize(toWorld(fr, ll));
            rp = rp + n * (T(0.001f) * signv(dot(dr, n)));
        } else {
            if (mat.emission > T(0.001f)) light = light + mat.rgb * mat.emission;
            if (c.sun[0] == 1.0f) {
                V3<T> ld = sunDirection<T>(rng, i, c, e);
                int ss = 0;
                if (sunVisible(rp, n, ld, c, e, &ss))
                    light = light + V3<T>(T(c.sun_color[0]), T(c.sun_color[1]), T(c.sun_color[2])) *
                                        (T(c.sun[3]) * std::max(dot(n, ld), T(0)) * mat.roughness * (T(1) - mat.translucency));
                if (st) st->shadow_steps += ss;
            }
            T r1 = T(rng.uniform(SLOT_SCATTER, i)), r2 = T(rng.uniform(SLOT_FRESNEL, i));
            if (r1 > mat.translucency) {
                V3<T> metal = vreflect(dr, n);
                V3<T> diffuse = randomVector(n, T(rng.uniform(SLOT_DIR0, i)), T(rng.uniform(SLOT_DIR1, i)));
                T f0 = std::pow((mat.ior - T(1)) / (mat.ior + T(1)), T(2));
                T ct = clampv(dot(n, -dr), T(0), T(1));
                T fres = f0 + (T(1) - f0) * pow5(T(1) - ct);
                dr = normalize(vmix(metal, diffuse, mat.roughness));
                if (r2 < fres * mat.specular) dr = metal;
                else color = color * mat.rgb;
            } else {
                T eta = side == T(1) ? T(1) / mat.ior : mat.ior;
                if (side != T(1)) n = -n;
                T f0 = std::pow((mat.ior - T(1)) / (mat.ior + T(1)), T(2));
                T ct = clampv(dot(n, -dr), T(0), T(1));
                T fres = f0 + (T(1) - f0) * pow5(T(1) - ct);
                V3<T> refr = vrefract(dr, n, eta);
                V3<T> refl = vreflect(dr, n);
                if (dot(refr, refr) < T(0.000001f) || !std::isfinite(refr.x) || r2 < fres) {
                    dr = normalize(refl);
                } else {
                    dr = normalize(refr);
                    side = side * T(-1);
                    color = color * (vmix(V3<T>(T(1)), mat.rgb, T(0.35f)) * (T(1) - fres * T(0.5f)));
                }
            }
            rp = rp + n * (T(0.001f) * signv(dot(dr, n)));
        }
        if (c.sdf_russian_roulette != 0u && i + 1 < bounces && T(i + 1) >= T(c.sdf_rr_start)) {
            T surv = clampv(maxc(color), clampv(T(c.sdf_rr_min_prob), T(0.01f), T(1)), T(1));
            T rr = T(rng.uniform(SLOT_RR, i));
            if (rr > surv) break;
            color = color / surv;
        }
    }
    V3<T> col = ggx ? light : light * color;
    if (c.world[6] == 1.0f) col = vmix(col, grad, sky_mask);
    return vmin(col, V3<T>(T(8)));
}

// ------------------------------------------------------------------ present
template <class T> V3<T> gammaSrgb(V3<T> lin) {                                  // :6778-6782
    V3<T> out;
    for (int k = 0; k < 3; ++k) {
        T l = lin[k];
        out[k] = l <= T(0.0031308f) ? l * T(12.92f) : T(1.055f) * std::pow(std::max(l, T(0)), T(1) / T(2.4f)) - T(0.055f);
    }
    return out;
}
template <class T> V3<T> aces(V3<T> x) {                                         // :6784-6791
    V3<T> o;
    for (int k = 0; k < 3; ++k) o[k] = clampv((x[k] * (T(2.51f) * x[k] + T(0.03f))) / (x[k] * (T(2.43f) * x[k] + T(0.59f)) + T(0.14f)), T(0), T(1));
    return o;
}
template <class T> V3<T> pbrNeutral(V3<T> c) {                                   // :6793-6806
    T x = std::min(c.x, std::min(c.y, c.z));
    T off = x < T(0.08f) ? x - T(6.25f) * x * x : T(0.04f);
    c = c - off;
    T peak = maxc(c);
    if (peak < T(0.76f)) return c;
    T d = T(1) - T(0.76f);
    T np = T(1) - d * d / (peak + d - T(0.76f));
    c = c * (np / peak);
    T g = T(1) - T(1) / (T(0.15f) * (peak - np) + T(1));
    return vmix(c, V3<T>(np), g);
}
template <class T> V3<T> toneMap(V3<T> c, const Cfg &cfg) {                      // :6808-6816
    float n = cfg.post[0];
    if (n == 0.0f) return gammaSrgb(c);
    if (n == 1.0f) return V3<T>(std::pow(c.x, T(1) / T(2.4f)), std::pow(c.y, T(1) / T(2.4f)), std::pow(c.z, T(1) / T(2.4f)));
    if (n == 2.0f) return V3<T>(std::pow(c.x, T(1) / T(2.6f)), std::pow(c.y, T(1) / T(2.6f)), std::pow(c.z, T(1) / T(2.6f)));
    if (n == 3.0f) return aces(c);
    if (n == 4.0f) return pbrNeutral(c);
    return c;
}
template <class T> V3<T> postProcess(V3<T> c, const Cfg &cfg) {                  // :6818-6825
    c = toneMap(c, cfg);
    c = c * T(cfg.post[1]) + T(cfg.post[2]);
    c = (c - V3<T>(T(0.5f))) * T(cfg.post[4]) + V3<T>(T(0.5f));
    T l = dot(c, V3<T>(T(0.2126f), T(0.7152f), T(0.0722f)));
    c = vmix(V3<T>(l), c, T(cfg.post[3]));
    return vclamp(c, T(0), T(1));
}

}  // namespace oracle

// ====================================================================== C API
using namespace oracle;

namespace {
const FptCudaSceneExt kNoExt{};
inline const FptCudaSceneExt &ext_or_default(const FptCudaSceneExt *e) { return e ? *e : kNoExt; }

template <class T> void sample_distance_impl(const Cfg &c, const Ext &e, const float *pts, size_t n, double *out, double *grad) {
#pragma omp parallel for schedule(dynamic, 256)
    for (long long i = 0; i < (long long)n; ++i) {
        V3<T> p(T(pts[i * 4 + 0]), T(pts[i * 4 + 1]), T(pts[i * 4 + 2]));
        out[i * 4 + 0] = double(distanceSdf(p, c, e));
        out[i * 4 + 1] = e.formula ? double(extDistance(p, c, e, nullptr).orbit) : 0.0;
        if (c.sdf_id == FPT_SDF_MANDELBULBER) {
            Field4<T> f = fieldSample(p, c, e, 1);
            out[i * 4 + 2] = double(f.dr);
            out[i * 4 + 3] = double(std::fabs(f.state));
        } else {
            out[i * 4 + 2] = 0.0;
            out[i * 4 + 3] = 0.0;
        }
        if (grad) {
            V3<double> g(0, 0, 0);
            if (e.formula) g = extGradient(V3<double>(pts[i * 4 + 0], pts[i * 4 + 1], pts[i * 4 + 2]), c, e);
            else if (c.sdf_id == FPT_SDF_PROGRAM) {
                V3<T> gg = programSurface(p, c).gradient;
                g = V3<double>(double(gg.x), double(gg.y), double(gg.z));
            }
            grad[i * 3 + 0] = g.x; grad[i * 3 + 1] = g.y; grad[i * 3 + 2] = g.z;
        }
    }
}

template <class T> void trace_primary_impl(const Cfg &c, const Ext &e, uint32_t y0, uint32_t y1, double *out) {
    // out: per pixel {distance, nx, ny, nz, steps, hit}
    const long long W = c.width;
    const long long total = (long long)(y1 - y0) * W;
#pragma omp parallel for schedule(dynamic, 64)
    for (long long k = 0; k < total; ++k) {
        uint32_t gy = y0 + uint32_t(k / W), gx = uint32_t(k % W);
        V2<float> uv = screenUv(gx, gy, c);
        PathRng rng{false, 0, 0, 0, uv.x, uv.y, 0.0f};
        V3<T> rp, dr;
        double *o = out + (size_t(gy) * W + gx) * 6;
        if (!cameraRay(uv, rng, false, T(0), c, rp, dr)) {
            o[0] = 0; o[1] = o[2] = o[3] = 0; o[4] = 0; o[5] = 0;
            continue;
        }
        V3<T> cam = rp;
        MarchOut<T> m = march(dr, rp, int(c.render[1]), T(c.render[3]), T(0.0002f), c, e);
        T travel = length(m.pos - cam);
        bool hit = m.found && std::isfinite(travel) && travel < T(c.render[4]) * T(0.99f);
        V3<T> n(T(0));
        if (hit) n = normalAt(m.pos, c, e);
        o[0] = double(travel); o[1] = double(n.x); o[2] = double(n.y); o[3] = double(n.z);
        o[4] = double(m.steps); o[5] = hit ? 1.0 : 0.0;
    }
}

template <class T> void render_impl(const Cfg &c, const Ext &e, uint32_t y0, uint32_t y1, uint32_t y_stride, uint32_t x_stride,
                                    float *accum, double *stats) {
    T focus = c.focus_distance > 0.0f ? T(c.focus_distance) : estimateFocus<T>(c, e);
    uint32_t samples = std::min(std::max(c.samples, 1u), 512u);
    const long long W = c.width;
    const long long cols = (W + x_stride - 1) / x_stride;
    const long long rows = (long long)(y1 - y0 + y_stride - 1) / y_stride;
    const long long total = rows * cols;
    long long steps = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : steps)
    for (long long k = 0; k < total; ++k) {
        uint32_t gy = y0 + uint32_t(k / cols) * y_stride, gx = uint32_t((k % cols) * x_stride);
        V2<float> uv = screenUv(gx, gy, c);
        uint32_t pixel = gy * c.width + gx;
        V3<T> col(T(0));
        for (uint32_t s = 0; s < samples; ++s) {
            PathStats<T> st;
            V3<T> sc = renderPath(uv, pixel, s, focus, c, e, &st);
            steps += st.primary_steps + st.shadow_steps;
            col = vmix(col, sc, T(1) / T(s + 1u));
        }
        float *a = accum + size_t(pixel) * 4;
        a[0] = float(col.x); a[1] = float(col.y); a[2] = float(col.z); a[3] = 1.0f;
    }
    if (stats) stats[0] = double(steps);
}
}  // namespace

extern "C" {

int oracle_config_size(void) { return int(sizeof(FptRenderConfig)); }
int oracle_ext_size(void) { return int(sizeof(FptCudaSceneExt)); }

void oracle_set_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}
int oracle_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// out: n x {distance, orbit, derivative, iterations}; grad (optional): n x 3.
void oracle_sample_distance(const FptRenderConfig *c, const FptCudaSceneExt *e, const float *pts, size_t n, int fp64,
                            double *out, double *grad) {
    if (fp64) sample_distance_impl<double>(*c, ext_or_default(e), pts, n, out, grad);
    else sample_distance_impl<float>(*c, ext_or_default(e), pts, n, out, grad);
}

// fpt_mandelbulber_sample_field semantics (shaders/Shaders.metal:1001-1009).
void oracle_field_sample(const FptRenderConfig *c, const FptCudaSceneExt *e, const float *pts, size_t n, int fp64,
                         double *out) {
    const Ext &ex = ext_or_default(e);
    for (size_t i = 0; i < n; ++i) {
        if (fp64) {
            Field4<double> f = fieldSample(V3<double>(pts[i * 4], pts[i * 4 + 1], pts[i * 4 + 2]), *c, ex, 1);
            out[i * 4] = f.d; out[i * 4 + 1] = f.r; out[i * 4 + 2] = f.dr; out[i * 4 + 3] = std::fabs(f.state);
        } else {
            Field4<float> f = fieldSample(V3<float>(pts[i * 4], pts[i * 4 + 1], pts[i * 4 + 2]), *c, ex, 1);
            out[i * 4] = f.d; out[i * 4 + 1] = f.r; out[i * 4 + 2] = f.dr; out[i * 4 + 3] = std::fabs(f.state);
        }
    }
}

// Orbit formula alone (no world transform): the known-answer hook for
// src/mandelbulber/orbit.rs:1866-1960.  out = {x, y, z, w, dr, r, iterations, escaped, distance, colour}.
void oracle_orbit_step(const FptCudaSceneExt *e, const double *p4, int iterations, double bailout, int add_c, double *out) {
    Ext ex = *e;
    double z[4] = {p4[0], p4[1], p4[2], p4[3]};
    double c0[4] = {p4[0], p4[1], p4[2], p4[3]};
    double dr = 1.0, color = 1.0;
    double r = len4(z);
    int it = 0;
    bool esc = false;
    for (int i = 0; i < iterations; ++i) {
        switch (ex.formula) {
            case FPT_CUDA_FORMULA_MANDELBULB: stepMandelbulb(z, dr, r, double(ex.power)); break;
            case FPT_CUDA_FORMULA_MANDELBULB_POWER2: stepMandelbulbPower2(z, dr, r); break;
            case FPT_CUDA_FORMULA_MANDELBOX: stepMandelbox(z, dr, color, ex); break;
            case FPT_CUDA_FORMULA_MENGER_FOLD: stepMenger(z, dr, double(ex.menger_scale)); break;
            default: break;
        }
        if (add_c) for (int k = 0; k < 4; ++k) z[k] += c0[k];
        r = len4(z);
        it = i + 1;
        if (r > bailout) { esc = true; break; }
    }
    out[0] = z[0]; out[1] = z[1]; out[2] = z[2]; out[3] = z[3];
    out[4] = dr; out[5] = r; out[6] = it; out[7] = esc ? 1 : 0;
    OrbitOut<double> o = orbitEval(ex, iterations, bailout, V3<double>(p4[0], p4[1], p4[2]));
    out[8] = o.d;
    out[9] = color;
}

// Per-pixel primary march; out has width*height*6 doubles
// {distance, nx, ny, nz, steps, hit}; rows [y0, y1) are filled.
void oracle_trace_primary(const FptRenderConfig *c, const FptCudaSceneExt *e, int fp64, uint32_t y0, uint32_t y1, double *out) {
    if (fp64) trace_primary_impl<double>(*c, ext_or_default(e), y0, y1, out);
    else trace_primary_impl<float>(*c, ext_or_default(e), y0, y1, out);
}

double oracle_focus_distance(const FptRenderConfig *c, const FptCudaSceneExt *e, int fp64) {
    if (fp64) return estimateFocus<double>(*c, ext_or_default(e));
    return double(estimateFocus<float>(*c, ext_or_default(e)));
}

// Batch accumulation (accumulate_all_kernel, shaders/Shaders.metal:7721-7737)
// of rows [y0, y1), every x_stride-th column; accum is width*height*4 floats.
void oracle_render(const FptRenderConfig *c, const FptCudaSceneExt *e, int fp64, uint32_t y0, uint32_t y1, uint32_t x_stride,
                   float *accum, double *stats) {
    if (x_stride == 0) x_stride = 1;
    if (fp64) render_impl<double>(*c, ext_or_default(e), y0, y1, 1u, x_stride, accum, stats);
    else render_impl<float>(*c, ext_or_default(e), y0, y1, 1u, x_stride, accum, stats);
}

// Every y_stride-th row of [y0, y1) and every x_stride-th pixel of those rows:
// a sample spread evenly over the frame.
void oracle_render_grid(const FptRenderConfig *c, const FptCudaSceneExt *e, int fp64, uint32_t y0, uint32_t y1, uint32_t y_stride,
                        uint32_t x_stride, float *accum, double *stats) {
    if (x_stride == 0) x_stride = 1;
    if (y_stride == 0) y_stride = 1;
    if (fp64) render_impl<double>(*c, ext_or_default(e), y0, y1, y_stride, x_stride, accum, stats);
    else render_impl<float>(*c, ext_or_default(e), y0, y1, y_stride, x_stride, accum, stats);
}

// One path sample (debug hook): rgb out.
void oracle_render_path(const FptRenderConfig *c, const FptCudaSceneExt *e, uint32_t gx, uint32_t gy, uint32_t sample,
                        float focus, float *rgb) {
    V2<float> uv = screenUv(gx, gy, *c);
    V3<float> col = renderPath<float>(uv, gy * c->width + gx, sample, focus, *c, ext_or_default(e), nullptr);
    rgb[0] = col.x; rgb[1] = col.y; rgb[2] = col.z;
}

// present_kernel: shaders/Shaders.metal:8012-8025 with highlightAt
// (7466-7481), sampleAccumBilinear (7483-7496), chromaticAt (7498-7507) and
// the vertical flip of outputIndex (7462-7464).
void oracle_present(const FptRenderConfig *c, const float *accum, uint8_t *rgba) {
    const uint32_t W = c->width, H = c->height;
    auto A = [&](uint32_t x, uint32_t y) {
        const float *a = accum + (size_t(y) * W + x) * 4;
        return V3<float>(a[0], a[1], a[2]);
    };
    auto bil = [&](float u, float v) {
        float px = clampv(u, 0.0f, 1.0f) * float(W) - 0.5f, py = clampv(v, 0.0f, 1.0f) * float(H) - 0.5f;
        int bx = int(std::floor(px)), by = int(std::floor(py));
        float fx = fractv(px), fy = fractv(py);
        uint32_t x0 = uint32_t(clampv(bx, 0, int(W - 1))), y0 = uint32_t(clampv(by, 0, int(H - 1)));
        uint32_t x1 = std::min(x0 + 1u, W - 1u), y1 = std::min(y0 + 1u, H - 1u);
        return vmix(vmix(A(x0, y0), A(x1, y0), fx), vmix(A(x0, y1), A(x1, y1), fx), fy);
    };
    for (uint32_t y = 0; y < H; ++y)
        for (uint32_t x = 0; x < W; ++x) {
            float u = (float(x) + 0.5f) / float(W), v = (float(y) + 0.5f) / float(H);
            float dx = u - 0.5f, dy = v - 0.5f;
            float len = std::sqrt(dx * dx + dy * dy);
            float ox = dx * c->post[5] * len / 8.0f, oy = dy * c->post[5] * len / 8.0f;
            V3<float> center = bil(u, v), col = center;
            if (std::fabs(c->post[5]) > 0.00001f) {
                V3<float> g = bil(u - ox, v - oy), b = bil(u - 2.0f * ox, v - 2.0f * oy);
                col = V3<float>(center.x, g.y, b.z);
            }
            V3<float> hl(0.0f);
            float inten = c->post[6];
            if (inten > 0.00001f) {
                uint32_t x0 = x > 0 ? x - 1 : x, x1 = std::min(x + 1, W - 1), y0 = y > 0 ? y - 1 : y, y1 = std::min(y + 1, H - 1);
                V3<float> br = vmax(A(x, y) - V3<float>(0.5f), V3<float>(0.0f));
                br = br + A(x1, y) * 0.25f + A(x0, y) * 0.25f + A(x, y1) * 0.25f + A(x, y0) * 0.25f;
                hl = br * inten;
            }
            V3<float> o = postProcess(col + hl, *c);
            uint8_t *p = rgba + (size_t(H - 1 - y) * W + x) * 4;
            p[0] = uint8_t(clampv(o.x, 0.0f, 1.0f) * 255.0f);
            p[1] = uint8_t(clampv(o.y, 0.0f, 1.0f) * 255.0f);
            p[2] = uint8_t(clampv(o.z, 0.0f, 1.0f) * 255.0f);
            p[3] = 255;
        }
}

// Image metrics of src/metal_bridge.mm:2383-2495 and 6078-6104:
// out = {mae, rmse, max_abs, changed_pct, luminance_ssim, low_frequency_ssim}.
void oracle_image_metrics(const uint8_t *a, const uint8_t *b, uint32_t W, uint32_t H, double *out) {
    auto luma = [](const uint8_t *img, size_t p) {
        const uint8_t *q = img + p * 4;
        return 0.2126 * double(q[0]) + 0.7152 * double(q[1]) + 0.0722 * double(q[2]);
    };
    double abs_sum = 0, sq = 0; uint32_t maxd = 0; uint64_t changed = 0;
    size_t px = size_t(W) * H;
    for (size_t p = 0; p < px; ++p) {
        bool ch = false;
        for (int k = 0; k < 3; ++k) {
            uint32_t d = uint32_t(std::abs(int(a[p * 4 + k]) - int(b[p * 4 + k])));
            abs_sum += d; sq += double(d) * d; maxd = std::max(maxd, d); if (d) ch = true;
        }
        if (ch) ++changed;
    }
    double n = double(px * 3);
    out[0] = abs_sum / n; out[1] = std::sqrt(sq / n); out[2] = maxd; out[3] = px ? 100.0 * double(changed) / double(px) : 0;
    const double c1 = 6.5025, c2 = 58.5225;
    double ws = 0, wt = 0;
    for (uint32_t by = 0; by < H; by += 8)
        for (uint32_t bx = 0; bx < W; bx += 8) {
            uint32_t ye = std::min(H, by + 8), xe = std::min(W, bx + 8);
            double cnt = double((ye - by) * (xe - bx)), ma = 0, mb = 0;
            for (uint32_t y = by; y < ye; ++y) for (uint32_t x = bx; x < xe; ++x) { size_t p = size_t(y) * W + x; ma += luma(a, p); mb += luma(b, p); }
            ma /= cnt; mb /= cnt;
            double va = 0, vb = 0, cv = 0;
            for (uint32_t y = by; y < ye; ++y) for (uint32_t x = bx; x < xe; ++x) {
                size_t p = size_t(y) * W + x; double da = luma(a, p) - ma, db = luma(b, p) - mb;
                va += da * da; vb += db * db; cv += da * db;
            }
            double den = std::max(1.0, cnt - 1.0); va /= den; vb /= den; cv /= den;
            double num = (2 * ma * mb + c1) * (2 * cv + c2), dd = (ma * ma + mb * mb + c1) * (va + vb + c2);
            ws += (dd > 0 ? num / dd : 1.0) * cnt; wt += cnt;
        }
    out[4] = wt > 0 ? std::clamp(ws / wt, -1.0, 1.0) : 0.0;
    std::vector<double> A(64 * 64), B(64 * 64);
    for (uint32_t y = 0; y < 64; ++y) {
        uint32_t y0 = uint32_t((uint64_t(y) * H) / 64), y1 = std::max(uint32_t((uint64_t(y + 1) * H) / 64), y0 + 1);
        for (uint32_t x = 0; x < 64; ++x) {
            uint32_t x0 = uint32_t((uint64_t(x) * W) / 64), x1 = std::max(uint32_t((uint64_t(x + 1) * W) / 64), x0 + 1);
            double sa = 0, sb = 0, cnt = 0;
            for (uint32_t sy = y0; sy < y1; ++sy) for (uint32_t sx = x0; sx < x1; ++sx) {
                size_t p = size_t(sy) * W + sx; sa += luma(a, p); sb += luma(b, p); cnt += 1;
            }
            A[y * 64 + x] = sa / cnt; B[y * 64 + x] = sb / cnt;
        }
    }
    double ma = 0, mb = 0, nn = double(A.size());
    for (size_t i = 0; i < A.size(); ++i) { ma += A[i]; mb += B[i]; }
    ma /= nn; mb /= nn;
    double va = 0, vb = 0, cv = 0;
    for (size_t i = 0; i < A.size(); ++i) { double da = A[i] - ma, db = B[i] - mb; va += da * da; vb += db * db; cv += da * db; }
    double den = std::max(1.0, nn - 1.0); va /= den; vb /= den; cv /= den;
    double num = (2 * ma * mb + c1) * (2 * cv + c2), dd = (ma * ma + mb * mb + c1) * (va + vb + c2);
    out[5] = dd > 0 ? std::clamp(num / dd, -1.0, 1.0) : 1.0;
}

}  // extern "C"

// ====================================================================== voxels
// CPU restatement of the voxel classifier (shaders/Shaders.metal:4196-4244,
// legacy coverage), buildVoxelCell (5388-5414), the raster-order host
// compaction (src/metal_bridge.mm:1738-1812) and the DDA traversal
// (4091-4190, traceVoxel 4492-4612).  Compiled without contraction, so the
// same float operations give the same bits as the GPU build.
namespace oracle {

struct VGrid {
    float bmin[3], bmax[3], cs[3];
    uint32_t res, bs, bg;      // resolution, brick size, bricks per axis
    uint32_t storage;          // 0 dense reference cells, 1 reference bricks, 4 occupancy bricks
    const uint32_t *table;
    const uint8_t *occ;
    const uint32_t *cells;
};

inline bool classify(const Cfg &c, const Ext &e, const float bmin[3], const float cs[3], float radius, uint32_t x, uint32_t y,
                     uint32_t z, float &d, V3<float> &p) {
    p = V3<float>(bmin[0] + (float(x) + 0.5f) * cs[0], bmin[1] + (float(y) + 0.5f) * cs[1], bmin[2] + (float(z) + 0.5f) * cs[2]);
    d = distanceSdf(p, c, e);
    bool occ = std::isfinite(d) && std::fabs(d) <= radius * std::max(c.voxel_surface_band, 0.25f);
    if (c.voxel_fill_interior != 0u && std::isfinite(d) && d < 0.0f) occ = true;
    return occ;
}

// IEEE binary16 round-to-nearest-even (the conversion __float2half_rn performs).
inline uint16_t float_to_half_rne(float f) {
    uint32_t x = float_bits(f);
    uint32_t sign = (x >> 16) & 0x8000u;
    uint32_t ax = x & 0x7fffffffu;
    if (ax >= 0x7f800000u) return uint16_t(sign | 0x7c00u | (ax > 0x7f800000u ? 0x200u : 0u));
    if (ax >= 0x477ff000u) return uint16_t(sign | 0x7c00u);   // rounds to infinity
    if (ax < 0x38800000u) {                                    // subnormal half or zero
        if (ax < 0x33000000u) return uint16_t(sign);           // below half of the smallest subnormal
        uint32_t e = ax >> 23;
        uint32_t m = (ax & 0x7fffffu) | 0x800000u;
        uint32_t shift = 126u - e;
        uint32_t q = m >> shift, rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1u);
        if (rem > half || (rem == half && (q & 1u))) ++q;
        return uint16_t(sign | q);
    }
    uint32_t e = (ax >> 23) - 112u;
    uint32_t m = ax & 0x7fffffu;
    uint32_t q = (e << 10) | (m >> 13);
    uint32_t rem = m & 0x1fffu;
    if (rem > 0x1000u || (rem == 0x1000u && (q & 1u))) ++q;
    return uint16_t(sign | q);
}

inline uint32_t pack_unorm4(float a, float b, float c, float d) {
    auto q = [](float v) { return uint32_t(std::nearbyint(std::min(std::max(v, 0.0f), 1.0f) * 255.0f)); };
    return q(a) | (q(b) << 8) | (q(c) << 16) | (q(d) << 24);
}

inline bool ray_aabb(V3<float> o, V3<float> d, const float *bmin, const float *bmax, float &near_t, float &far_t, V3<float> &en) {
    near_t = -kInf;
    far_t = kInf;
    en = V3<float>(0.f);
    for (int a = 0; a < 3; ++a) {
        if (d[a] == 0.0f) {
            if (o[a] < bmin[a] || o[a] > bmax[a]) return false;
            continue;
        }
        float t0 = (bmin[a] - o[a]) / d[a], t1 = (bmax[a] - o[a]) / d[a];
        float an = std::min(t0, t1), af = std::max(t0, t1);
        if (an > near_t) {
            near_t = an;
            en = V3<float>(0.f);
            en[a] = d[a] > 0.0f ? -1.0f : 1.0f;
        }
        far_t = std::min(far_t, af);
        if (near_t > far_t) return false;
    }
    float entry = std::max(near_t, 0.0f);
    return std::isfinite(entry) && std::isfinite(far_t) && far_t >= entry;
}
inline bool cell_coordinate(V3<float> p, V3<float> d, const VGrid &g, int c[3]) {
    for (int a = 0; a < 3; ++a) if (p[a] < g.bmin[a] || p[a] > g.bmax[a]) return false;
    for (int a = 0; a < 3; ++a) if ((d[a] < 0.0f && p[a] <= g.bmin[a]) || (d[a] > 0.0f && p[a] >= g.bmax[a])) return false;
    for (int a = 0; a < 3; ++a) {
        float gp = (p[a] - g.bmin[a]) / g.cs[a];
        float fl = std::floor(gp);
        int ci = int(fl) - ((d[a] < 0.0f && gp == fl) ? 1 : 0);
        ci = std::min(ci, int(g.res) - 1);
        if (ci < 0 || ci >= int(g.res)) return false;
        c[a] = ci;
    }
    return true;
}
inline float next_positive_float(float v) {
    if (!std::isfinite(v) || v < 0.0f) return kInf;
    if (v == 0.0f) return bits_float(1u);
    return bits_float(float_bits(v) + 1u);
}
inline bool advance(int c[3], const int st[3], float nt[3], const float dt[3], float &et, V3<float> &en) {
    float bt = std::min(nt[0], std::min(nt[1], nt[2]));
    if (!std::isfinite(bt)) return false;
    bool cr[3] = {nt[0] == bt, nt[1] == bt, nt[2] == bt};
    float ne = bt;
    if (!(ne > et)) {
        ne = next_positive_float(et);
        if (!std::isfinite(ne) || !(ne > et)) return false;
    }
    et = ne;
    en = V3<float>(0.f);
    int na = cr[0] ? 0 : (cr[1] ? 1 : 2);
    en[na] = st[na] > 0 ? -1.0f : 1.0f;
    for (int a = 0; a < 3; ++a) if (cr[a]) { c[a] += st[a]; nt[a] = nt[a] + dt[a]; }
    return true;
}
inline bool occupied(const VGrid &g, const int c[3], uint32_t &payload) {
    uint32_t x = uint32_t(c[0]), y = uint32_t(c[1]), z = uint32_t(c[2]);
    if (g.storage == 0u) { payload = x + y * g.res + z * g.res * g.res; return (g.cells[size_t(payload) * 3] & 0x80000000u) != 0u; }
    uint32_t b = x / g.bs + (y / g.bs) * g.bg + (z / g.bs) * g.bg * g.bg;
    uint32_t page = g.table[b];
    if (page == 0u) return false;
    payload = (page - 1u) * g.bs * g.bs * g.bs + (x % g.bs) + (y % g.bs) * g.bs + (z % g.bs) * g.bs * g.bs;
    if (g.storage == 4u) return g.occ[payload] != 0u;
    return (g.cells[size_t(payload) * 3] & 0x80000000u) != 0u;
}
struct VHit { bool hit; float t; int cell[3]; V3<float> normal; uint32_t steps; uint32_t payload; };
inline VHit trace(const VGrid &g, V3<float> o, V3<float> d, std::vector<uint32_t> *seq) {
    VHit h{false, kInf, {0, 0, 0}, V3<float>(0.f), 0u, 0u};
    float near_t, far_t;
    V3<float> en;
    if (!ray_aabb(o, d, g.bmin, g.bmax, near_t, far_t, en)) return h;
    float et = std::max(near_t, 0.0f);
    V3<float> start(std::min(std::max(o.x + d.x * et, g.bmin[0]), g.bmax[0]), std::min(std::max(o.y + d.y * et, g.bmin[1]), g.bmax[1]),
                    std::min(std::max(o.z + d.z * et, g.bmin[2]), g.bmax[2]));
    int c[3];
    if (!cell_coordinate(start, d, g, c)) return h;
    int st[3] = {0, 0, 0};
    float nt[3] = {kInf, kInf, kInf}, dt[3] = {kInf, kInf, kInf};
    for (int a = 0; a < 3; ++a) {
        float n = kInf, dd = kInf;
        if (d[a] > 0.0f) {
            st[a] = 1;
            float boundary = g.bmin[a] + float(c[a] + 1) * g.cs[a];
            n = (boundary - o[a]) / d[a];
            dd = g.cs[a] / d[a];
        } else if (d[a] < 0.0f) {
            st[a] = -1;
            float boundary = g.bmin[a] + float(c[a]) * g.cs[a];
            n = (boundary - o[a]) / d[a];
            dd = -g.cs[a] / d[a];
        }
        if (!std::isfinite(n) || !std::isfinite(dd)) { n = kInf; dd = kInf; }
        nt[a] = n; dt[a] = dd;
    }
    const uint32_t max_steps = g.res * 3u + 3u;
    for (uint32_t s = 0; s < max_steps && et <= far_t; ++s) {
        if (c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= int(g.res) || c[1] >= int(g.res) || c[2] >= int(g.res)) break;
        if (seq) seq->push_back(uint32_t(c[0]) + uint32_t(c[1]) * g.res + uint32_t(c[2]) * g.res * g.res);
        uint32_t payload = 0;
        if (occupied(g, c, payload)) {
            h.hit = true; h.t = et; h.cell[0] = c[0]; h.cell[1] = c[1]; h.cell[2] = c[2]; h.normal = en; h.steps = s + 1;
            h.payload = payload;
            return h;
        }
        if (!advance(c, st, nt, dt, et, en)) break;
    }
    return h;
}

// offsetVoxelRayOrigin and precisionOffsetRayOrigin (shaders/Shaders.metal:4057-4090).
inline V3<float> voxel_offset_origin(V3<float> pos, V3<float> n, V3<float> dir, const Cfg &c, float eps) {
    const float side = dot(dir, n) >= 0.0f ? 1.0f : -1.0f;
    const V3<float> dn = n * side;
    if (c.voxel_offset_mode != FPT_VOXEL_OFFSET_PRECISION) return pos + dn * eps;
    V3<float> r;
    for (int a = 0; a < 3; ++a) {
        const int off = int(256.0f * dn[a]);
        int32_t bits = int32_t(float_bits(pos[a]));
        bits += pos[a] < 0.0f ? -off : off;
        r[a] = std::fabs(pos[a]) < 1.0f / 32.0f ? pos[a] + (1.0f / 65536.0f) * dn[a] : bits_float(uint32_t(bits));
    }
    return r;
}

// unpackVoxelMaterial (shaders/Shaders.metal:4023-4035).
inline Material<float> voxel_material(const uint32_t *cell) {
    Material<float> m;
    const uint32_t pc = cell[0], pp = cell[1];
    m.rgb = V3<float>(float(pc & 255u) / 255.0f, float((pc >> 8) & 255u) / 255.0f, float((pc >> 16) & 255u) / 255.0f);
    m.roughness = float(pp & 255u) / 255.0f;
    m.specular = float((pp >> 8) & 255u) / 255.0f;
    m.translucency = float((pp >> 16) & 255u) / 255.0f;
    m.ior = mixv(1.0f, 2.5f, float((pp >> 24) & 255u) / 255.0f);
    m.emission = bits_float(cell[2]);
    return m;
}

// renderVoxelPath (shaders/Shaders.metal:6526-6621) with face normals, stored
// materials and no leaf refinement, and voxelSunContributionWithSurface
// (6490-6515) for the sun term.
inline V3<float> render_voxel_path(const VGrid &g, V2<float> uv, uint32_t pixel, uint32_t sample, float focus, const Cfg &c,
                                   const Ext &e) {
    PathRng rng{e.rng == FPT_CUDA_RNG_PCG, e.seed, pixel, sample, uv.x, uv.y, float(sample)};
    V3<float> pos = cameraPos<float>(c);
    const float focal = 1.0f / std::tan(c.camera_fov / 2.0f * float(kPi) / 180.0f);
    const float aa = 0.3f / std::max(float(c.width), float(c.height));
    const float h1 = rng.uniform(SLOT_LENS0, 0), h2 = rng.uniform(SLOT_LENS1, 0);
    const V2<float> j = randomPoint(aa, h1, h2);
    V3<float> dir = normalize(V3<float>(uv.x + j.x, uv.y + j.y, focal));
    dir = rotateCamera(dir, c.camera_yaw_pitch[0], c.camera_yaw_pitch[1], c.camera_roll);
    const V3<float> fp = pos + dir * focus;
    const V2<float> lens = randomPoint(c.camera_dof, h1, h2);
    pos = pos + rotateCamera(V3<float>(lens.x, lens.y, 0.0f), c.camera_yaw_pitch[0], c.camera_yaw_pitch[1], c.camera_roll);
    dir = normalize(fp - pos);
    V3<float> light(0.0f), color(1.0f);
    float sky_mask = 0.0f;
    const V3<float> grad = backgroundGradient(dir, c);
    int bounces = std::min(int(c.render[0]), 8);
    if (c.sdf_bounce_cap > 0u) bounces = std::min(bounces, int(c.sdf_bounce_cap));
    const float cell = std::min(g.cs[0], std::min(g.cs[1], g.cs[2]));
    const float eps = cell * 0.01f;
    for (int b = 0; b < bounces; ++b) {
        const VHit hit = trace(g, pos, dir, nullptr);
        if (!hit.hit) {
            if (b == 0) sky_mask = 1.0f;
            light = light + environment(dir, c, e);
            break;
        }
        const Material<float> mt = voxel_material(g.cells + size_t(hit.payload) * 3);
        const V3<float> hp = pos + dir * hit.t;
        if (mt.emission > 0.001f) light = light + mt.rgb * mt.emission;
        V3<float> n = hit.normal;
        if (dot(n, dir) > 0.0f) n = -n;
        if (c.sun[0] == 1.0f) {
            V3<float> ld = rotateCamera(V3<float>(0.0f, 0.0f, 1.0f), c.sun[1] * float(kPi) / 180.0f, c.sun[2] * float(kPi) / 180.0f);
            const float a1 = rng.uniform(SLOT_SUN0, b), a2 = rng.uniform(SLOT_SUN1, b);
            const float sa = std::sin(a1 * 2.0f * float(kPi)), ca = std::cos(a1 * 2.0f * float(kPi));
            const float ss = std::sqrt(a2) * c.sun[4];
            ld = rotateCamera(ld, ca * ss, sa * ss);
            const VHit sh = trace(g, voxel_offset_origin(hp, n, ld, c, eps), ld, nullptr);
            if (!sh.hit)
                light = light + V3<float>(c.sun_color[0], c.sun_color[1], c.sun_color[2]) *
                                    (c.sun[3] * std::max(dot(n, ld), 0.0f) * mt.roughness * (1.0f - mt.translucency));
        }
        const float rs = rng.uniform(SLOT_SCATTER, b), rf = rng.uniform(SLOT_FRESNEL, b);
        bool transmitted = false;
        const float f0 = std::pow((mt.ior - 1.0f) / (mt.ior + 1.0f), 2.0f);
        const float ct = clampv(dot(n, -dir), 0.0f, 1.0f);
        const float fres = f0 + (1.0f - f0) * pow5(1.0f - ct);
        if (rs > mt.translucency) {
            const V3<float> refl = vreflect(dir, n);
            const V3<float> diffuse = randomVector(n, rng.uniform(SLOT_DIR0, b), rng.uniform(SLOT_DIR1, b));
            dir = normalize(vmix(refl, diffuse, mt.roughness));
            if (rf < fres * mt.specular) dir = refl;
            else color = color * mt.rgb;
        } else {
            const V3<float> refr = vrefract(dir, n, 1.0f / mt.ior);
            const V3<float> refl = vreflect(dir, n);
            if (dot(refr, refr) < 0.000001f || !std::isfinite(refr.x) || rf < fres) {
                dir = normalize(refl);
            } else {
                dir = normalize(refr);
                color = color * (vmix(V3<float>(1.0f), mt.rgb, 0.35f) * (1.0f - fres * 0.5f));
                transmitted = true;
            }
        }
        pos = transmitted ? hp + dir * (cell * 1.05f) : voxel_offset_origin(hp, n, dir, c, eps);
        if (c.sdf_russian_roulette != 0u && b + 1 < bounces && float(b + 1) >= c.sdf_rr_start) {
            const float surv = clampv(maxc(color), clampv(c.sdf_rr_min_prob, 0.01f, 1.0f), 1.0f);
            if (rng.uniform(SLOT_RR, b) > surv) break;
            color = color / surv;
        }
    }
    V3<float> col = light * color;
    if (c.world[6] == 1.0f) col = vmix(col, grad, sky_mask);
    return vmin(col, V3<float>(8.0f));
}

}  // namespace oracle

extern "C" {

// Builds the voxel grid on the CPU.  brick_size 8: occupancy bricks (occ,
// dist per compact cell); 4: reference cells (3 words per compact cell).
// Returns the number of active bricks, or -1 when cell_cap is too small.
long long oracle_voxel_build(const FptRenderConfig *cfg, const FptCudaSceneExt *e, uint32_t brick_size, uint32_t *table, uint8_t *occ,
                             uint16_t *dist, uint32_t *cells, size_t cell_cap, unsigned long long *active_cells) {
    const Ext &ex = ext_or_default(e);
    const FptRenderConfig &c = *cfg;
    uint32_t res = c.voxel_resolution, bs = brick_size, bg = (res + bs - 1) / bs;
    float bmin[3], cs[3];
    for (int k = 0; k < 3; ++k) { bmin[k] = c.voxel_bounds_min[k]; cs[k] = (c.voxel_bounds_max[k] - c.voxel_bounds_min[k]) / float(res); }
    float hx = cs[0] * 0.5f, hy = cs[1] * 0.5f, hz = cs[2] * 0.5f;
    float radius = std::sqrt(hx * hx + hy * hy + hz * hz);
    size_t nb = size_t(bg) * bg * bg;
    std::vector<uint32_t> count(nb, 0);
    unsigned long long cells_total = 0;
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : cells_total)
    for (long long b = 0; b < (long long)nb; ++b) {
        uint32_t bx = uint32_t(b % bg), by = uint32_t((b / bg) % bg), bz = uint32_t(b / (size_t(bg) * bg));
        uint32_t n = 0;
        for (uint32_t l = 0; l < bs * bs * bs; ++l) {
            uint32_t x = bx * bs + l % bs, y = by * bs + (l / bs) % bs, z = bz * bs + l / (bs * bs);
            if (x >= res || y >= res || z >= res) continue;
            float d; V3<float> p;
            if (classify(c, ex, bmin, cs, radius, x, y, z, d, p)) ++n;
        }
        count[size_t(b)] = n;
        cells_total += n;
    }
    uint32_t active = 0;
    for (size_t b = 0; b < nb; ++b) table[b] = count[b] ? ++active : 0u;   // raster order, x fastest
    if (active_cells) *active_cells = cells_total;
    size_t bvol = size_t(bs) * bs * bs;
    if (size_t(active) * bvol > cell_cap) return -1;
#pragma omp parallel for schedule(dynamic, 16)
    for (long long b = 0; b < (long long)nb; ++b) {
        if (!table[b]) continue;
        uint32_t bx = uint32_t(b % bg), by = uint32_t((b / bg) % bg), bz = uint32_t(b / (size_t(bg) * bg));
        size_t base = size_t(table[b] - 1) * bvol;
        for (uint32_t l = 0; l < bs * bs * bs; ++l) {
            uint32_t x = bx * bs + l % bs, y = by * bs + (l / bs) % bs, z = bz * bs + l / (bs * bs);
            bool inside = x < res && y < res && z < res;
            float d = 0.0f; V3<float> p;
            bool o = inside && classify(c, ex, bmin, cs, radius, x, y, z, d, p);
            if (occ) occ[base + l] = o ? 1u : 0u;
            if (dist) dist[base + l] = float_to_half_rne(inside ? d : 0.0f);
            if (cells) {
                uint32_t c0 = 0, c1 = 0, c2 = 0;
                if (o) {
                    Material<float> m = userMaterial(p, c, ex);
                    c0 = pack_unorm4(m.rgb.x, m.rgb.y, m.rgb.z, 0.0f) | 0x80000000u;
                    c1 = pack_unorm4(m.roughness, m.specular, m.translucency, (m.ior - 1.0f) / 1.5f);
                    c2 = float_bits(m.emission);
                }
                cells[(base + l) * 3] = c0; cells[(base + l) * 3 + 1] = c1; cells[(base + l) * 3 + 2] = c2;
            }
        }
    }
    return (long long)active;
}

// Occupancy and fp16 distance of the cells of one brick (spot checks at full size).
void oracle_voxel_brick(const FptRenderConfig *cfg, const FptCudaSceneExt *e, uint32_t brick_size, uint32_t bx, uint32_t by,
                        uint32_t bz, uint8_t *occ, uint16_t *dist) {
    const Ext &ex = ext_or_default(e);
    const FptRenderConfig &c = *cfg;
    uint32_t res = c.voxel_resolution, bs = brick_size;
    float bmin[3], cs[3];
    for (int k = 0; k < 3; ++k) { bmin[k] = c.voxel_bounds_min[k]; cs[k] = (c.voxel_bounds_max[k] - c.voxel_bounds_min[k]) / float(res); }
    float hx = cs[0] * 0.5f, hy = cs[1] * 0.5f, hz = cs[2] * 0.5f;
    float radius = std::sqrt(hx * hx + hy * hy + hz * hz);
    for (uint32_t l = 0; l < bs * bs * bs; ++l) {
        uint32_t x = bx * bs + l % bs, y = by * bs + (l / bs) % bs, z = bz * bs + l / (bs * bs);
        bool inside = x < res && y < res && z < res;
        float d = 0.0f; V3<float> p;
        bool o = inside && classify(c, ex, bmin, cs, radius, x, y, z, d, p);
        occ[l] = o ? 1u : 0u;
        dist[l] = float_to_half_rne(inside ? d : 0.0f);
    }
}

// Traces rays (6 floats each) through a grid given as arrays; records up to
// cap cells per ray.  out_hits: n x {t, cell, steps, hit} as doubles.
void oracle_dda(const FptRenderConfig *cfg, uint32_t brick_size, const uint32_t *table, const uint8_t *occ, const uint32_t *cells,
                const float *rays, size_t n, uint32_t cap, uint32_t *seq, uint32_t *seq_len, double *out_hits) {
    VGrid g;
    const FptRenderConfig &c = *cfg;
    for (int k = 0; k < 3; ++k) {
        g.bmin[k] = c.voxel_bounds_min[k]; g.bmax[k] = c.voxel_bounds_max[k];
        g.cs[k] = (c.voxel_bounds_max[k] - c.voxel_bounds_min[k]) / float(c.voxel_resolution);
    }
    g.res = c.voxel_resolution; g.bs = brick_size ? brick_size : 1; g.bg = brick_size ? (g.res + brick_size - 1) / brick_size : 0;
    g.storage = brick_size == 8 ? 4u : (brick_size == 0 ? 0u : 1u);
    g.table = table; g.occ = occ; g.cells = cells;
#pragma omp parallel for schedule(dynamic, 64)
    for (long long i = 0; i < (long long)n; ++i) {
        const float *r = rays + i * 6;
        std::vector<uint32_t> s;
        VHit h = trace(g, V3<float>(r[0], r[1], r[2]), V3<float>(r[3], r[4], r[5]), seq ? &s : nullptr);
        if (seq) {
            seq_len[i] = uint32_t(s.size());
            for (size_t k = 0; k < s.size() && k < cap; ++k) seq[size_t(i) * cap + k] = s[k];
        }
        double *o = out_hits + i * 4;
        o[0] = h.hit ? double(h.t) : -1.0;
        o[1] = h.hit ? double(uint32_t(h.cell[0]) + uint32_t(h.cell[1]) * g.res + uint32_t(h.cell[2]) * g.res * g.res) : -1.0;
        o[2] = h.steps;
        o[3] = h.hit ? 1.0 : 0.0;
    }
}

// Primary + shadow ray per pixel centre through an occupancy-brick grid
// (pixel rows [y0, y1)); out: W*H x {t, cell, lit, steps, shadow_steps}.
void oracle_voxel_primary(const FptRenderConfig *cfg, const FptCudaSceneExt *e, const uint32_t *table, const uint8_t *occ, uint32_t y0,
                          uint32_t y1, double *out) {
    const FptRenderConfig &c = *cfg;
    VGrid g;
    for (int k = 0; k < 3; ++k) {
        g.bmin[k] = c.voxel_bounds_min[k]; g.bmax[k] = c.voxel_bounds_max[k];
        g.cs[k] = (c.voxel_bounds_max[k] - c.voxel_bounds_min[k]) / float(c.voxel_resolution);
    }
    g.res = c.voxel_resolution; g.bs = 8; g.bg = (g.res + 7) / 8; g.storage = 4; g.table = table; g.occ = occ; g.cells = nullptr;
    float sun[3];
    if (e && e->sun_intensity > 0.0f) {
        float n = std::sqrt(e->sun_direction[0] * e->sun_direction[0] + e->sun_direction[1] * e->sun_direction[1] +
                            e->sun_direction[2] * e->sun_direction[2]);
        for (int k = 0; k < 3; ++k) sun[k] = e->sun_direction[k] / n;
    } else {
        float yaw = c.sun[1] * 3.14159265359f / 180.0f, pitch = c.sun[2] * 3.14159265359f / 180.0f;
        float y = std::sin(pitch), z = std::cos(pitch);
        sun[0] = z * std::sin(yaw); sun[1] = y; sun[2] = z * std::cos(yaw);
    }
    float focal = 1.0f / std::tan(c.camera_fov / 2.0f * 3.14159265359f / 180.0f);
    float sr = std::sin(c.camera_roll), cr = std::cos(c.camera_roll);
    float sp = std::sin(c.camera_yaw_pitch[1]), cp = std::cos(c.camera_yaw_pitch[1]);
    float sy = std::sin(c.camera_yaw_pitch[0]), cy = std::cos(c.camera_yaw_pitch[0]);
    float eps = std::min(g.cs[0], std::min(g.cs[1], g.cs[2])) * 0.01f;
    const uint32_t W = c.width, H = c.height;
#pragma omp parallel for schedule(dynamic, 4)
    for (long long yy = y0; yy < (long long)y1; ++yy) {
        for (uint32_t x = 0; x < W; ++x) {
            uint32_t y = uint32_t(yy);
            float u = (float(x) + 0.5f) / float(W) - 0.5f, v = (float(y) + 0.5f) / float(H) - 0.5f;
            u = u * (float(W) / float(H));
            float len = std::sqrt(u * u + v * v + focal * focal);
            float dx = u / len, dy = v / len, dz = focal / len;
            float rx = cr * dx - sr * dy, ry = sr * dx + cr * dy;
            dx = rx; dy = ry;
            float y1b = dz * sp + dy * cp, z1b = dz * cp - dy * sp;
            dy = y1b; dz = z1b;
            V3<float> d(dx * cy + dz * sy, dy, -dx * sy + dz * cy);
            V3<float> o(c.camera_position[0], c.camera_position[1], c.camera_position[2]);
            VHit h = trace(g, o, d, nullptr);
            double *r = out + (size_t(y) * W + x) * 5;
            r[0] = h.hit ? double(h.t) : -1.0;
            r[1] = h.hit ? double(uint32_t(h.cell[0]) + uint32_t(h.cell[1]) * g.res + uint32_t(h.cell[2]) * g.res * g.res) : -1.0;
            r[2] = 0.0; r[3] = h.steps; r[4] = 0.0;
            if (h.hit) {
                V3<float> pos(o.x + d.x * h.t, o.y + d.y * h.t, o.z + d.z * h.t);
                V3<float> n = h.normal;
                if (n.x * d.x + n.y * d.y + n.z * d.z > 0.0f) n = V3<float>(-n.x, -n.y, -n.z);
                float side = (sun[0] * n.x + sun[1] * n.y + sun[2] * n.z) >= 0.0f ? 1.0f : -1.0f;
                V3<float> so(pos.x + n.x * side * eps, pos.y + n.y * side * eps, pos.z + n.z * side * eps);
                VHit s = trace(g, so, V3<float>(sun[0], sun[1], sun[2]), nullptr);
                r[2] = s.hit ? 0.0 : 1.0;
                r[4] = s.steps;
            }
        }
    }
}

// renderVoxelPath accumulated over all samples of each pixel of rows [y0, y1)
// (voxel_accumulate_all_kernel, shaders/Shaders.metal:7977-7992) through a grid
// of reference cells (brick_size 4: page table + bricks; 0: dense cells).
// accum: W*H x 4 floats, row 0 at the bottom; the focus distance follows
// estimateVoxelFocusDistance (:6517-6523) when the config gives none.
void oracle_voxel_render(const FptRenderConfig *cfg, const FptCudaSceneExt *e, uint32_t brick_size, const uint32_t *table,
                         const uint32_t *cells, uint32_t y0, uint32_t y1, float *accum) {
    const FptRenderConfig &c = *cfg;
    const Ext &ex = ext_or_default(e);
    VGrid g;
    for (int k = 0; k < 3; ++k) {
        g.bmin[k] = c.voxel_bounds_min[k]; g.bmax[k] = c.voxel_bounds_max[k];
        g.cs[k] = (c.voxel_bounds_max[k] - c.voxel_bounds_min[k]) / float(c.voxel_resolution);
    }
    g.res = c.voxel_resolution; g.bs = brick_size ? brick_size : 1; g.bg = brick_size ? (g.res + brick_size - 1) / brick_size : 0;
    g.storage = brick_size == 0 ? 0u : 1u;
    g.table = table; g.occ = nullptr; g.cells = cells;
    float focus = c.focus_distance;
    if (!(focus > 0.0f)) {
        const float focal = 1.0f / std::tan(c.camera_fov / 2.0f * float(kPi) / 180.0f);
        const V3<float> d = rotateCamera(normalize(V3<float>(0.0f, 0.0f, focal)), c.camera_yaw_pitch[0], c.camera_yaw_pitch[1],
                                         c.camera_roll);
        const VHit h = trace(g, cameraPos<float>(c), d, nullptr);
        focus = h.hit && h.t > 0.001f ? h.t : 5.0f;
    }
    const uint32_t W = c.width, H = c.height, spp = std::min(std::max(c.samples, 1u), 512u);
#pragma omp parallel for schedule(dynamic, 1)
    for (long long yy = y0; yy < (long long)y1; ++yy) {
        const uint32_t y = uint32_t(yy);
        for (uint32_t x = 0; x < W; ++x) {
            float u = (float(x) + 0.5f) / float(W) - 0.5f, v = (float(y) + 0.5f) / float(H) - 0.5f;
            u = u * (float(W) / float(H));
            V3<float> mean(0.0f);
            for (uint32_t s = 0; s < spp; ++s)
                mean = vmix(mean, render_voxel_path(g, V2<float>{u, v}, y * W + x, s, focus, c, ex), 1.0f / float(s + 1u));
            float *o = accum + (size_t(y) * W + x) * 4;
            o[0] = mean.x; o[1] = mean.y; o[2] = mean.z; o[3] = 1.0f;
        }
    }
}

// HDRI hydration of the reference (src/metal_bridge.mm:2163-2300): the
// Radiance RLE reader (new-style scanlines, RGBE decode (m + 0.5) 2^(e - 136),
// -Y / +X orientation flags), then the 32 x 16 box-filtered LUT with float
// sums in raster order and the round-half-up float -> half conversion.
// Returns 0 and fills lut (32*16*3 halves), or 1 with a message.
static uint16_t reference_half(float value) {
    const uint32_t bits = float_bits(value);
    const uint32_t sign = (bits >> 16u) & 0x8000u;
    int exponent = int((bits >> 23u) & 0xffu) - 127 + 15;
    uint32_t mantissa = bits & 0x7fffffu;
    if (exponent <= 0) {
        if (exponent < -10) return uint16_t(sign);
        mantissa = (mantissa | 0x800000u) >> uint32_t(1 - exponent);
        return uint16_t(sign | ((mantissa + 0x1000u) >> 13u));
    }
    if (exponent >= 31) return uint16_t(sign | 0x7c00u);
    return uint16_t(sign | (uint32_t(exponent) << 10u) | ((mantissa + 0x1000u) >> 13u));
}

int oracle_hdri_lut(const char *path, uint16_t *lut, char *error, size_t error_len) {
    auto fail = [&](const std::string &m) { std::snprintf(error, error_len, "%s", m.c_str()); return 1; };
    std::ifstream in(path, std::ios::binary);
    if (!in) return fail(std::string("failed to open HDRI ") + path);
    std::string line;
    bool rle = false;
    while (std::getline(in, line)) {
        if (!line.empty() && line.back() == '\r') line.pop_back();
        if (line.rfind("FORMAT=32-bit_rle_rgbe", 0) == 0) rle = true;
        if (line.empty()) break;
    }
    if (!std::getline(in, line)) return fail("missing HDRI resolution");
    char ys = 0, xs = 0;
    int w = 0, h = 0;
    if (std::sscanf(line.c_str(), " %cY %d %cX %d", &ys, &h, &xs, &w) != 4 || w <= 0 || h <= 0) return fail("bad resolution line");
    if (!rle || w < 8 || w > 32767) return fail("unsupported non-RLE Radiance HDRI");
    std::vector<float> rgb(size_t(w) * h * 3, 0.0f);
    std::vector<uint8_t> scan(size_t(w) * 4);
    for (int fy = 0; fy < h; ++fy) {
        unsigned char hd[4];
        in.read(reinterpret_cast<char *>(hd), 4);
        if (!in || hd[0] != 2 || hd[1] != 2 || ((int(hd[2]) << 8) | hd[3]) != w) return fail("invalid HDRI scanline");
        for (int ch = 0; ch < 4; ++ch) {
            int x = 0;
            while (x < w) {
                unsigned char code = 0;
                in.read(reinterpret_cast<char *>(&code), 1);
                if (!in || code == 0) return fail("truncated HDRI scanline");
                if (code > 128) {
                    unsigned char v = 0;
                    in.read(reinterpret_cast<char *>(&v), 1);
                    const int n = code - 128;
                    if (!in || x + n > w) return fail("corrupt HDRI run");
                    for (int k = 0; k < n; ++k) scan[size_t(x++) * 4 + ch] = v;
                } else {
                    if (x + code > w) return fail("corrupt HDRI literal");
                    for (int k = 0; k < code; ++k) {
                        unsigned char v = 0;
                        in.read(reinterpret_cast<char *>(&v), 1);
                        scan[size_t(x++) * 4 + ch] = v;
                    }
                }
            }
        }
        const int oy = ys == '-' ? fy : h - 1 - fy;
        for (int fx = 0; fx < w; ++fx) {
            const int ox = xs == '+' ? fx : w - 1 - fx;
            const uint8_t e = scan[size_t(fx) * 4 + 3];
            const float sc = e == 0 ? 0.0f : std::ldexp(1.0f, int(e) - 136);
            for (int k = 0; k < 3; ++k) rgb[(size_t(oy) * w + ox) * 3 + k] = (float(scan[size_t(fx) * 4 + k]) + 0.5f) * sc;
        }
    }
    const uint32_t LW = FPT_HDRI_LUT_WIDTH, LH = FPT_HDRI_LUT_HEIGHT, W = uint32_t(w), H = uint32_t(h);
    for (uint32_t y = 0; y < LH; ++y) {
        const uint32_t sy0 = uint32_t(uint64_t(y) * H / LH), sy1 = std::max(sy0 + 1u, uint32_t(uint64_t(y + 1) * H / LH));
        for (uint32_t x = 0; x < LW; ++x) {
            const uint32_t sx0 = uint32_t(uint64_t(x) * W / LW), sx1 = std::max(sx0 + 1u, uint32_t(uint64_t(x + 1) * W / LW));
            float sum[3] = {0.0f, 0.0f, 0.0f};
            uint32_t n = 0;
            for (uint32_t sy = sy0; sy < std::min(sy1, H); ++sy)
                for (uint32_t sx = sx0; sx < std::min(sx1, W); ++sx, ++n)
                    for (int k = 0; k < 3; ++k) sum[k] += rgb[(size_t(sy) * W + sx) * 3 + k];
            for (int k = 0; k < 3; ++k) lut[(size_t(y) * LW + x) * 3 + k] = reference_half(sum[k] / float(std::max(n, 1u)));
        }
    }
    return 0;
}

// voxel_dda_contract_test cases (shaders/Shaders.metal:5164-5211); bit k = failed case k.
uint32_t oracle_dda_contract(void) {
    uint32_t f = 0u;
    VGrid g;
    for (int k = 0; k < 3; ++k) { g.bmin[k] = 0.0f; g.bmax[k] = 4.0f; g.cs[k] = 1.0f; }
    g.res = 4; g.bs = 4; g.bg = 1; g.storage = 1; g.table = nullptr; g.occ = nullptr; g.cells = nullptr;
    int c[3];
    auto eq = [&](int x, int y, int z) { return c[0] == x && c[1] == y && c[2] == z; };
    if (!cell_coordinate(V3<float>(1, 2, 3), V3<float>(1, 1, 1), g, c) || !eq(1, 2, 3)) f |= 1u << 0;
    if (!cell_coordinate(V3<float>(1, 2, 3), V3<float>(-1, -1, -1), g, c) || !eq(0, 1, 2)) f |= 1u << 1;
    if (!cell_coordinate(V3<float>(4, 4, 4), V3<float>(-1, -1, -1), g, c) || !eq(3, 3, 3)) f |= 1u << 2;
    if (cell_coordinate(V3<float>(4, 4, 4), V3<float>(1, 1, 1), g, c)) f |= 1u << 3;
    if (!cell_coordinate(V3<float>(4, 4, 4), V3<float>(0, 0, 0), g, c) || !eq(3, 3, 3)) f |= 1u << 4;
    c[0] = c[1] = c[2] = 0;
    int st[3] = {1, 1, 1};
    float nt[3] = {1, 1, 2}, dt[3] = {1, 1, 1}, et = 0.0f;
    V3<float> en;
    if (!advance(c, st, nt, dt, et, en) || !eq(1, 1, 0) || nt[0] != 2 || nt[1] != 2 || nt[2] != 2 || et != 1.0f || en.x != -1.0f ||
        en.y != 0.0f || en.z != 0.0f)
        f |= 1u << 5;
    if (!advance(c, st, nt, dt, et, en) || !eq(2, 2, 1) || nt[0] != 3 || nt[1] != 3 || nt[2] != 3 || et != 2.0f) f |= 1u << 6;
    c[0] = c[1] = c[2] = 0;
    nt[0] = 1; nt[1] = 2; nt[2] = 3;
    et = 1.0f;
    if (!advance(c, st, nt, dt, et, en) || float_bits(et) != float_bits(1.0f) + 1u || !eq(1, 0, 0)) f |= 1u << 7;
    float nr, fr;
    if (!ray_aabb(V3<float>(-1, 2, 2), V3<float>(1.0e-9f, 0, 0), g.bmin, g.bmax, nr, fr, en) || !(nr > 0.0f) || !(fr > nr)) f |= 1u << 8;
    if (ray_aabb(V3<float>(-1, 5, 2), V3<float>(1, 0, 0), g.bmin, g.bmax, nr, fr, en)) f |= 1u << 9;
    return f;
}

uint16_t oracle_float_to_half(float f) { return float_to_half_rne(f); }

}  // extern "C"

// ---------------------------------------------------------------- learned surrogate
// FP64 restatement of the surrogate network (no counterpart in the
// reference): features, forward pass and the gradients of the mean
// asymmetric squared loss.  With `emulate` set, values are rounded to BF16
// where the CUDA kernels store BF16 (weights, features, pre-activations,
// activations and deltas), so the remaining differences come from the
// accumulation order and the hardware tanh/sin/cos approximations.
namespace mlp_ref {

constexpr int kFreq = 16, kIn = 99, kInPad = 112, kHid = 64;
constexpr int kW0 = 0, kB0 = kW0 + kHid * kInPad, kW1 = kB0 + kHid, kB1 = kW1 + kHid * kHid, kW2 = kB1 + kHid,
              kB2 = kW2 + kHid * kHid, kW3 = kB2 + kHid, kB3 = kW3 + kHid * kHid, kW4 = kB3 + kHid, kB4 = kW4 + kHid,
              kParams = kB4 + 1;
const int kWOff[4] = {kW0, kW1, kW2, kW3}, kBOff[4] = {kB0, kB1, kB2, kB3}, kK[4] = {kInPad, kHid, kHid, kHid};

double bf16(double v, bool emulate) {
    if (!emulate) return v;
    float f = float(v);
    uint32_t u;
    std::memcpy(&u, &f, 4);
    u += 0x7fffu + ((u >> 16) & 1u);   // round to nearest even
    u &= 0xffff0000u;
    std::memcpy(&f, &u, 4);
    return double(f);
}
double sigmoid(double z) { return 1.0 / (1.0 + std::exp(-z)); }
double silu(double z) { return z * sigmoid(z); }
double silu_grad(double z) {
    double s = sigmoid(z);
    return s + z * s * (1.0 - s);
}

struct Net {
    std::vector<double> p;   // parameters (weights rounded when emulating)
    double center[3], inv_half[3], label_scale;
    bool emulate;
};

Net make_net(const float *params, const float *center, const float *inv_half, float label_scale, bool emulate) {
    Net n;
    n.p.assign(params, params + kParams);
    for (int l = 0; l < 4; ++l)
        for (int i = 0; i < kHid * kK[l]; ++i) n.p[kWOff[l] + i] = bf16(n.p[kWOff[l] + i], emulate);
    for (int j = 0; j < kHid; ++j) n.p[kW4 + j] = bf16(n.p[kW4 + j], emulate);
    for (int k = 0; k < 3; ++k) { n.center[k] = center[k]; n.inv_half[k] = inv_half[k]; }
    n.label_scale = label_scale;
    n.emulate = emulate;
    return n;
}

// u, then (sin, cos)(pi 2^(6k/15) u_i) for k < 16, i < 3; zero padding to 112.
void features(const Net &n, const float *pt, double *x) {
    double u[3];
    for (int i = 0; i < 3; ++i) u[i] = double(float((pt[i] - float(n.center[i])) * float(n.inv_half[i])));
    for (int i = 0; i < 3; ++i) x[i] = bf16(u[i], n.emulate);
    for (int k = 0; k < kFreq; ++k) {
        double f = 3.14159265358979323846 * std::exp2(6.0 * k / 15.0);
        for (int i = 0; i < 3; ++i) {
            x[3 + (k * 3 + i) * 2] = bf16(std::sin(f * u[i]), n.emulate);
            x[3 + (k * 3 + i) * 2 + 1] = bf16(std::cos(f * u[i]), n.emulate);
        }
    }
    for (int j = kIn; j < kInPad; ++j) x[j] = 0.0;
}

struct Trace {
    double x[kInPad];
    double z[4][kHid], h[4][kHid];
    double out;
};

void forward(const Net &n, const float *pt, Trace &t) {
    features(n, pt, t.x);
    const double *in = t.x;
    for (int l = 0; l < 4; ++l) {
        for (int o = 0; o < kHid; ++o) {
            double acc = 0.0;
            for (int k = 0; k < kK[l]; ++k) acc += in[k] * n.p[kWOff[l] + o * kK[l] + k];
            double z = acc + double(float(n.p[kBOff[l] + o]));
            t.z[l][o] = bf16(z, n.emulate);
            t.h[l][o] = bf16(silu(z), n.emulate);
        }
        in = t.h[l];
    }
    double out = n.p[kB4];
    for (int j = 0; j < kHid; ++j) out += t.h[3][j] * n.p[kW4 + j];
    t.out = out;
}

}  // namespace mlp_ref

extern "C" {

// Network output (distance units) at n xyzw points.
void oracle_mlp_forward(const float *params, const float *center, const float *inv_half, float label_scale, const float *pts,
                        size_t n, int emulate, double *out) {
    mlp_ref::Net net = mlp_ref::make_net(params, center, inv_half, label_scale, emulate != 0);
#pragma omp parallel for schedule(static)
    for (long i = 0; i < long(n); ++i) {
        mlp_ref::Trace t;
        mlp_ref::forward(net, pts + 4 * i, t);
        out[i] = t.out * net.label_scale;
    }
}

// Gradients of L = (1/n) sum_b w_b (out_b - y_b)^2, y_b = label_b / label_scale,
// w_b = over_weight when out_b > y_b else 1 (the CUDA training loss).
void oracle_mlp_gradients(const float *params, const float *center, const float *inv_half, float label_scale, const float *pts,
                          size_t n, float over_weight, int emulate, double *grad, double *loss) {
    using namespace mlp_ref;
    Net net = make_net(params, center, inv_half, label_scale, emulate != 0);
    std::vector<double> g(kParams, 0.0);
    double total = 0.0;
    const double inv_scale = double(1.0f / label_scale);
    for (size_t b = 0; b < n; ++b) {
        Trace t;
        forward(net, pts + 4 * b, t);
        const double y = double(float(pts[4 * b + 3] * float(inv_scale)));
        const double e = t.out - y;
        const double w = e > 0.0 ? double(over_weight) : 1.0;
        total += w * e * e;
        const double dout = 2.0 * w * e / double(n);
        g[kB4] += dout;
        double dz[kHid], dzn[kHid];
        for (int j = 0; j < kHid; ++j) {
            g[kW4 + j] += dout * t.h[3][j];
            dz[j] = bf16(dout * net.p[kW4 + j] * silu_grad(t.z[3][j]), net.emulate);
        }
        for (int l = 3; l >= 0; --l) {
            const double *in = l == 0 ? t.x : t.h[l - 1];
            for (int o = 0; o < kHid; ++o) {
                g[kBOff[l] + o] += dz[o];
                for (int k = 0; k < kK[l]; ++k) g[kWOff[l] + o * kK[l] + k] += dz[o] * in[k];
            }
            if (l == 0) break;
            for (int i = 0; i < kHid; ++i) {
                double acc = 0.0;
                for (int o = 0; o < kHid; ++o) acc += dz[o] * net.p[kWOff[l] + o * kHid + i];
                dzn[i] = bf16(acc * silu_grad(t.z[l - 1][i]), net.emulate);
            }
            std::memcpy(dz, dzn, sizeof(dz));
        }
    }
    for (int i = 0; i < kParams; ++i) grad[i] = g[i];
    if (loss) *loss = total / double(n);
}

}  // extern "C"
