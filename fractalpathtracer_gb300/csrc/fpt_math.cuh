// fpt_math.cuh -- vector helpers, dual numbers and hashes for the sm_103a kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace fpt {

constexpr float kPi = 3.14159265359f;   // the reference's pi constant (shaders/Shaders.metal:4)
constexpr float kInf = 1.0e20f;         // shaders/Shaders.metal:5

// ------------------------------------------------------------ float3 helpers
__host__ __device__ __forceinline__ float3 mk3(float a, float b, float c) { return make_float3(a, b, c); }
__host__ __device__ __forceinline__ float3 mk3(float a) { return make_float3(a, a, a); }
__host__ __device__ __forceinline__ float3 operator+(float3 a, float3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ float3 operator-(float3 a, float3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ float3 operator-(float3 a) { return mk3(-a.x, -a.y, -a.z); }
__host__ __device__ __forceinline__ float3 operator*(float3 a, float3 b) { return mk3(a.x * b.x, a.y * b.y, a.z * b.z); }
__host__ __device__ __forceinline__ float3 operator/(float3 a, float3 b) { return mk3(a.x / b.x, a.y / b.y, a.z / b.z); }
__host__ __device__ __forceinline__ float3 operator*(float3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float3 operator*(float s, float3 a) { return mk3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ float3 operator/(float3 a, float s) { return mk3(a.x / s, a.y / s, a.z / s); }
__host__ __device__ __forceinline__ float3 operator+(float3 a, float s) { return mk3(a.x + s, a.y + s, a.z + s); }
__host__ __device__ __forceinline__ float3 operator-(float3 a, float s) { return mk3(a.x - s, a.y - s, a.z - s); }
__host__ __device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__host__ __device__ __forceinline__ float len3(float3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ float3 normalize3(float3 a) { return a * rsqrtf(dot(a, a)); }
__host__ __device__ __forceinline__ float3 cross3(float3 a, float3 b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__host__ __device__ __forceinline__ float3 abs3(float3 a) { return mk3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }
__host__ __device__ __forceinline__ float3 max3(float3 a, float3 b) { return mk3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
__host__ __device__ __forceinline__ float3 min3(float3 a, float3 b) { return mk3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }
__host__ __device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
__host__ __device__ __forceinline__ float3 clamp3(float3 a, float lo, float hi) { return mk3(clampf(a.x, lo, hi), clampf(a.y, lo, hi), clampf(a.z, lo, hi)); }
__host__ __device__ __forceinline__ float mixf(float a, float b, float t) { return a + (b - a) * t; }
__host__ __device__ __forceinline__ float3 mix3(float3 a, float3 b, float t) { return a + (b - a) * t; }
__host__ __device__ __forceinline__ float maxc3(float3 a) { return fmaxf(a.x, fmaxf(a.y, a.z)); }
__host__ __device__ __forceinline__ float signf(float v) { return v > 0.0f ? 1.0f : (v < 0.0f ? -1.0f : 0.0f); }
__device__ __forceinline__ float fractf(float v) { return v - floorf(v); }
__host__ __device__ __forceinline__ float3 reflect3(float3 i, float3 n) { return i - n * (2.0f * dot(n, i)); }
__device__ __forceinline__ float3 refract3(float3 i, float3 n, float eta) {
    float d = dot(n, i);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return mk3(0.0f);
    return i * eta - n * (eta * d + sqrtf(k));
}
__device__ __forceinline__ bool finite3(float3 a) { return isfinite(a.x) && isfinite(a.y) && isfinite(a.z); }
__device__ __forceinline__ float mod1f(float x, float y) { return x - y * floorf(x / y); }
__device__ __forceinline__ float3 mod3f(float3 x, float y) { return mk3(mod1f(x.x, y), mod1f(x.y, y), mod1f(x.z, y)); }
__device__ __forceinline__ float pow5f(float x) { float x2 = x * x; return x2 * x2 * x; }

// rot2 (shaders/Shaders.metal:419-423) with precomputed sine and cosine.
__device__ __forceinline__ float2 rot2sc(float px, float py, float s, float c) { return make_float2(c * px - s * py, s * px + c * py); }
__device__ __forceinline__ float2 rot2a(float px, float py, float a) { float s, c; sincosf(a, &s, &c); return rot2sc(px, py, s, c); }

// rotateCamera (shaders/Shaders.metal:425-436).
__device__ __forceinline__ float3 rotate_camera(float3 v, float yaw, float pitch) {
    float sp, cp, sy, cy;
    sincosf(pitch, &sp, &cp);
    sincosf(yaw, &sy, &cy);
    v = mk3(v.x, v.z * sp + v.y * cp, v.z * cp - v.y * sp);
    return mk3(v.x * cy + v.z * sy, v.y, -v.x * sy + v.z * cy);
}
__device__ __forceinline__ float3 rotate_camera(float3 v, float yaw, float pitch, float roll) {
    float2 r = rot2a(v.x, v.y, roll);
    return rotate_camera(mk3(r.x, r.y, v.z), yaw, pitch);
}

// ------------------------------------------------------------ dual numbers
// Value plus the three partial derivatives d/dx, d/dy, d/dz (forward mode);
// used to differentiate the extension distance estimators for analytic normals.
struct D4 {
    float v, x, y, z;
    __device__ D4() : v(0.f), x(0.f), y(0.f), z(0.f) {}
    __device__ D4(float a) : v(a), x(0.f), y(0.f), z(0.f) {}  // NOLINT: constant lift
    __device__ D4(float a, float b, float c, float d) : v(a), x(b), y(c), z(d) {}
};
__device__ __forceinline__ D4 operator+(D4 a, D4 b) { return D4(a.v + b.v, a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ D4 operator-(D4 a, D4 b) { return D4(a.v - b.v, a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ D4 operator-(D4 a) { return D4(-a.v, -a.x, -a.y, -a.z); }
__device__ __forceinline__ D4 operator*(D4 a, D4 b) {
    return D4(a.v * b.v, a.x * b.v + a.v * b.x, a.y * b.v + a.v * b.y, a.z * b.v + a.v * b.z);
}
__device__ __forceinline__ D4 operator/(D4 a, D4 b) {
    float inv = 1.0f / b.v, q = a.v * inv;
    return D4(q, (a.x - q * b.x) * inv, (a.y - q * b.y) * inv, (a.z - q * b.z) * inv);
}
__device__ __forceinline__ D4 chain(D4 a, float f, float df) { return D4(f, df * a.x, df * a.y, df * a.z); }
__device__ __forceinline__ bool operator<(D4 a, D4 b) { return a.v < b.v; }
__device__ __forceinline__ bool operator>(D4 a, D4 b) { return a.v > b.v; }
__device__ __forceinline__ bool operator<=(D4 a, D4 b) { return a.v <= b.v; }
__device__ __forceinline__ D4 dsqrt(D4 a) { float s = sqrtf(a.v); return chain(a, s, s > 0.f ? 0.5f / s : 0.f); }
__device__ __forceinline__ D4 dlog(D4 a) { return chain(a, logf(a.v), 1.0f / a.v); }
__device__ __forceinline__ D4 dabs(D4 a) { return a.v < 0.f ? -a : a; }
__device__ __forceinline__ D4 dmax(D4 a, D4 b) { return a.v >= b.v ? a : b; }
__device__ __forceinline__ D4 dmin(D4 a, D4 b) { return a.v <= b.v ? a : b; }

// Overload set used by the templated estimators.
// double overloads serve the FP64 hit-point continuation.
__device__ __forceinline__ double s_sqrt(double a) { return sqrt(a); }
__device__ __forceinline__ double s_log(double a) { return log(a); }
__device__ __forceinline__ double s_abs(double a) { return fabs(a); }
__device__ __forceinline__ double s_max(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ double s_min(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ double s_val(double a) { return a; }
__device__ __forceinline__ double s_asin(double a) { return asin(a); }
__device__ __forceinline__ double s_atan2(double y, double x) { return atan2(y, x); }
__device__ __forceinline__ double s_pow(double a, float p) { return pow(a, double(p)); }
__device__ __forceinline__ void s_sincos(double a, double *s, double *c) { sincos(a, s, c); }
__device__ __forceinline__ float s_sqrt(float a) { return sqrtf(a); }
__device__ __forceinline__ D4 s_sqrt(D4 a) { return dsqrt(a); }
__device__ __forceinline__ float s_log(float a) { return logf(a); }
__device__ __forceinline__ D4 s_log(D4 a) { return dlog(a); }
__device__ __forceinline__ float s_abs(float a) { return fabsf(a); }
__device__ __forceinline__ D4 s_abs(D4 a) { return dabs(a); }
__device__ __forceinline__ float s_max(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ D4 s_max(D4 a, D4 b) { return dmax(a, b); }
__device__ __forceinline__ float s_min(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ D4 s_min(D4 a, D4 b) { return dmin(a, b); }
__device__ __forceinline__ float s_val(float a) { return a; }
__device__ __forceinline__ float s_val(D4 a) { return a.v; }
__device__ __forceinline__ float s_asin(float a) { return asinf(a); }
__device__ __forceinline__ D4 s_asin(D4 a) { return chain(a, asinf(a.v), rsqrtf(fmaxf(1.0f - a.v * a.v, 1e-30f))); }
__device__ __forceinline__ float s_atan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ D4 s_atan2(D4 y, D4 x) {
    float r2 = x.v * x.v + y.v * y.v;
    float gx = r2 > 0.f ? -y.v / r2 : 0.f, gy = r2 > 0.f ? x.v / r2 : 0.f;
    return D4(atan2f(y.v, x.v), gy * y.x + gx * x.x, gy * y.y + gx * x.y, gy * y.z + gx * x.z);
}
__device__ __forceinline__ float s_pow(float a, float p) { return powf(a, p); }
__device__ __forceinline__ D4 s_pow(D4 a, float p) { float f = powf(a.v, p); return chain(a, f, p * powf(a.v, p - 1.0f)); }
__device__ __forceinline__ void s_sincos(float a, float *s, float *c) { sincosf(a, s, c); }
__device__ __forceinline__ void s_sincos(D4 a, D4 *s, D4 *c) {
    float sv, cv;
    sincosf(a.v, &sv, &cv);
    *s = chain(a, sv, cv);
    *c = chain(a, cv, -sv);
}

// ------------------------------------------------------------ hashes
// hash13bits / hash13: shaders/Shaders.metal:541-555.
__host__ __device__ __forceinline__ uint32_t hash13bits(float x, float y, float z) {
#ifdef __CUDA_ARCH__
    uint32_t bx = __float_as_uint(x), by = __float_as_uint(y), bz = __float_as_uint(z);
#else
    union { float f; uint32_t u; } a{x}, b{y}, c{z};
    uint32_t bx = a.u, by = b.u, bz = c.u;
#endif
    uint32_t h = 1190494759u;
    h = (h ^ bx) * 0x5bd1e995u;
    h = (h ^ by) * 0x5bd1e995u;
    h = (h ^ bz) * 0x5bd1e995u;
    h ^= h >> 13u;
    h *= 0x5bd1e995u;
    h ^= h >> 15u;
    return h;
}
__host__ __device__ __forceinline__ float hash13(float x, float y, float z) {
    return float(hash13bits(x, y, z) & 0x00ffffffu) * (1.0f / 16777216.0f);
}
// PCG hash (Jarzynski & Olano, JCGT 2020, "Hash Functions for GPU Rendering").
__host__ __device__ __forceinline__ uint32_t pcg_hash(uint32_t v) {
    uint32_t state = v * 747796405u + 2891336453u;
    uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
    return (word >> 22u) ^ word;
}

}  // namespace fpt
