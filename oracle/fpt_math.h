// fpt_math.h -- scalar vector math and dual numbers for the CPU oracle.
//
// TEST INFRASTRUCTURE ONLY.  This header belongs to the oracle (a CPU
// restatement of FPT Metal's sphere-tracing path used to check the CUDA
// library); nothing in the product links it.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>

namespace oracle {

constexpr float kPi = 3.14159265359f;      // shaders/Shaders.metal:4
constexpr float kInf = 1.0e20f;            // shaders/Shaders.metal:5

// ---------------------------------------------------------------- dual numbers
// Forward-mode value with three partial derivatives (d/dpx, d/dpy, d/dpz).
struct Dual {
    double v, d[3];
    Dual() : v(0), d{0, 0, 0} {}
    Dual(double a) : v(a), d{0, 0, 0} {}  // NOLINT: implicit constant lift
    static Dual var(double a, int k) { Dual r(a); r.d[k] = 1.0; return r; }
};
inline Dual mk(double v, double a, double b, double c) { Dual r(v); r.d[0] = a; r.d[1] = b; r.d[2] = c; return r; }
inline Dual operator+(Dual a, Dual b) { return mk(a.v + b.v, a.d[0] + b.d[0], a.d[1] + b.d[1], a.d[2] + b.d[2]); }
inline Dual operator-(Dual a, Dual b) { return mk(a.v - b.v, a.d[0] - b.d[0], a.d[1] - b.d[1], a.d[2] - b.d[2]); }
inline Dual operator-(Dual a) { return mk(-a.v, -a.d[0], -a.d[1], -a.d[2]); }
inline Dual operator*(Dual a, Dual b) {
    return mk(a.v * b.v, a.d[0] * b.v + a.v * b.d[0], a.d[1] * b.v + a.v * b.d[1], a.d[2] * b.v + a.v * b.d[2]);
}
inline Dual operator/(Dual a, Dual b) {
    double q = a.v / b.v;
    return mk(q, (a.d[0] - q * b.d[0]) / b.v, (a.d[1] - q * b.d[1]) / b.v, (a.d[2] - q * b.d[2]) / b.v);
}
inline Dual &operator+=(Dual &a, Dual b) { a = a + b; return a; }
inline Dual &operator-=(Dual &a, Dual b) { a = a - b; return a; }
inline Dual &operator*=(Dual &a, Dual b) { a = a * b; return a; }
inline Dual chain(Dual a, double f, double df) { return mk(f, df * a.d[0], df * a.d[1], df * a.d[2]); }
inline bool operator<(Dual a, Dual b) { return a.v < b.v; }
inline bool operator>(Dual a, Dual b) { return a.v > b.v; }
inline bool operator<=(Dual a, Dual b) { return a.v <= b.v; }
inline bool operator>=(Dual a, Dual b) { return a.v >= b.v; }

}  // namespace oracle

namespace std {
inline oracle::Dual sqrt(oracle::Dual a) { double s = std::sqrt(a.v); return oracle::chain(a, s, s > 0 ? 0.5 / s : 0.0); }
inline oracle::Dual log(oracle::Dual a) { return oracle::chain(a, std::log(a.v), 1.0 / a.v); }
inline oracle::Dual sin(oracle::Dual a) { return oracle::chain(a, std::sin(a.v), std::cos(a.v)); }
inline oracle::Dual cos(oracle::Dual a) { return oracle::chain(a, std::cos(a.v), -std::sin(a.v)); }
inline oracle::Dual asin(oracle::Dual a) { return oracle::chain(a, std::asin(a.v), 1.0 / std::sqrt(std::max(1.0 - a.v * a.v, 1e-300))); }
inline oracle::Dual fabs(oracle::Dual a) { return a.v < 0 ? -a : a; }
inline oracle::Dual atan2(oracle::Dual y, oracle::Dual x) {
    double r2 = x.v * x.v + y.v * y.v;
    double gx = r2 > 0 ? -y.v / r2 : 0.0, gy = r2 > 0 ? x.v / r2 : 0.0;
    return oracle::mk(std::atan2(y.v, x.v), gy * y.d[0] + gx * x.d[0], gy * y.d[1] + gx * x.d[1], gy * y.d[2] + gx * x.d[2]);
}
inline oracle::Dual floor(oracle::Dual a) { return oracle::Dual(std::floor(a.v)); }
inline oracle::Dual pow(oracle::Dual a, double p) { double f = std::pow(a.v, p); return oracle::chain(a, f, p * std::pow(a.v, p - 1.0)); }
inline oracle::Dual max(oracle::Dual a, oracle::Dual b) { return a.v >= b.v ? a : b; }
inline oracle::Dual min(oracle::Dual a, oracle::Dual b) { return a.v <= b.v ? a : b; }
inline bool isfinite(oracle::Dual a) { return std::isfinite(a.v); }
}  // namespace std

namespace oracle {

// ---------------------------------------------------------------- scalars
template <class T> inline T sq(T v) { return v * v; }
inline float f_abs(float v) { return std::fabs(v); }
inline double f_abs(double v) { return std::fabs(v); }

template <class T> inline T clampv(T v, T lo, T hi) { return std::min(std::max(v, lo), hi); }
template <class T> inline T mixv(T a, T b, T t) { return a + (b - a) * t; }
template <class T> inline T signv(T v) { return v > T(0) ? T(1) : (v < T(0) ? T(-1) : T(0)); }
template <class T> inline T fractv(T v) { return v - std::floor(v); }

inline uint32_t float_bits(float v) { uint32_t b; std::memcpy(&b, &v, 4); return b; }
inline float bits_float(uint32_t b) { float v; std::memcpy(&v, &b, 4); return v; }

// ---------------------------------------------------------------- vec3
template <class T> struct V3 {
    T x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    explicit V3(T a) : x(a), y(a), z(a) {}
    T &operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> inline V3<T> operator/(V3<T> a, V3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline V3<T> operator+(V3<T> a, T s) { return {a.x + s, a.y + s, a.z + s}; }
template <class T> inline V3<T> operator-(V3<T> a, T s) { return {a.x - s, a.y - s, a.z - s}; }
template <class T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline T length(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> inline V3<T> normalize(V3<T> a) { return a / length(a); }
template <class T> inline V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> inline V3<T> vabs(V3<T> a) { return {std::fabs(a.x), std::fabs(a.y), std::fabs(a.z)}; }
template <class T> inline V3<T> vmax(V3<T> a, V3<T> b) { return {std::max(a.x, b.x), std::max(a.y, b.y), std::max(a.z, b.z)}; }
template <class T> inline V3<T> vmin(V3<T> a, V3<T> b) { return {std::min(a.x, b.x), std::min(a.y, b.y), std::min(a.z, b.z)}; }
template <class T> inline V3<T> vclamp(V3<T> a, T lo, T hi) { return {clampv(a.x, lo, hi), clampv(a.y, lo, hi), clampv(a.z, lo, hi)}; }
template <class T> inline V3<T> vfloor(V3<T> a) { return {std::floor(a.x), std::floor(a.y), std::floor(a.z)}; }
template <class T> inline V3<T> vmix(V3<T> a, V3<T> b, T t) { return a + (b - a) * t; }
template <class T> inline V3<T> vreflect(V3<T> i, V3<T> n) { return i - n * (T(2) * dot(n, i)); }
// Metal's refract(I, N, eta): zero vector on total internal reflection.
template <class T> inline V3<T> vrefract(V3<T> i, V3<T> n, T eta) {
    T d = dot(n, i);
    T k = T(1) - eta * eta * (T(1) - d * d);
    if (k < T(0)) return V3<T>(T(0));
    return i * eta - n * (eta * d + std::sqrt(k));
}
template <class T> inline T maxc(V3<T> a) { return std::max(a.x, std::max(a.y, a.z)); }
template <class T> inline bool finite3(V3<T> a) { return std::isfinite(a.x) && std::isfinite(a.y) && std::isfinite(a.z); }

template <class T> struct V2 { T x, y; };

}  // namespace oracle
