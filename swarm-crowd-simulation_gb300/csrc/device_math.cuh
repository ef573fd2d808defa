// Device arithmetic of the crowd step. The step's numerics are the reference's (DedovSergei/swarm-crowd-simulation,
// src/cpu_crowd_sim.cpp, which ports its GLSL shaders): glm vector arithmetic evaluated per component and left to right,
// glm::mix(x, y, a) = x * (1 - a) + y * a, std::min / std::max / std::clamp with their exact tie and signed-zero
// behaviour, IEEE division and square root. Every translation unit that includes this is compiled with -fmad=false
// (no contraction into fused multiply-adds) and without fast math, so a float expression here rounds exactly as the
// same expression on the host.
#pragma once

#include <cstdint>

// SWARM_HD: device functions that also compile for the host (the seated venue's geometry is checked there against
// the reference's CPU functions by a test harness)
#define SWARM_HD __host__ __device__

namespace swarm_gpu {

template <class T> struct V2 { T x, y; };
template <class T> struct V3 { T x, y, z; };
using f2 = V2<float>;
using f3 = V3<float>;

template <class T> SWARM_HD __forceinline__ V2<T> operator+(V2<T> a, V2<T> b) { return {a.x + b.x, a.y + b.y}; }
template <class T> SWARM_HD __forceinline__ V2<T> operator-(V2<T> a, V2<T> b) { return {a.x - b.x, a.y - b.y}; }
template <class T> SWARM_HD __forceinline__ V2<T> operator-(V2<T> a) { return {-a.x, -a.y}; }
template <class T> SWARM_HD __forceinline__ V2<T> operator*(V2<T> a, T s) { return {a.x * s, a.y * s}; }
template <class T> SWARM_HD __forceinline__ V2<T> operator*(T s, V2<T> a) { return {s * a.x, s * a.y}; }
template <class T> SWARM_HD __forceinline__ V2<T> operator*(V2<T> a, V2<T> b) { return {a.x * b.x, a.y * b.y}; }
template <class T> SWARM_HD __forceinline__ V2<T> operator/(V2<T> a, T s) { return {a.x / s, a.y / s}; }
template <class T> SWARM_HD __forceinline__ V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> SWARM_HD __forceinline__ V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> SWARM_HD __forceinline__ V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> SWARM_HD __forceinline__ V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> SWARM_HD __forceinline__ V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> SWARM_HD __forceinline__ T dot(V2<T> a, V2<T> b) { return a.x * b.x + a.y * b.y; }
template <class T> SWARM_HD __forceinline__ T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
SWARM_HD __forceinline__ float length(f2 a) { return sqrtf(dot(a, a)); }
SWARM_HD __forceinline__ float length(f3 a) { return sqrtf(dot(a, a)); }
SWARM_HD __forceinline__ float mix(float a, float b, float t) { return a * (1.0f - t) + b * t; }
SWARM_HD __forceinline__ f2 mix(f2 a, f2 b, float t) { return {mix(a.x, b.x, t), mix(a.y, b.y, t)}; }
SWARM_HD __forceinline__ f2 xy(f3 a) { return {a.x, a.y}; }
SWARM_HD __forceinline__ f2 xy(float4 a) { return {a.x, a.y}; }
SWARM_HD __forceinline__ f3 xyz(float4 a) { return {a.x, a.y, a.z}; }
SWARM_HD __forceinline__ void setXY(f3& v, f2 a) { v.x = a.x; v.y = a.y; }
SWARM_HD __forceinline__ bool nonzero(f2 a) { return a.x != 0.0f || a.y != 0.0f; }

// std::max / std::min / std::clamp, exactly (the first argument wins ties; no NaN or signed-zero rewriting). clamp is
// libstdc++'s min(max(v, lo), hi) -- also glm::clamp's -- so an empty range (lo > hi) gives hi, as on the host.
template <class T> SWARM_HD __forceinline__ T smax(T a, T b) { return a < b ? b : a; }
template <class T> SWARM_HD __forceinline__ T smin(T a, T b) { return b < a ? b : a; }
template <class T> SWARM_HD __forceinline__ T sclamp(T v, T lo, T hi) { return smin(smax(v, lo), hi); }

SWARM_HD __forceinline__ f2 safeNormalize(f2 v, float eps) {
    float l = length(v);
    return l > eps ? v / l : f2{0.0f, 0.0f};
}
SWARM_HD __forceinline__ f3 safeNormalize(f3 v, float eps) {
    float l = length(v);
    return l > eps ? f3{v.x / l, v.y / l, v.z / l} : f3{0.0f, 0.0f, 0.0f};
}

// lowbias32: the stacked pair's separation direction (reference cpu_crowd_sim.cpp:120-133)
SWARM_HD __forceinline__ uint32_t hash32(uint32_t x) {
    x ^= x >> 16; x *= 0x7feb352du;
    x ^= x >> 15; x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
// cos / sin of the hashed angle, evaluated in double and rounded once: the correctly rounded float in all but
// vanishingly rare cases (only pairs stacked within 1e-6 take this path)
SWARM_HD __forceinline__ f2 pairDirection(uint32_t self, uint32_t other, float hashToRadians) {
    uint32_t lo = self < other ? self : other, hi = self < other ? other : self;
    float angle = float(hash32(hash32(lo) ^ hi)) * hashToRadians;
    f2 dir{float(cos(double(angle))), float(sin(double(angle)))};
    return self == lo ? dir : -dir;
}

}  // namespace swarm_gpu
