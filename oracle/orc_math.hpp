// ORACLE — test infrastructure only.  CPU restatement of the reference's GLSL
// math for the hybrid pass.  Nothing in the product links or calls this code;
// tests, __graft_entry__.smoke() and bench.py's cpu_baseline leg use it as the
// checker.  Pinned against the reference's own shader sources: oracle/glsl_ref
// compiles them as C++ (from the reference checkout, into oracle/_ref) and
// tests/golden holds their outputs; the oracle reproduces them bit for bit.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>

namespace orc {

// ---- GLSL vector subset -----------------------------------------------------
template <class T> struct V2 { T x, y; };
template <class T> struct V3 {
    T x, y, z;
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> inline V3<T> v3(T x, T y, T z) { return V3<T>{x, y, z}; }
template <class T> inline V3<T> operator+(V3<T> a, V3<T> b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> inline V3<T> operator-(V3<T> a, V3<T> b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, V3<T> b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> inline V3<T> operator/(V3<T> a, V3<T> b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
template <class T> inline V3<T> operator*(V3<T> a, T s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> inline V3<T> operator*(T s, V3<T> a) { return {s * a.x, s * a.y, s * a.z}; }
template <class T> inline V3<T> operator/(V3<T> a, T s) { return {a.x / s, a.y / s, a.z / s}; }
template <class T> inline V3<T> operator-(V3<T> a) { return {-a.x, -a.y, -a.z}; }
template <class T> inline V3<T> splat(T s) { return {s, s, s}; }
template <class T> inline T dot(V3<T> a, V3<T> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> inline V3<T> cross(V3<T> a, V3<T> b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> inline T length(V3<T> a) { return std::sqrt(dot(a, a)); }
template <class T> inline V3<T> normalize(V3<T> a) { return a / length(a); }
template <class T> inline T clampv(T v, T lo, T hi) { return std::fmin(std::fmax(v, lo), hi); }
template <class T> inline T mixv(T a, T b, T t) { return a * (T(1) - t) + b * t; }
template <class T> inline V3<T> mix3(V3<T> a, V3<T> b, T t) {
    return {mixv(a.x, b.x, t), mixv(a.y, b.y, t), mixv(a.z, b.z, t)};
}
template <class T> inline V3<T> pow3(V3<T> a, T e) {
    return {std::pow(a.x, e), std::pow(a.y, e), std::pow(a.z, e)};
}
// GLSL reflect / refract (GLSL 4.60 spec, 8.5 Geometric Functions)
template <class T> inline V3<T> reflect(V3<T> I, V3<T> N) { return I - T(2) * dot(N, I) * N; }
template <class T> inline V3<T> refract(V3<T> I, V3<T> N, T eta) {
    T d = dot(N, I);
    T k = T(1) - eta * eta * (T(1) - d * d);
    if (k < T(0)) return splat(T(0));
    return eta * I - (eta * d + std::sqrt(k)) * N;
}

// ---- constants (helpers.glsl:5-8, miss.rmiss:11) -----------------------------
template <class T> struct K {
    static constexpr T PI = T(3.14159265359);  // helpers.glsl:5
    static constexpr T PI_MISS = T(3.141592);  // miss.rmiss:11 (#define PI 3.141592)
};

// ---- RNG (random.glsl:3-33) -------------------------------------------------
// 16-round TEA (random.glsl:3-17); all arithmetic wraps mod 2^32.
inline uint32_t tea(uint32_t val0, uint32_t val1) {
    uint32_t v0 = val0, v1 = val1, s0 = 0;
    for (uint32_t n = 0; n < 16; n++) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}
// Numerical Recipes LCG (random.glsl:21-27)
inline uint32_t lcg(uint32_t& prev) {
    prev = 1664525u * prev + 1013904223u;
    return prev & 0x00FFFFFFu;
}
// rnd (random.glsl:30-33): exact in float (24-bit integer / 2^24)
inline float rnd(uint32_t& prev) { return float(lcg(prev)) / float(0x01000000); }

// ---- shading (helpers.glsl:33-93) -------------------------------------------
template <class T> inline T DistributionGGX(V3<T> N, V3<T> H, T roughness) {
    T a = roughness * roughness;
    T a2 = a * a;
    T NdotH = std::fmax(dot(N, H), T(0));
    T NdotH2 = NdotH * NdotH;
    T denom = (NdotH2 * (a2 - T(1)) + T(1));
    denom = K<T>::PI * denom * denom;
    return a2 / denom;
}
template <class T> inline T GeometrySchlickGGX(T NdotV, T roughness) {
    T r = roughness + T(1);
    T k = (r * r) / T(8);
    return NdotV / (NdotV * (T(1) - k) + k);
}
template <class T> inline T GeometrySmith(V3<T> N, V3<T> V, V3<T> L, T roughness) {
    T NdotV = std::fmax(dot(N, V), T(0));
    T NdotL = std::fmax(dot(N, L), T(0));
    return GeometrySchlickGGX(NdotV, roughness) * GeometrySchlickGGX(NdotL, roughness);
}
template <class T> inline V3<T> FresnelSchlick(T cosTheta, V3<T> F0) {
    T p = std::pow(T(1) - cosTheta, T(5));
    return F0 + (splat(T(1)) - F0) * p;
}
// sampleDisk (helpers.glsl:82-93).  `seed` is the caller's state: the
// reference passes it by value (REFERENCE mode: the caller keeps its copy);
// DECORRELATED mode passes the caller's variable so it advances.
template <class T> inline V3<T> sampleDisk(const float lpos_radius, V3<T> position, V3<T> L, uint32_t& seed) {
    T radius = T(lpos_radius) * std::sqrt(T(rnd(seed)));
    T angle = T(rnd(seed)) * T(2) * K<T>::PI;
    T px = radius * std::cos(angle), py = radius * std::sin(angle);
    V3<T> up = v3(T(0), T(1), T(0));
    V3<T> tangent = normalize(cross(L, up));
    if (L.x == T(0) && L.y == T(1) && L.z == T(0)) tangent = v3(T(0), T(0), T(1));
    V3<T> bitangent = normalize(cross(tangent, L));
    V3<T> target = position + L + px * tangent + py * bitangent;
    return normalize(target - position);
}

// GGX-sampled reflection, the HY_FLAG_GGX_REFLECTION extension (the reference
// reflects perfectly, hybridRaygen.rgen:125): a microfacet normal H with
// density D(H) (N.H) for DistributionGGX above (alpha = roughness^2), from the
// uniform draws u1 (azimuth 2 pi u1) and u2 (polar angle from the inverse of
// the lobe's cumulative distribution, tan^2 = alpha^2 u2 / (1 - u2), a form
// without the cancellation of 1 - cos^2 for narrow lobes), in a frame around N
// built from the world axis least aligned with N; the ray is
// reflect(normalize(-V), H), or the mirror direction when that would leave
// below the surface.  The kernels run the same single-rounded sequence.
template <class T> inline V3<T> ggx_reflect(V3<T> N, V3<T> V, T roughness, T u1, T u2) {
    const T a = roughness * roughness;
    const T a2 = a * a;
    const T t2 = (a2 * u2) / (T(1) - u2);
    const T cosT = T(1) / std::sqrt(T(1) + t2);
    const T sinT = std::sqrt(t2) * cosT;
    const T phi = T(2) * K<T>::PI * u1;
    const V3<T> up = std::fabs(N.y) < T(0.999f) ? v3(T(0), T(1), T(0)) : v3(T(1), T(0), T(0));
    const V3<T> Tn = normalize(cross(up, N));
    const V3<T> Bn = cross(N, Tn);
    const V3<T> Hm = Tn * (sinT * std::cos(phi)) + Bn * (sinT * std::sin(phi)) + N * cosT;
    const V3<T> I = normalize(-V);
    const V3<T> d = reflect(I, Hm);
    return dot(d, N) > T(0) ? d : reflect(I, N);
}

// ---- bit helpers shared by the BVH code --------------------------------------
inline uint32_t fbits(float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; }
inline float bitsf(uint32_t u) { float f; std::memcpy(&f, &u, 4); return f; }

}  // namespace orc
