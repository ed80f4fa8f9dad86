// Forward-mode dual numbers for the backward pass.
//
// Each pixel's shading depends on few parameters (its material, one light at
// a time), so the backward kernel evaluates every term with K tangents and
// contracts the result with the upstream gradient right away; the sums over
// pixels are then scattered into the parameter gradients.  Dn<K>: value and K
// partial derivatives, with the operations the shading uses.
#pragma once
#include <cuda_runtime.h>

namespace hy {

template <int K> struct Dn {
    float v;
    float d[K];
};

template <int K> __device__ __forceinline__ Dn<K> dconst(float v) {
    Dn<K> r;
    r.v = v;
#pragma unroll
    for (int i = 0; i < K; i++) r.d[i] = 0.f;
    return r;
}
template <int K> __device__ __forceinline__ Dn<K> dvar(float v, int i) {
    Dn<K> r = dconst<K>(v);
    r.d[i] = 1.f;
    return r;
}
template <int K> __device__ __forceinline__ Dn<K> operator+(const Dn<K>& a, const Dn<K>& b) {
    Dn<K> r;
    r.v = a.v + b.v;
#pragma unroll
    for (int i = 0; i < K; i++) r.d[i] = a.d[i] + b.d[i];
    return r;
}
template <int K> __device__ __forceinline__ Dn<K> operator-(const Dn<K>& a, const Dn<K>& b) {
    Dn<K> r;
    r.v = a.v - b.v;
#pragma unroll
    for (int i = 0; i < K; i++) r.d[i] = a.d[i] - b.d[i];
    return r;
}
template <int K> __device__ __forceinline__ Dn<K> operator*(const Dn<K>& a, const Dn<K>& b) {
    Dn<K> r;
    r.v = a.v * b.v;
#pragma unroll
    for (int i = 0; i < K; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
    return r;
}
template <int K> __device__ __forceinline__ Dn<K> operator/(const Dn<K>& a, const Dn<K>& b) {
    Dn<K> r;
    r.v = a.v / b.v;
    const float ib = 1.0f / b.v;
#pragma unroll
    for (int i = 0; i < K; i++) r.d[i] = (a.d[i] - r.v * b.d[i]) * ib;
    return r;
}
template <int K> __device__ __forceinline__ Dn<K> operator+(const Dn<K>& a, float s) { Dn<K> r = a; r.v += s; return r; }
template <int K> __device__ __forceinline__ Dn<K> operator+(float s, const Dn<K>& a) { return a + s; }
template <int K> __device__ __forceinline__ Dn<K> operator-(const Dn<K>& a, float s) { Dn<K> r = a; r.v -= s; return r; }
template <int K> __device__ __forceinline__ Dn<K> operator-(float s, const Dn<K>& a) {
    Dn<K> r;
    r.v = s - a.v;
#pragma unroll
    for (int i = 0; i < K; i++) r.d[i] = -a.d[i];
    return r;
}
template <int K> __device__ __forceinline__ Dn<K> operator-(const Dn<K>& a) { return 0.f - a; }
template <int K> __device__ __forceinline__ Dn<K> operator*(const Dn<K>& a, float s) {
    Dn<K> r;
    r.v = a.v * s;
#pragma unroll
    for (int i = 0; i < K; i++) r.d[i] = a.d[i] * s;
    return r;
}
template <int K> __device__ __forceinline__ Dn<K> operator*(float s, const Dn<K>& a) { return a * s; }
template <int K> __device__ __forceinline__ Dn<K> operator/(const Dn<K>& a, float s) { return a * (1.0f / s); }
template <int K> __device__ __forceinline__ Dn<K> operator/(float s, const Dn<K>& a) { return dconst<K>(s) / a; }
template <int K> __device__ __forceinline__ Dn<K> dsqrt(const Dn<K>& a) {
    Dn<K> r;
    r.v = sqrtf(a.v);
    const float h = r.v > 0.f ? 0.5f / r.v : 0.f;
#pragma unroll
    for (int i = 0; i < K; i++) r.d[i] = a.d[i] * h;
    return r;
}
// x^e for a constant exponent (x >= 0 where the shaders use it)
template <int K> __device__ __forceinline__ Dn<K> dpow(const Dn<K>& a, float e) {
    Dn<K> r;
    r.v = powf(a.v, e);
    const float g = a.v > 0.f ? e * powf(a.v, e - 1.0f) : (e == 1.0f ? 1.0f : 0.f);
#pragma unroll
    for (int i = 0; i < K; i++) r.d[i] = a.d[i] * g;
    return r;
}
// max/min/clamp take the derivative of the selected branch (0 when clamped)
template <int K> __device__ __forceinline__ Dn<K> dmax(const Dn<K>& a, float s) { return a.v >= s ? a : dconst<K>(s); }
template <int K> __device__ __forceinline__ Dn<K> dmin(const Dn<K>& a, float s) { return a.v <= s ? a : dconst<K>(s); }
template <int K> __device__ __forceinline__ Dn<K> dclamp(const Dn<K>& a, float lo, float hi) {
    return dmin(dmax(a, lo), hi);
}

template <int K> struct Dn3 { Dn<K> x, y, z; };
template <int K> __device__ __forceinline__ Dn3<K> dvec(float x, float y, float z) {
    return Dn3<K>{dconst<K>(x), dconst<K>(y), dconst<K>(z)};
}
template <int K> __device__ __forceinline__ Dn3<K> operator+(const Dn3<K>& a, const Dn3<K>& b) {
    return {a.x + b.x, a.y + b.y, a.z + b.z};
}
template <int K> __device__ __forceinline__ Dn3<K> operator-(const Dn3<K>& a, const Dn3<K>& b) {
    return {a.x - b.x, a.y - b.y, a.z - b.z};
}
template <int K> __device__ __forceinline__ Dn3<K> operator*(const Dn3<K>& a, const Dn<K>& s) { return {a.x * s, a.y * s, a.z * s}; }
template <int K> __device__ __forceinline__ Dn3<K> operator*(const Dn3<K>& a, const Dn3<K>& b) {
    return {a.x * b.x, a.y * b.y, a.z * b.z};
}
template <int K> __device__ __forceinline__ Dn3<K> operator*(const Dn3<K>& a, float s) { return {a.x * s, a.y * s, a.z * s}; }
template <int K> __device__ __forceinline__ Dn<K> ddot(const Dn3<K>& a, const Dn3<K>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <int K> __device__ __forceinline__ Dn<K> dlength(const Dn3<K>& a) { return dsqrt(ddot(a, a)); }
template <int K> __device__ __forceinline__ Dn3<K> dnormalize(const Dn3<K>& a) {
    const Dn<K> l = dlength(a);
    return {a.x / l, a.y / l, a.z / l};
}

}  // namespace hy
