// Device-side building blocks of the hybrid pass (sm_103a).
//
//  * GLSL-semantics vector math, the reference RNG (random.glsl:3-33) and the
//    shading helpers of helpers.glsl:33-93.
//  * G-buffer texel decode for the reference's attachment formats.
//  * The compressed 8-wide BVH node (80 B, 5 x 128-bit loads), the packed
//    triangle record (48 B, 3 x 128-bit loads) and the stack traversal with
//    a watertight ray/triangle test (Woop, Benthin & Wald, JCGT 2013).
//
// Traversal and BVH arithmetic is written with explicit __f*_rn intrinsics:
// every operation is one IEEE-rounded op in a fixed order, so a CPU build of
// the same algorithm visits the same nodes and returns the same hits.
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

#include "../../include/hybridrt.h"

namespace hy {

// ------------------------------------------------------------------------------
// vector math
// ------------------------------------------------------------------------------
struct f3 { float x, y, z; };
__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ f3 operator/(f3 a, f3 b) { return {a.x / b.x, a.y / b.y, a.z / b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ f3 splat(float s) { return {s, s, s}; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float length(f3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ f3 normalize(f3 a) { return a / length(a); }
__device__ __forceinline__ float clampf(float v, float lo, float hi) { return fminf(fmaxf(v, lo), hi); }
__device__ __forceinline__ float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
__device__ __forceinline__ f3 mix3(f3 a, f3 b, float t) { return {mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)}; }
__device__ __forceinline__ f3 pow3(f3 a, float e) { return {powf(a.x, e), powf(a.y, e), powf(a.z, e)}; }
__device__ __forceinline__ f3 reflect(f3 I, f3 N) { return I - 2.0f * dot(N, I) * N; }
__device__ __forceinline__ f3 refract(f3 I, f3 N, float eta) {
    float d = dot(N, I);
    float k = 1.0f - eta * eta * (1.0f - d * d);
    if (k < 0.0f) return splat(0.0f);
    return eta * I - (eta * d + sqrtf(k)) * N;
}

// unfused variants for the ray-construction path (same op order as written)
__device__ __forceinline__ float dot_rn(f3 a, f3 b) {
    return __fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z));
}
__device__ __forceinline__ f3 add_rn(f3 a, f3 b) { return {__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z)}; }
__device__ __forceinline__ f3 sub_rn(f3 a, f3 b) { return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)}; }
__device__ __forceinline__ f3 scale_rn(f3 a, float s) { return {__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s)}; }
__device__ __forceinline__ float length_rn(f3 a) { return __fsqrt_rn(dot_rn(a, a)); }
__device__ __forceinline__ f3 normalize_rn(f3 a) {
    float l = length_rn(a);
    return {__fdiv_rn(a.x, l), __fdiv_rn(a.y, l), __fdiv_rn(a.z, l)};
}
__device__ __forceinline__ f3 cross_rn(f3 a, f3 b) {
    return {__fsub_rn(__fmul_rn(a.y, b.z), __fmul_rn(a.z, b.y)), __fsub_rn(__fmul_rn(a.z, b.x), __fmul_rn(a.x, b.z)),
            __fsub_rn(__fmul_rn(a.x, b.y), __fmul_rn(a.y, b.x))};
}

constexpr float PI = 3.14159265359f;       // helpers.glsl:5
constexpr float PI_MISS = 3.141592f;       // miss.rmiss:11

// ------------------------------------------------------------------------------
// RNG (random.glsl:3-33)
// ------------------------------------------------------------------------------
__device__ __forceinline__ uint32_t tea(uint32_t val0, uint32_t val1) {
    uint32_t v0 = val0, v1 = val1, s0 = 0;
#pragma unroll
    for (uint32_t n = 0; n < 16; n++) {
        s0 += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + s0) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + s0) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}
__device__ __forceinline__ uint32_t lcg(uint32_t& prev) {
    prev = 1664525u * prev + 1013904223u;
    return prev & 0x00FFFFFFu;
}
// n steps of the LCG at once: x -> A x + C composed with itself by squaring
// (jump-ahead), exactly the state n calls of lcg() reach
__device__ __forceinline__ uint32_t lcg_jump(uint32_t s, uint32_t n) {
    uint32_t A = 1664525u, C = 1013904223u;  // one step of random.glsl:21-27
    while (n) {
        if (n & 1u) s = A * s + C;
        C = (A + 1u) * C;                    // the map composed with itself
        A = A * A;
        n >>= 1;
    }
    return s;
}
// The maps of 2k LCG steps, x -> a x + c (mod 2^32), for k < 64: sample k of a
// pixel-light starts 2k steps (two draws per sample) after its first state,
// and one load plus one multiply-add replaces the squaring loop.
struct LcgJumpTable {
    alignas(8) uint32_t ac[128];  // (a, c) of 2k steps at ac[2k], ac[2k + 1]
    constexpr LcgJumpTable() : ac() {
        const uint32_t A2 = 1664525u * 1664525u, C2 = (1664525u + 1u) * 1013904223u;  // two steps
        uint32_t a = 1u, c = 0u;
        for (int k = 0; k < 64; k++) {
            ac[2 * k] = a;
            ac[2 * k + 1] = c;
            c = A2 * c + C2;
            a = A2 * a;
        }
    }
};
__device__ const LcgJumpTable g_lcg_jump2{};

// lcg_jump(s, 2k)
__device__ __forceinline__ uint32_t lcg_jump_even(uint32_t s, uint32_t k) {
    if (k < 64u) {
        const uint2 m = __ldg(reinterpret_cast<const uint2*>(g_lcg_jump2.ac) + k);
        return m.x * s + m.y;
    }
    return lcg_jump(s, 2u * k);
}
// float(lcg) / 16777216: the division by 2^24 is the exact product with 2^-24
__device__ __forceinline__ float rnd(uint32_t& prev) { return __fmul_rn((float)lcg(prev), 0x1p-24f); }

// ------------------------------------------------------------------------------
// shading helpers (helpers.glsl:33-93)
// ------------------------------------------------------------------------------
__device__ __forceinline__ float DistributionGGX(f3 N, f3 H, float roughness) {
    float a = roughness * roughness;
    float a2 = a * a;
    float NdotH = fmaxf(dot(N, H), 0.0f);
    float NdotH2 = NdotH * NdotH;
    float denom = (NdotH2 * (a2 - 1.0f) + 1.0f);
    denom = PI * denom * denom;
    return a2 / denom;
}
__device__ __forceinline__ float GeometrySchlickGGX(float NdotV, float roughness) {
    float r = roughness + 1.0f;
    float k = (r * r) / 8.0f;
    return NdotV / (NdotV * (1.0f - k) + k);
}
__device__ __forceinline__ float GeometrySmith(f3 N, f3 V, f3 L, float roughness) {
    float NdotV = fmaxf(dot(N, V), 0.0f);
    float NdotL = fmaxf(dot(N, L), 0.0f);
    return GeometrySchlickGGX(NdotV, roughness) * GeometrySchlickGGX(NdotL, roughness);
}
__device__ __forceinline__ f3 FresnelSchlick(float cosTheta, f3 F0) {
    float p = powf(1.0f - cosTheta, 5.0f);
    return F0 + (splat(1.0f) - F0) * p;
}
// sampleDisk (helpers.glsl:82-93); `seed` advances (the caller passes a copy
// for the reference's by-value semantics).  Split in two: the disk's frame
// (tangent, bitangent, position + L) depends only on the pixel and the light,
// so a caller drawing many samples of one pixel-light computes it once.
struct DiskFrame { f3 T, B, PL; };
__device__ __forceinline__ DiskFrame disk_frame(f3 position, f3 L) {
    DiskFrame d;
    d.T = normalize_rn(cross_rn(L, mk(0.f, 1.f, 0.f)));
    if (L.x == 0.f && L.y == 1.f && L.z == 0.f) d.T = mk(0.f, 0.f, 1.f);
    d.B = normalize_rn(cross_rn(d.T, L));
    d.PL = add_rn(position, L);
    return d;
}
__device__ __forceinline__ f3 sampleDisk(float light_radius, f3 position, const DiskFrame& d, uint32_t& seed) {
    float r1 = rnd(seed);
    float radius = __fmul_rn(light_radius, __fsqrt_rn(r1));
    float r2 = rnd(seed);
    float angle = __fmul_rn(__fmul_rn(r2, 2.0f), PI);
    float px = __fmul_rn(radius, cosf(angle)), py = __fmul_rn(radius, sinf(angle));
    f3 target = add_rn(add_rn(d.PL, scale_rn(d.T, px)), scale_rn(d.B, py));
    return normalize_rn(sub_rn(target, position));
}
__device__ __forceinline__ f3 sampleDisk(float light_radius, f3 position, f3 L, uint32_t& seed) {
    return sampleDisk(light_radius, position, disk_frame(position, L), seed);
}

// GGX-sampled reflection (HY_FLAG_GGX_REFLECTION): a microfacet normal H with
// density D(H) (N.H) for the reference's DistributionGGX (helpers.glsl:33-45,
// alpha = roughness^2), from the uniform draws u1 (azimuth) and u2 (polar:
// tan^2 = alpha^2 u2 / (1 - u2); u2 < 1 on rnd()'s grid), around N in a frame
// built from the world axis least aligned with N; the ray is reflect(normalize(-V), H),
// or the mirror direction reflect(normalize(-V), N) when that would leave
// below the surface.  Single-rounded ops in the written order (the oracle's
// ggx_reflect is the same sequence).
__device__ __forceinline__ f3 reflect_rn(f3 I, f3 N) { return sub_rn(I, scale_rn(N, __fmul_rn(2.0f, dot_rn(N, I)))); }
__device__ __forceinline__ f3 ggx_reflect(f3 N, f3 V, float roughness, float u1, float u2) {
    const float a = __fmul_rn(roughness, roughness);
    const float a2 = __fmul_rn(a, a);
    const float t2 = __fdiv_rn(__fmul_rn(a2, u2), __fsub_rn(1.0f, u2));
    const float cosT = __fdiv_rn(1.0f, __fsqrt_rn(__fadd_rn(1.0f, t2)));
    const float sinT = __fmul_rn(__fsqrt_rn(t2), cosT);
    const float phi = __fmul_rn(__fmul_rn(2.0f, PI), u1);
    const f3 up = fabsf(N.y) < 0.999f ? mk(0.f, 1.f, 0.f) : mk(1.f, 0.f, 0.f);
    const f3 T = normalize_rn(cross_rn(up, N));
    const f3 B = cross_rn(N, T);
    const f3 Hm = add_rn(add_rn(scale_rn(T, __fmul_rn(sinT, cosf(phi))), scale_rn(B, __fmul_rn(sinT, sinf(phi)))),
                         scale_rn(N, cosT));
    const f3 I = normalize_rn(mk(-V.x, -V.y, -V.z));
    const f3 d = reflect_rn(I, Hm);
    return dot_rn(d, N) > 0.f ? d : reflect_rn(I, N);
}

// ------------------------------------------------------------------------------
// texel decode
// ------------------------------------------------------------------------------
__device__ __forceinline__ float4 fetch_texel(const void* plane, uint32_t fmt, size_t i) {
    switch (fmt) {
        case HY_FMT_RGBA32F: return __ldg((const float4*)plane + i);
        case HY_FMT_RG32F: { float2 v = __ldg((const float2*)plane + i); return make_float4(v.x, v.y, 0.f, 0.f); }
        case HY_FMT_RGBA16F: {
            uint2 u = __ldg((const uint2*)plane + i);
            __half2 a = *reinterpret_cast<__half2*>(&u.x), b = *reinterpret_cast<__half2*>(&u.y);
            return make_float4(__low2float(a), __high2float(a), __low2float(b), __high2float(b));
        }
        case HY_FMT_RG16F: {
            uint32_t u = __ldg((const uint32_t*)plane + i);
            __half2 a = *reinterpret_cast<__half2*>(&u);
            return make_float4(__low2float(a), __high2float(a), 0.f, 0.f);
        }
        default: {
            uint32_t u = __ldg((const uint32_t*)plane + i);
            return make_float4(__fdiv_rn((float)(u & 0xffu), 255.f), __fdiv_rn((float)((u >> 8) & 0xffu), 255.f),
                               __fdiv_rn((float)((u >> 16) & 0xffu), 255.f), __fdiv_rn((float)(u >> 24), 255.f));
        }
    }
}

__device__ __forceinline__ uint8_t quant8(float v) {
    return (uint8_t)__float2uint_rn(__fmul_rn(fminf(fmaxf(v, 0.f), 1.f), 255.0f));
}
__device__ __forceinline__ float accum_load(uint32_t fmt, const void* buf, size_t i) {
    if (fmt == HY_ACCUM_U8) return __fdiv_rn((float)((const uint8_t*)buf)[i], 255.0f);
    return ((const float*)buf)[i];
}
__device__ __forceinline__ void accum_store(uint32_t fmt, void* buf, size_t i, float v) {
    if (fmt == HY_ACCUM_U8) ((uint8_t*)buf)[i] = quant8(v);
    else ((float*)buf)[i] = v;
}

// ------------------------------------------------------------------------------
// BVH8 node / triangle layout
// ------------------------------------------------------------------------------
// node words (uint4 q[5]):
//  q0 = p.x, p.y, p.z, e.x | e.y<<8 | e.z<<16 | imask<<24
//  q1 = child_base, tri_base, meta[0..3], meta[4..7]
//  q2 = qlo_x[0..3], qlo_x[4..7], qlo_y[0..3], qlo_y[4..7]
//  q3 = qlo_z[0..3], qlo_z[4..7], qhi_x[0..3], qhi_x[4..7]
//  q4 = qhi_y[0..3], qhi_y[4..7], qhi_z[0..3], qhi_z[4..7]
// meta[s]: 0 = empty slot, 0x80 = internal child, else (count << 5) | triangle offset
// triangle (float4 t[3]) = (v0, id bits), (v1, 0), (v2, 0)
struct Node8 { uint4 q[5]; };
constexpr int kLeafMax = 3;
constexpr int kStackMax = 64;
constexpr uint32_t kMaxIters = 1u << 22;

struct SceneDev {
    const Node8* nodes;
    const float4* tris;          // 3 per triangle
    const float4* vattr;         // 2 per vertex: (normal.xyz, color.r), (uv.xy, color.g, color.b)
    const uint32_t* idx;
    const HyPrimitive* prims;
    const uint32_t* tri_prim;    // global triangle -> primitive
    const uint32_t* prim_tri0;   // primitive -> first global triangle
    const float* nrm;            // 9 floats per transform (column-major normal matrix)
    const HyMaterial* mats;
    const HyLight* lights;
    const uchar4* env0;
    const uchar4* env1;
    uint32_t num_mats, num_lights;
    uint32_t num_nodes, num_tris;
    uint32_t env_w[2], env_h[2];
    const uchar4* tex_px;        // material textures, concatenated RGBA8 texels
    const uint4* tex_tab;        // per texture: first texel, width, height, 0
    uint32_t num_tex;
    // two-level structure: nodes / tris start with the TLAS (instance entries
    // as leaf records), each BLAS follows; 4 x float4 per instance
    const float4* inst;
    uint32_t num_inst;
    uint32_t two_level;
    // any-hit traversal ranks a node's children slot ^ near ^ anyhit_flip:
    // 7 walks them far first, 0 near first (closest-hit rays: always near first)
    uint32_t anyhit_flip;
    // per-ray limits of the walk: node visits (HY_STATUS_TIMEOUT beyond) and
    // stack entries (HY_STATUS_STACK_OVERFLOW beyond, <= kStackMax); both are
    // tested before the access they guard, so a ray that runs out stops cleanly
    uint32_t max_iters;
    int stack_cap;
};

struct Hit { float t; uint32_t id; float b1, b2; };

struct RayPre {
    f3 o;
    float d[3];
    int kx, ky, kz;
    float Sx, Sy, Sz;
    float invd[3];
    uint32_t near;
};

__device__ __forceinline__ float comp(f3 v, int k) { return k == 0 ? v.x : (k == 1 ? v.y : v.z); }

__device__ __forceinline__ RayPre ray_pre(f3 o, f3 d) {
    RayPre r;
    r.o = o;
    r.d[0] = d.x; r.d[1] = d.y; r.d[2] = d.z;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    r.kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
    r.kx = r.kz + 1; if (r.kx == 3) r.kx = 0;
    r.ky = r.kx + 1; if (r.ky == 3) r.ky = 0;
    if (comp(d, r.kz) < 0.f) { int t = r.kx; r.kx = r.ky; r.ky = t; }
    float dz = comp(d, r.kz);
    r.Sx = __fdiv_rn(comp(d, r.kx), dz);
    r.Sy = __fdiv_rn(comp(d, r.ky), dz);
    r.Sz = __frcp_rn(dz);  // the correctly rounded reciprocal: 1 / dz, bit for bit
#pragma unroll
    for (int a = 0; a < 3; a++) {
        float dd = fabsf(r.d[a]) > 1e-20f ? r.d[a] : copysignf(1e-20f, r.d[a]);
        r.invd[a] = __frcp_rn(dd);
    }
    r.near = (r.invd[0] < 0.f ? 1u : 0u) | (r.invd[1] < 0.f ? 2u : 0u) | (r.invd[2] < 0.f ? 4u : 0u);
    return r;
}

__device__ __forceinline__ float sel3(const float* a, int k) { return k == 0 ? a[0] : (k == 1 ? a[1] : a[2]); }

// Woop et al. 2013 with a double-precision fallback on zero edge functions.
__device__ __forceinline__ bool tri_test(const RayPre& r, float4 v0, float4 v1, float4 v2, float tmin, float tmax,
                                         float& t, float& b1, float& b2) {
    float A[3] = {__fsub_rn(v0.x, r.o.x), __fsub_rn(v0.y, r.o.y), __fsub_rn(v0.z, r.o.z)};
    float B[3] = {__fsub_rn(v1.x, r.o.x), __fsub_rn(v1.y, r.o.y), __fsub_rn(v1.z, r.o.z)};
    float C[3] = {__fsub_rn(v2.x, r.o.x), __fsub_rn(v2.y, r.o.y), __fsub_rn(v2.z, r.o.z)};
    float Akz = sel3(A, r.kz), Bkz = sel3(B, r.kz), Ckz = sel3(C, r.kz);
    float Ax = __fsub_rn(sel3(A, r.kx), __fmul_rn(r.Sx, Akz)), Ay = __fsub_rn(sel3(A, r.ky), __fmul_rn(r.Sy, Akz));
    float Bx = __fsub_rn(sel3(B, r.kx), __fmul_rn(r.Sx, Bkz)), By = __fsub_rn(sel3(B, r.ky), __fmul_rn(r.Sy, Bkz));
    float Cx = __fsub_rn(sel3(C, r.kx), __fmul_rn(r.Sx, Ckz)), Cy = __fsub_rn(sel3(C, r.ky), __fmul_rn(r.Sy, Ckz));
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.f || V == 0.f || W == 0.f) {
        U = __double2float_rn(__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx)));
        V = __double2float_rn(__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx)));
        W = __double2float_rn(__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax)));
    }
    if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
    float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.f) return false;
    float Az = __fmul_rn(r.Sz, Akz), Bz = __fmul_rn(r.Sz, Bkz), Cz = __fmul_rn(r.Sz, Ckz);
    float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    float tt = __fdiv_rn(T, det);
    if (!(tt >= tmin && tt <= tmax)) return false;
    t = tt;
    b1 = __fdiv_rn(V, det);
    b2 = __fdiv_rn(W, det);
    return true;
}

__device__ __forceinline__ uint32_t byte_at(uint32_t lo4, uint32_t hi4, int slot) {
    uint32_t w = slot < 4 ? lo4 : hi4;
    return (w >> ((slot & 3) * 8)) & 0xffu;
}

// three-input max / min (one instruction on sm_100+); NaN inputs are ignored as by fmaxf / fminf
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// packed pairs of f32 (sm_100+ f32x2 arithmetic: two IEEE single-rounded ops per instruction)
__device__ __forceinline__ unsigned long long f2_pack(float a, float b) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ unsigned long long f2_pack_bits(uint32_t a, uint32_t b) {
    unsigned long long r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "r"(a), "r"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(unsigned long long v, float& a, float& b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ unsigned long long f2_add(unsigned long long a, unsigned long long b) {
    unsigned long long d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ unsigned long long f2_fma(unsigned long long a, unsigned long long b,
                                                     unsigned long long c) {
    unsigned long long d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// the two halves of h as floats (exact)
__device__ __forceinline__ void h2_to_f2(uint32_t h, float& lo, float& hi) {
    asm("{ .reg .b16 l, u; mov.b32 {l, u}, %2; cvt.f32.f16 %0, l; cvt.f32.f16 %1, u; }"
        : "=f"(lo), "=f"(hi) : "r"(h));
}

// bit k set when byte k of hi4:lo4 is nonzero
__device__ __forceinline__ uint32_t nonzero_bytes(uint32_t lo4, uint32_t hi4) {
    const uint32_t a = __vcmpne4(lo4, 0u) & 0x80808080u, b = __vcmpne4(hi4, 0u) & 0x80808080u;
    return ((a * 0x00204081u) >> 28) | (((b * 0x00204081u) >> 28) << 4);
}

// bit s of an 8-bit slot mask moved to bit s ^ ord (the slots' traversal ranks)
__device__ __forceinline__ uint32_t slots_to_ranks(uint32_t m, uint32_t ord) {
    if (ord & 1u) m = ((m & 0x55u) << 1) | ((m >> 1) & 0x55u);
    if (ord & 2u) m = ((m & 0x33u) << 2) | ((m >> 2) & 0x33u);
    if (ord & 4u) m = ((m & 0x0Fu) << 4) | ((m >> 4) & 0x0Fu);
    return m;
}

// Traversal stacks: a per-lane array (local memory), or a short stack whose
// first kShortStack entries sit in shared memory (entry i of lane t at
// sh[i * 128 + t]: conflict-free) and whose deeper entries spill to the
// lane's local array.
constexpr int kShortStack = 8;
template <int SH, int STRIDE>  // SH entries in shared memory, STRIDE = threads per block
struct SplitStackT {
    uint2* sh;    // &smem[threadIdx.x], entries STRIDE apart
    uint2* deep;  // local array for the entries past SH
};
using SplitStack = SplitStackT<kShortStack, 128>;
__device__ __forceinline__ void stack_put(uint2* s, int i, uint2 v) { s[i] = v; }
__device__ __forceinline__ uint2 stack_get(const uint2* s, int i) { return s[i]; }
template <int SH, int STRIDE>
__device__ __forceinline__ void stack_put(const SplitStackT<SH, STRIDE>& s, int i, uint2 v) {
    if (i < SH) s.sh[i * STRIDE] = v;
    else s.deep[i - SH] = v;
}
template <int SH, int STRIDE>
__device__ __forceinline__ uint2 stack_get(const SplitStackT<SH, STRIDE>& s, int i) {
    return i < SH ? s.sh[i * STRIDE] : s.deep[i - SH];
}

// Stack traversal of the 8-wide BVH.  ANY: TerminateOnFirstHit semantics.
// COUNT: accumulate node visits / triangle tests.
//
// Traversal state of one ray.  A node group is (first child index, bits):
// bits[31:24] hold the not-yet-visited hit children in traversal rank order
// (rank = slot ^ ord), bits[7:0] the node's internal-child slot mask.  ord is
// the ray's near octant for closest-hit rays (front to back); for any-hit
// rays the scene chooses (SceneDev::anyhit_flip): the far octant (a shadow ray
// starts on a surface and meets its occluders away from it, so walking from
// the light's end reaches them before the boxes around the ray's own origin)
// or the near one (successive rays of a tile start at the same nodes, which
// matters when node fetches miss L2).  A group of one rank bit and an empty
// slot mask stands for the single node at g_base (the root of a walk).
struct Trav {
    uint32_t g_base, g_bits;
    int sp;
    uint32_t iters;
    float tmax;
    Hit h;
    // triangles of the last visited node's hit leaf slots, not yet tested: bit b
    // is the record at pend_base + b (trav_node leaves them, trav_tri tests them
    // one by one before the ray's next node visit)
    uint32_t pend_base, pend_bits;
    // two-level walk only (dead, and dropped by the compiler, in one-level code)
    RayPre cur;                  // the ray in the frame of the level being walked
    uint32_t inst_base, inst_bits;  // hit instance entries of the last TLAS leaf set
    uint32_t id_off;             // first global triangle of the instance being walked
    int sp_base;                 // stack height when the instance was entered
    bool level;                  // inside a BLAS
};

__device__ __forceinline__ void trav_init(Trav& t, const RayPre& r, float tmax) {
    t.g_base = 0;
    t.g_bits = 1u << 24;  // a virtual group holding the root
    t.sp = 0;
    t.iters = 0;
    t.tmax = tmax;
    t.h = Hit{tmax, HY_NO_HIT, 0.f, 0.f};
    t.pend_base = 0;
    t.pend_bits = 0;
    t.cur = r;
    t.inst_base = 0;
    t.inst_bits = 0;
    t.id_off = 0;
    t.sp_base = 0;
    t.level = false;
}

// world -> object: ((r.x o.x + r.y o.y) + r.z o.z) + r.w per row; the
// direction without r.w (not renormalised, so t is the same in both frames)
__device__ __forceinline__ f3 xform_point(float4 r0, float4 r1, float4 r2, f3 o) {
    const float4 R[3] = {r0, r1, r2};
    float v[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
        v[k] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(R[k].x, o.x), __fmul_rn(R[k].y, o.y)), __fmul_rn(R[k].z, o.z)),
                         R[k].w);
    return mk(v[0], v[1], v[2]);
}
__device__ __forceinline__ f3 xform_dir(float4 r0, float4 r1, float4 r2, f3 d) {
    const float4 R[3] = {r0, r1, r2};
    float v[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
        v[k] = __fadd_rn(__fadd_rn(__fmul_rn(R[k].x, d.x), __fmul_rn(R[k].y, d.y)), __fmul_rn(R[k].z, d.z));
    return mk(v[0], v[1], v[2]);
}

// A lane's world ray: its set-up in registers (RayPre), or, for the two-level
// walk, in shared memory (WorldRaySlot: word k of lane t at p[128 k], the 16
// words of RayPre, conflict-free; 64 B a lane).  The two-level walk reads the
// world ray only to enter and leave instances, so its registers go to the walk.
// (Keeping only the origin and direction there and recomputing the set-up on
// leaving an instance freed more shared memory for L1 but made the 4K two-level
// frame slower: 293.4 against 282 ms.)
struct WorldRaySlot {
    float* p;
};
__device__ __forceinline__ f3 world_o(const RayPre& r) { return r.o; }
__device__ __forceinline__ f3 world_d(const RayPre& r) { return mk(r.d[0], r.d[1], r.d[2]); }
__device__ __forceinline__ const RayPre& world_pre(const RayPre& r) { return r; }
__device__ __forceinline__ const RayPre& world_set(RayPre& r, f3 o, f3 d) {
    r = ray_pre(o, d);
    return r;
}
__device__ __forceinline__ f3 world_o(const WorldRaySlot& w) { return mk(w.p[0], w.p[128], w.p[256]); }
__device__ __forceinline__ f3 world_d(const WorldRaySlot& w) { return mk(w.p[384], w.p[512], w.p[640]); }
__device__ __forceinline__ RayPre world_pre(const WorldRaySlot& w) {
    RayPre r;
    r.o = world_o(w);
    r.d[0] = w.p[384]; r.d[1] = w.p[512]; r.d[2] = w.p[640];
    r.kx = __float_as_int(w.p[768]); r.ky = __float_as_int(w.p[896]); r.kz = __float_as_int(w.p[1024]);
    r.Sx = w.p[1152]; r.Sy = w.p[1280]; r.Sz = w.p[1408];
    r.invd[0] = w.p[1536]; r.invd[1] = w.p[1664]; r.invd[2] = w.p[1792];
    r.near = __float_as_uint(w.p[1920]);
    return r;
}
__device__ __forceinline__ RayPre world_set(WorldRaySlot& w, f3 o, f3 d) {
    const RayPre r = ray_pre(o, d);
    w.p[0] = r.o.x; w.p[128] = r.o.y; w.p[256] = r.o.z;
    w.p[384] = r.d[0]; w.p[512] = r.d[1]; w.p[640] = r.d[2];
    w.p[768] = __int_as_float(r.kx); w.p[896] = __int_as_float(r.ky); w.p[1024] = __int_as_float(r.kz);
    w.p[1152] = r.Sx; w.p[1280] = r.Sy; w.p[1408] = r.Sz;
    w.p[1536] = r.invd[0]; w.p[1664] = r.invd[1]; w.p[1792] = r.invd[2];
    w.p[1920] = __uint_as_float(r.near);
    return r;
}

// the ray of the level being walked: the world ray, or (two-level) t.cur
template <bool TWO, class RW>
__device__ __forceinline__ const RayPre& cur_ray(const Trav& t, const RW& rw) {
    if constexpr (TWO) return t.cur;
    else return rw;
}

// Two-level walk: brings t to a non-empty node group.  A TLAS leaf hands its
// hit instance entries over one at a time; entering one saves the pending
// TLAS group on the stack, moves the ray into object space and walks the
// BLAS above the saved stack height; once that part of the stack is empty
// the world ray is restored.  Returns false when the walk is over.
template <class Stack, class RW>
__device__ __forceinline__ bool two_level_settle(const SceneDev& S, const RW& rw, Trav& t, Stack stk,
                                                 uint32_t* status) {
    for (;;) {
        if (!t.level && t.inst_bits) {
            if (t.g_bits & 0xff000000u) {
                if (t.sp >= S.stack_cap) { atomicOr(status, HY_STATUS_STACK_OVERFLOW); return false; }
                stack_put(stk, t.sp, make_uint2(t.g_base, t.g_bits));
                t.sp++;
            }
            const uint32_t b = __ffs(t.inst_bits) - 1;
            t.inst_bits &= t.inst_bits - 1u;
            const uint32_t rec = t.inst_base + b;
            if (rec >= S.num_tris) { atomicOr(status, HY_STATUS_BAD_INDEX); return false; }
            const uint32_t iid = __float_as_uint(__ldg(&S.tris[(size_t)rec * 3].w));
            if (iid >= S.num_inst) { atomicOr(status, HY_STATUS_BAD_INDEX); return false; }
            const float4* I = S.inst + (size_t)iid * 4;
            const float4 r0 = __ldg(I), r1 = __ldg(I + 1), r2 = __ldg(I + 2), m = __ldg(I + 3);
            t.cur = ray_pre(xform_point(r0, r1, r2, world_o(rw)), xform_dir(r0, r1, r2, world_d(rw)));
            t.level = true;
            t.sp_base = t.sp;
            t.id_off = __float_as_uint(m.y);
            t.g_base = __float_as_uint(m.x);
            t.g_bits = 1u << 24;  // virtual group holding the BLAS root
            return true;
        }
        if (t.g_bits & 0xff000000u) return true;
        if (t.level && t.sp == t.sp_base) {
            t.level = false;
            t.cur = world_pre(rw);
            continue;
        }
        if (t.sp == 0) return false;
        --t.sp;
        const uint2 e = stack_get(stk, t.sp);
        t.g_base = e.x;
        t.g_bits = e.y;
    }
}

// One node visit: its 8 box tests; hit internal children become the next
// node group (the rest of the current group goes to the stack), the
// triangles of hit leaf slots become the ray's pending triangles
// (t.pend_base / t.pend_bits), which trav_tri tests before the ray's next
// node visit.  Returns true when the walk is over (nothing left, or a limit
// ran out).  A caller that interleaves trav_node and trav_tri this way makes
// the same node visits and triangle tests, in the same order, as a walk that
// tests each node's triangles at once.
// TWO: the two-level structure (r is the world ray; t.cur the current one).
// top / ntop: the structure's first ntop nodes (its top levels, BFS order)
// staged in shared memory by the caller's block.
template <bool ANY, bool COUNT, bool TWO = false, class Stack = uint2*, class RW = RayPre>
__device__ __forceinline__ bool trav_node(const SceneDev& S, const RW& rw, float tmin, Trav& t, Stack stk,
                                          uint32_t& nodes_ctr, uint32_t* status, const uint4* top = nullptr,
                                          uint32_t ntop = 0) {
    if (++t.iters > S.max_iters) { atomicOr(status, HY_STATUS_TIMEOUT); return true; }
    if (TWO) {
        if (!two_level_settle(S, rw, t, stk, status)) return true;
    } else if ((t.g_bits & 0xff000000u) == 0) {
        if (t.sp == 0) return true;
        --t.sp;
        const uint2 e = stack_get(stk, t.sp);
        t.g_base = e.x;
        t.g_bits = e.y;
    }
    const RayPre& r = cur_ray<TWO>(t, rw);
    const uint32_t rb = __ffs(t.g_bits >> 24) - 1;
    t.g_bits &= ~(1u << (24 + rb));
    const uint32_t ord = ANY ? r.near ^ S.anyhit_flip : r.near;
    const uint32_t sl = rb ^ ord;
    const uint32_t idx = t.g_base + __popc(t.g_bits & 0xffu & ((1u << sl) - 1u));
    if (t.g_bits & 0xff000000u) {
        if (t.sp >= S.stack_cap) { atomicOr(status, HY_STATUS_STACK_OVERFLOW); return true; }
        stack_put(stk, t.sp, make_uint2(t.g_base, t.g_bits));
        t.sp++;
    }
    if (idx >= S.num_nodes) { atomicOr(status, HY_STATUS_BAD_INDEX); return true; }
    uint4 q0, q1, q2, q3, q4;
    if (idx < ntop) {
        const uint4* np = top + (size_t)idx * 5;
        q0 = np[0]; q1 = np[1]; q2 = np[2]; q3 = np[3]; q4 = np[4];
    } else {
        const uint4* np = S.nodes[idx].q;
        q0 = __ldg(np + 0); q1 = __ldg(np + 1); q2 = __ldg(np + 2); q3 = __ldg(np + 3); q4 = __ldg(np + 4);
    }
    if (COUNT) nodes_ctr++;
    float adj[3], org[3];
    const float p[3] = {__uint_as_float(q0.x), __uint_as_float(q0.y), __uint_as_float(q0.z)};
    const float oo[3] = {r.o.x, r.o.y, r.o.z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const uint32_t ea = (q0.w >> (8 * a)) & 0xffu;
        adj[a] = __fmul_rn(__uint_as_float(ea << 23), r.invd[a]);
        org[a] = __fmul_rn(__fsub_rn(p[a], oo[a]), r.invd[a]);
    }
    const uint32_t imask = q0.w >> 24;
    // near/far planes per axis: a ray going in -a enters through the max plane,
    // so the quantised lo/hi byte planes swap once per node, not per child
    uint32_t qn[3][2], qf[3][2];
    {
        const uint32_t qlo[3][2] = {{q2.x, q2.y}, {q2.z, q2.w}, {q3.x, q3.y}};
        const uint32_t qhi[3][2] = {{q3.z, q3.w}, {q4.x, q4.y}, {q4.z, q4.w}};
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const bool neg = r.invd[a] < 0.f;
#pragma unroll
            for (int w = 0; w < 2; w++) {
                qn[a][w] = neg ? qhi[a][w] : qlo[a][w];
                qf[a][w] = neg ? qlo[a][w] : qhi[a][w];
            }
        }
    }
    uint32_t hitbits = 0;
    // Plane bytes as subnormal halves: one PRMT makes 0x00qq:0x00qq, the
    // halves q * 2^-24 of two slots, whose conversion to float is exact; with
    // adj scaled by 2^24 (exact) one fma gives q * adj + org rounded once, the
    // same value as fma(q, adj, org).  Per axis, the (near, far) pair of a
    // slot is one f32x2 fma.
    unsigned long long adj2[3], org2[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        const float a24 = __fmul_rn(adj[a], 16777216.0f);
        adj2[a] = f2_pack(a24, a24);
        org2[a] = f2_pack(org[a], org[a]);
    }
#pragma unroll
    for (int j = 0; j < 4; j++) {  // the slot pair 2j, 2j + 1: bytes (2j) & 3 and the next of word j / 2
        const uint32_t kSel = (j & 1) ? 0x4342u : 0x4140u;
        float tn[2][3], tf[2][3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            float n0, n1, f0, f1;
            h2_to_f2(__byte_perm(qn[a][j >> 1], 0u, kSel), n0, n1);
            h2_to_f2(__byte_perm(qf[a][j >> 1], 0u, kSel), f0, f1);
            f2_unpack(f2_fma(f2_pack(n0, f0), adj2[a], org2[a]), tn[0][a], tf[0][a]);
            f2_unpack(f2_fma(f2_pack(n1, f1), adj2[a], org2[a]), tn[1][a], tf[1][a]);
        }
#pragma unroll
        for (int h = 0; h < 2; h++) {
            // max(max(tn0, tn1), max(tn2, tmin)) and its min twin, as two instructions each
            const float tnear = fmaxf(fmax3(tn[h][0], tn[h][1], tn[h][2]), tmin);
            const float tfar = fminf(fmin3(tf[h][0], tf[h][1], tf[h][2]), t.tmax);
            if (tnear <= __fmul_rn(tfar, 1.0000003f)) hitbits |= 1u << (2 * j + h);
        }
    }
    // empty slots (meta byte 0) never count; internal children go to the stack
    // in rank order, leaf slots give their triangles
    hitbits &= nonzero_bytes(q1.z, q1.w);
    const uint32_t hit_int = slots_to_ranks(hitbits & imask, ord);
    uint32_t hit_leaf = hitbits & ~imask, hit_tri = 0;
    while (hit_leaf) {
        const uint32_t slot = __ffs(hit_leaf) - 1;
        hit_leaf &= hit_leaf - 1u;
        const uint32_t m = __byte_perm(q1.z, q1.w, slot) & 0xffu;
        hit_tri |= ((1u << (m >> 5)) - 1u) << (m & 31u);
    }
    if (TWO && !t.level) {  // TLAS leaves: instance entries, walked by two_level_settle
        t.inst_base = q1.y;
        t.inst_bits = hit_tri;
        hit_tri = 0;
    }
    t.pend_base = q1.y;
    t.pend_bits = hit_tri;
    t.g_base = q1.x;
    t.g_bits = (hit_int << 24) | imask;
    return false;
}

// The next pending triangle of the ray (t.pend_bits must be nonzero).
// Returns true when the walk is over: an any-hit ray that hit, or a bad index.
template <bool ANY, bool COUNT, bool TWO = false, class RW = RayPre>
__device__ __forceinline__ bool trav_tri(const SceneDev& S, const RW& rw, float tmin, Trav& t,
                                         uint32_t& tris_ctr, uint32_t* status) {
    const RayPre& r = cur_ray<TWO>(t, rw);
    const uint32_t b = __ffs(t.pend_bits) - 1;
    t.pend_bits &= t.pend_bits - 1u;
    const uint32_t rec = t.pend_base + b;
    if (rec >= S.num_tris) { atomicOr(status, HY_STATUS_BAD_INDEX); t.pend_bits = 0; return true; }
    const float4* tp = S.tris + (size_t)rec * 3;
    const float4 v0 = __ldg(tp), v1 = __ldg(tp + 1), v2 = __ldg(tp + 2);
    const uint32_t id = TWO ? t.id_off + __float_as_uint(v0.w) : __float_as_uint(v0.w);
    if (COUNT) tris_ctr++;
    float tt, b1, b2;
    if (tri_test(r, v0, v1, v2, tmin, t.tmax, tt, b1, b2)) {
        if (t.h.id == HY_NO_HIT || tt < t.h.t || (tt == t.h.t && id < t.h.id)) {
            t.h = Hit{tt, id, b1, b2};
            t.tmax = tt;
        }
        if (ANY) { t.pend_bits = 0; return true; }
    }
    return false;
}

// One node visit and then its triangles (the walk of a single ray).
// Returns true when the ray is finished: t.h holds the hit, or id HY_NO_HIT.
template <bool ANY, bool COUNT, bool TWO = false, class Stack = uint2*, class RW = RayPre>
__device__ __forceinline__ bool trav_step(const SceneDev& S, const RW& rw, float tmin, Trav& t, Stack stk,
                                          uint32_t& nodes_ctr, uint32_t& tris_ctr, uint32_t* status,
                                          const uint4* top = nullptr, uint32_t ntop = 0) {
    if (trav_node<ANY, COUNT, TWO>(S, rw, tmin, t, stk, nodes_ctr, status, top, ntop)) return true;
    while (t.pend_bits)
        if (trav_tri<ANY, COUNT, TWO>(S, rw, tmin, t, tris_ctr, status)) return true;
    return false;
}

template <bool ANY, bool COUNT, bool TWO = false>
__device__ __forceinline__ Hit traverse(const SceneDev& S, const RayPre& r, float tmin, float tmax,
                                        uint32_t* nodes_ctr, uint32_t* tris_ctr, uint32_t* status) {
    uint2 stk[kStackMax];
    Trav t;
    trav_init(t, r, tmax);
    uint32_t nn = 0, nt = 0;
    while (!trav_step<ANY, COUNT, TWO>(S, r, tmin, t, stk, nn, nt, status)) {
    }
    if (COUNT) { *nodes_ctr += nn; *tris_ctr += nt; }
    return t.h;
}

}  // namespace hy
