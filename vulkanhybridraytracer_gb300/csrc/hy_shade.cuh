// Shading building blocks shared by the forward pass (hy_pass.cu) and its
// adjoint (hy_grad.cu): the miss/environment lookups, hit attributes and the
// closest-hit program of hybridHit.rchit.
#pragma once
#include <cuda_runtime.h>

#include "hy_device.cuh"
#include "hy_pass.h"

namespace hy {

struct LaneStats {
    uint32_t shadow = 0, refl = 0, hshadow = 0;
    unsigned long long nodes = 0, tris = 0;
};

__device__ __forceinline__ void flush_stats(const LaneStats& s, unsigned long long* out) {
    unsigned long long v[5] = {s.shadow, s.refl, s.hshadow, s.nodes, s.tris};
#pragma unroll
    for (int k = 0; k < 5; k++) {
        unsigned long long x = v[k];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0 && x) atomicAdd(out + k, x);
    }
}

// LV: the structure the caller's kernel is compiled for — 1 one-level, 2
// two-level, 0 either (chosen per call from the scene).  A kernel compiled for
// one holds one copy of the walk instead of both (the shade kernel's
// instruction-cache misses were its top stall).
template <bool ANY, bool COUNT, int LV = 0>
__device__ __forceinline__ Hit trace(const SceneDev& S, f3 o, f3 d, float tmin, float tmax, LaneStats& ls,
                                     uint32_t* status) {
    RayPre r = ray_pre(o, d);
    uint32_t nn = 0, nt = 0;
    Hit h;
    if constexpr (LV == 1) h = traverse<ANY, COUNT, false>(S, r, tmin, tmax, &nn, &nt, status);
    else if constexpr (LV == 2) h = traverse<ANY, COUNT, true>(S, r, tmin, tmax, &nn, &nt, status);
    else h = S.two_level ? traverse<ANY, COUNT, true>(S, r, tmin, tmax, &nn, &nt, status)
                         : traverse<ANY, COUNT, false>(S, r, tmin, tmax, &nn, &nt, status);
    if (COUNT) { ls.nodes += nn; ls.tris += nt; }
    return h;
}

// equirect NEAREST / REPEAT lookup of an RGBA8 map
__device__ __forceinline__ f3 env_lookup(const uchar4* px, uint32_t w, uint32_t h, float u, float v) {
    if (w == 0 || h == 0) return mk(0.f, 0.f, 0.f);
    if (!(u == u)) u = 0.f;
    if (!(v == v)) v = 0.f;
    float fx = floorf(u * (float)w), fy = floorf(v * (float)h);
    fx = fminf(fmaxf(fx, -1e9f), 1e9f);
    fy = fminf(fmaxf(fy, -1e9f), 1e9f);
    long long ix = (long long)fx % (long long)w, iy = (long long)fy % (long long)h;
    if (ix < 0) ix += w;
    if (iy < 0) iy += h;
    uchar4 c = px[(size_t)iy * w + (size_t)ix];
    return mk(__fdiv_rn((float)c.x, 255.f), __fdiv_rn((float)c.y, 255.f), __fdiv_rn((float)c.z, 255.f));
}
__device__ __forceinline__ f3 irradiance_at(const SceneDev& S, f3 N) {
    float u = 0.5f + atan2f(N.x, N.z) / (2.0f * PI);
    float v = 0.5f - asinf(N.y) / PI;
    return env_lookup(S.env1, S.env_w[1], S.env_h[1], u, v);
}
__device__ __forceinline__ f3 miss_color(const SceneDev& S, f3 d) {
    f3 dir = normalize(d);
    float u = 0.5f + atan2f(dir.x, dir.z) / (2.0f * PI_MISS);
    float v = 0.5f - asinf(dir.y) / PI_MISS;
    return pow3(env_lookup(S.env0, S.env_w[0], S.env_h[0], u, v), 2.2f);
}

// material texture `id` at (u, v): RGBA8, NEAREST / REPEAT
__device__ __forceinline__ f3 tex_lookup(const SceneDev& S, float id, float u, float v) {
    const int i = (int)id;
    if (i < 0 || (uint32_t)i >= S.num_tex) return mk(0.f, 0.f, 0.f);
    const uint4 t = __ldg(S.tex_tab + i);
    return env_lookup(S.tex_px + t.x, t.y, t.z, u, v);
}

__device__ __forceinline__ bool has_textures(const HyMaterial& m) {
    return m.textures[0] > -1.f || m.textures[2] > -1.f || m.textures[3] > -1.f;
}

// a material's inputs at a surface point (hybridHit.rchit:62-66, closesthit.rchit:74-81):
// albedo before pow(2.2), emissive, rm = (_, roughness, metallic)
struct MatSample { f3 albedo, emissive, rm; };
__device__ __forceinline__ MatSample material_at(const SceneDev& S, const HyMaterial& m, float u, float v) {
    MatSample r;
    r.albedo = m.textures[0] > -1.f ? tex_lookup(S, m.textures[0], u, v) : mk(m.diffuse[0], m.diffuse[1], m.diffuse[2]);
    r.emissive = m.textures[2] > -1.f ? tex_lookup(S, m.textures[2], u, v) : mk(0.f, 0.f, 0.f);
    r.rm = m.textures[3] > -1.f ? tex_lookup(S, m.textures[3], u, v) : mk(0.f, m.smr[2], m.smr[1]);
    return r;
}

__device__ __forceinline__ int mat_index(float f, uint32_t n) {
    if (!(f > -1.f && f < (float)n)) return -1;
    return (int)f;
}

struct LightGeo { f3 L; float dist, maxd, NdotL; bool isDir; };

__device__ __forceinline__ LightGeo light_geo(const HyLight& lt, f3 position, f3 N) {
    LightGeo g;
    g.isDir = lt.pos[3] < 0.f;
    f3 lp = mk(lt.pos[0], lt.pos[1], lt.pos[2]);
    f3 L = g.isDir ? lp : sub_rn(lp, position);
    g.maxd = lt.pos[3];
    g.dist = length_rn(L);
    g.L = normalize_rn(L);
    g.NdotL = clampf(dot_rn(N, g.L), 0.f, 1.f);
    return g;
}

struct HitAttr { f3 N; uint32_t prim; };

__device__ __forceinline__ HitAttr hit_attributes(const SceneDev& S, const Hit& h) {
    uint32_t p = S.tri_prim[h.id];
    HyPrimitive pr = S.prims[p];
    uint32_t local = h.id - S.prim_tri0[p];
    float b0 = __fsub_rn(__fsub_rn(1.0f, h.b1), h.b2);
    float bw[3] = {b0, h.b1, h.b2};
    f3 n = mk(0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        uint32_t vi = S.idx[pr.first_index + 3 * local + k] + pr.vertex_offset;
        float4 a = __ldg(S.vattr + (size_t)vi * 2);
        n = n + mk(a.x, a.y, a.z) * bw[k];
    }
    const float* nm = S.nrm + (size_t)pr.transform_id * 9;
    f3 tn = mk(nm[0] * n.x + nm[3] * n.y + nm[6] * n.z, nm[1] * n.x + nm[4] * n.y + nm[7] * n.z,
               nm[2] * n.x + nm[5] * n.y + nm[8] * n.z);
    return HitAttr{normalize(tn), p};
}

// barycentric texture coordinates and vertex colour of a hit (uv = v0.uv*b0 + v1.uv*b1 + v2.uv*b2)
__device__ __forceinline__ void hit_uv_color(const SceneDev& S, const Hit& h, float& u, float& v, f3& col) {
    const uint32_t p = S.tri_prim[h.id];
    const HyPrimitive pr = S.prims[p];
    const uint32_t local = h.id - S.prim_tri0[p];
    const float b0 = __fsub_rn(__fsub_rn(1.0f, h.b1), h.b2);
    const float bw[3] = {b0, h.b1, h.b2};
    u = 0.f;
    v = 0.f;
    col = mk(0.f, 0.f, 0.f);
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const uint32_t vi = S.idx[pr.first_index + 3 * local + k] + pr.vertex_offset;
        const float4 a = __ldg(S.vattr + (size_t)vi * 2), t = __ldg(S.vattr + (size_t)vi * 2 + 1);
        u = __fadd_rn(u, __fmul_rn(t.x, bw[k]));
        v = __fadd_rn(v, __fmul_rn(t.y, bw[k]));
        col = add_rn(col, scale_rn(mk(a.w, t.z, t.w), bw[k]));
    }
}

// material inputs at a hit, sampling textures only for textured materials
__device__ __forceinline__ MatSample material_at_hit(const SceneDev& S, const HyMaterial& m, const Hit& h) {
    if (!has_textures(m)) return MatSample{mk(m.diffuse[0], m.diffuse[1], m.diffuse[2]), mk(0.f, 0.f, 0.f),
                                           mk(0.f, m.smr[2], m.smr[1])};
    float u, v;
    f3 col;
    hit_uv_color(S, h, u, v, col);
    return material_at(S, m, u, v);
}

struct Payload { f3 color; float t; f3 dir; float scattered; f3 origin; };

// hybridHit.rchit:24-183.  REC: also record, per light, whether the shadow
// factor came out 2 (lit side and unoccluded) into bit i of *vis — the
// visibility the adjoint holds fixed.
template <bool COUNT, bool REC = false, int LV = 0>
__device__ Payload closest_hit(const SceneDev& S, const PassParams& P, const Hit& h, f3 ro, f3 rd, uint32_t& seed,
                               LaneStats& ls, unsigned long long* vis = nullptr) {
    HitAttr a = hit_attributes(S, h);
    f3 N = a.N;
    f3 V = normalize(-rd);
    float NdotV = clampf(dot(N, V), 0.f, 1.f);
    f3 worldPos = ro + rd * h.t;
    HyPrimitive pr = S.prims[a.prim];
    const HyMaterial mat = S.mats[pr.material_id];
    int smode = (int)mat.smr[0];
    const MatSample ms = material_at_hit(S, mat, h);
    f3 albedo = pow3(ms.albedo, 2.2f);
    float roughness = ms.rm.y, metallic = ms.rm.z;
    f3 F0 = mix3(splat(0.04f), albedo, metallic);
    f3 irradiance = irradiance_at(S, N);
    f3 direction = mk(1.f, 1.f, 1.f);
    float dirw = 0.f;
    f3 Lo = mk(0.f, 0.f, 0.f);
    float attenuation = 1.0f;
    if (REC) *vis = 0ull;
    for (uint32_t i = 0; i < P.num_lights; i++) {
        const HyLight lt = S.lights[i];
        bool isDir = lt.pos[3] < 0.f;
        f3 lp = mk(lt.pos[0], lt.pos[1], lt.pos[2]);
        f3 L = isDir ? lp : lp - worldPos;
        float maxd = lt.pos[3];
        float dist = length(L);
        L = normalize(L);
        float I = isDir ? 1.0f : (lt.color[3] / (dist * dist));
        f3 H = normalize(V + L);
        float NdotL = clampf(dot(N, L), 0.f, 1.f);
        float NdotH = clampf(dot(N, H), 0.f, 1.f);
        float shadowFactor = 1.0f;
        if (I == 0.f) attenuation = 0.f;
        else {
            attenuation = maxd - dist;
            attenuation /= maxd;
            attenuation = fmaxf(attenuation, 0.f);
            attenuation = isDir ? 0.3f : attenuation * attenuation;
        }
        f3 lc = mk(lt.color[0], lt.color[1], lt.color[2]);
        if (smode == 0) {
            if (NdotL > 0.f) {
                bool shadowed = true;
                if (dist < maxd) {
                    uint32_t sd = seed;
                    f3 dir = P.rng_mode == HY_RNG_REFERENCE ? sampleDisk(lt.radius, worldPos, L, sd)
                                                            : sampleDisk(lt.radius, worldPos, L, seed);
                    Hit sh = trace<true, COUNT, LV>(S, add_rn(worldPos, scale_rn(dir, 1e-2f)), dir, 0.001f,
                                                __fadd_rn(dist, 1.0f), ls, P.status);
                    ls.hshadow++;
                    shadowed = sh.id != HY_NO_HIT;
                }
                if (!shadowed) {
                    shadowFactor += 1.0f;
                    if (REC && i < 64) *vis |= 1ull << i;
                }
            }
            f3 radiance = I * lc * attenuation * shadowFactor;
            f3 F = FresnelSchlick(NdotH, F0);
            float D = DistributionGGX(N, H, roughness);
            float G = GeometrySmith(N, V, L, roughness);
            f3 numerator = D * G * F;
            float denominator = fmaxf(4.0f * clampf(dot(N, V), 0.f, 1.f) * NdotL, 0.000001f);
            f3 specular = numerator / denominator;
            f3 kD = (splat(1.0f) - F) * (1.0f - metallic);
            Lo = Lo + (kD * albedo / PI + specular) * radiance * NdotL;
            direction = mk(1.f, 1.f, 1.f);
            dirw = 0.f;
        } else if (smode == 3) {
            f3 reflected = reflect(normalize(rd), N);
            bool sc = dot(reflected, N) > 0.f;
            Lo = Lo + ((NdotL > 0.f && I > 0.f) ? I * lc * attenuation * albedo * metallic
                                                : irradiance * albedo * metallic);
            direction = reflected;
            dirw = sc ? 1.f : 0.f;
        } else if (smode == 4) {
            float ior = mat.diffuse[3];
            float NdV = dot(N, normalize(rd));
            f3 refrN = NdV > 0.f ? -N : N;
            float eta = NdV > 0.f ? 1.0f / ior : ior;
            Lo = Lo + ((I > 0.f) ? I * lc * attenuation * albedo * metallic : irradiance * albedo * metallic);
            float radicand = 1.0f + powf(eta, 2.0f) * (NdV * NdV - 1.0f);
            direction = radicand < 0.f ? reflect(rd, N) : refract(normalize(rd), refrN, eta);
            dirw = 1.f;
        }
    }
    f3 F = FresnelSchlick(NdotV, F0);
    f3 kD = (splat(1.0f) - F) * (1.0f - metallic);
    f3 ambient = kD * albedo * irradiance;
    Payload p;
    p.color = Lo + ambient + ms.emissive;
    p.t = h.t;
    p.dir = direction;
    p.scattered = dirw;
    p.origin = worldPos;
    return p;
}

}  // namespace hy
