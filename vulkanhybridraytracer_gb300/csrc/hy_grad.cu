// Adjoint of the shading pass on sm_103a.
//
// The differentiated function is the image of hybridRaygen.rgen:27-186 with
// hybridHit.rchit:24-183 and miss.rmiss, as k_pixels<MODE_SHADE> computes it,
// with respect to each material's diffuse colour / roughness / metallic and
// each light's position / intensity.  Visibility is held fixed: the shadow
// images the primary shading reads, the bounce rays' hits and the bounce-hit
// shadow rays are constants (edges and soft-shadow boundaries are not
// differentiated).
//
// One lane per pixel, persistent warps over 8x4 tiles as in the forward pass:
//   1. re-trace the pixel's bounce chain with the forward's own closest-hit
//      program (hit records are recomputed, never stored by the forward),
//      recording each payload colour and the hit shadow rays' outcome;
//   2. walk the lights of the primary shading with 10-tangent dual numbers
//      (diffuse rgb, roughness, metallic, light position xyz, intensity, and
//      a slot for an attenuation carried over from an earlier light),
//      contracting each term with dLoss/dColour * prod(payloads);
//   3. walk each bounce hit's lights the same way, contracting with
//      dLoss/dColour * rayColor * prod(other payloads).
// Light gradients are summed across the warp and added to a block-local copy
// of the gradient vector in shared memory; material gradients are summed per
// distinct material of the warp.  Each block writes its partial vector once
// and a second kernel sums the partials.
#include <cuda_runtime.h>

#include "hy_dual.cuh"
#include "hy_shade.cuh"

namespace hy {

namespace {

constexpr int KG = 10;
enum { S_ALB = 0, S_ROUGH = 3, S_METAL = 4, S_LPOS = 5, S_INT = 8, S_ATT = 9 };
using Dg = Dn<KG>;
using Dg3 = Dn3<KG>;

__device__ __forceinline__ Dg3 dc3(f3 a) { return dvec<KG>(a.x, a.y, a.z); }
__device__ __forceinline__ f3 val3(const Dg3& a) { return mk(a.x.v, a.y.v, a.z.v); }
__device__ __forceinline__ Dg dotc(f3 a, const Dg3& b) { return b.x * a.x + b.y * a.y + b.z * a.z; }
__device__ __forceinline__ Dg3 mulc(const Dg3& a, f3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ __forceinline__ Dg3 one_minus(const Dg3& a) { return {1.0f - a.x, 1.0f - a.y, 1.0f - a.z}; }
__device__ __forceinline__ Dg3 div3(const Dg3& a, const Dg& s) { return {a.x / s, a.y / s, a.z / s}; }

// material inputs: albedo = pow(diffuse, 2.2); F0 = mix(vec3(0.04), albedo, metallic)
struct DMat { Dg3 albedo, F0; Dg rough, metal; };

// var_alb / var_rm: the diffuse colour / roughness-metallic are the material's own
// parameters (false where a texture supplies them: constants)
__device__ __forceinline__ DMat dmat(float dr, float dg, float db, float rough, float metal, bool var_alb = true,
                                     bool var_rm = true) {
    DMat m;
    m.albedo.x = dpow(var_alb ? dvar<KG>(dr, S_ALB + 0) : dconst<KG>(dr), 2.2f);
    m.albedo.y = dpow(var_alb ? dvar<KG>(dg, S_ALB + 1) : dconst<KG>(dg), 2.2f);
    m.albedo.z = dpow(var_alb ? dvar<KG>(db, S_ALB + 2) : dconst<KG>(db), 2.2f);
    m.rough = var_rm ? dvar<KG>(rough, S_ROUGH) : dconst<KG>(rough);
    m.metal = var_rm ? dvar<KG>(metal, S_METAL) : dconst<KG>(metal);
    const Dg keep = 1.0f - m.metal;
    m.F0 = {0.04f * keep + m.albedo.x * m.metal, 0.04f * keep + m.albedo.y * m.metal,
            0.04f * keep + m.albedo.z * m.metal};
    return m;
}

// helpers.glsl:33-80 on dual numbers
__device__ __forceinline__ Dg d_ggx(f3 N, const Dg3& H, const Dg& rough) {
    const Dg a = rough * rough;
    const Dg a2 = a * a;
    const Dg NdotH = dmax(dotc(N, H), 0.0f);
    const Dg NdotH2 = NdotH * NdotH;
    Dg denom = NdotH2 * (a2 - 1.0f) + 1.0f;
    denom = PI * denom * denom;
    return a2 / denom;
}
__device__ __forceinline__ Dg d_schlick_ggx(const Dg& NdotV, const Dg& rough) {
    const Dg r = rough + 1.0f;
    const Dg k = (r * r) / 8.0f;
    return NdotV / (NdotV * (1.0f - k) + k);
}
__device__ __forceinline__ Dg d_smith(f3 N, f3 V, const Dg3& L, const Dg& rough) {
    const Dg NdotV = dconst<KG>(fmaxf(dot(N, V), 0.0f));
    const Dg NdotL = dmax(dotc(N, L), 0.0f);
    return d_schlick_ggx(NdotV, rough) * d_schlick_ggx(NdotL, rough);
}
__device__ __forceinline__ Dg3 d_fresnel(const Dg& cosTheta, const Dg3& F0) {
    const Dg p = dpow(1.0f - cosTheta, 5.0f);
    return {F0.x + (1.0f - F0.x) * p, F0.y + (1.0f - F0.y) * p, F0.z + (1.0f - F0.z) * p};
}

// one light seen from a shading point; the position and intensity are the
// light's tangent slots
struct DLight { Dg3 L; Dg dist, I, NdotL; float maxd; bool isDir; };

__device__ __forceinline__ DLight d_light(const HyLight& lt, f3 pos, f3 N) {
    DLight g;
    g.isDir = lt.pos[3] < 0.f;
    g.maxd = lt.pos[3];
    const Dg3 lp{dvar<KG>(lt.pos[0], S_LPOS + 0), dvar<KG>(lt.pos[1], S_LPOS + 1), dvar<KG>(lt.pos[2], S_LPOS + 2)};
    const Dg3 L = g.isDir ? lp : lp - dc3(pos);
    g.dist = dlength(L);
    g.L = div3(L, g.dist);
    g.I = g.isDir ? dconst<KG>(1.0f) : dvar<KG>(lt.color[3], S_INT) / (g.dist * g.dist);
    g.NdotL = dclamp(dotc(N, g.L), 0.f, 1.f);
    return g;
}

// the attenuation both shaders compute from a light
__device__ __forceinline__ Dg d_atten(const DLight& g) {
    if (g.I.v == 0.f) return dconst<KG>(0.f);
    if (g.isDir) return dconst<KG>(0.3f);
    const Dg a = dmax((g.maxd - g.dist) / g.maxd, 0.f);
    return a * a;
}

// hybridRaygen.rgen:73-149: the term one light adds to rayColor
__device__ __forceinline__ Dg3 d_primary_term(int smode, const DMat& m, f3 N, f3 V, float NdotV, const DLight& g,
                                              const Dg& att, float sfac, f3 lc, f3 irr) {
    if (smode == 0) {
        const Dg s = g.I * att * sfac;
        const Dg3 radiance{s * lc.x, s * lc.y, s * lc.z};
        const Dg3 H = dnormalize(dc3(V) + g.L);
        const Dg D = d_ggx(N, H, m.rough);
        const Dg G = d_smith(N, V, g.L, m.rough);
        const Dg3 F = d_fresnel(dmax(dotc(V, H), 0.f), m.F0);
        const Dg3 kD = one_minus(F) * (1.0f - m.metal);
        const Dg3 numerator = F * (D * G);
        const Dg denominator = dmax((4.0f * NdotV) * g.NdotL, 0.001f);
        const Dg3 specular = div3(numerator, denominator);
        const Dg3 brdf = kD * m.albedo * (1.0f / PI) + specular;
        return brdf * radiance * g.NdotL;
    }
    if (smode == 3) {
        if (g.NdotL.v > 0.f && g.I.v > 0.f) return mulc(m.albedo * (g.I * att * sfac * m.metal), lc);
        return mulc(m.albedo * m.metal, irr);
    }
    if (smode == 4) {
        if (g.I.v > 0.f) return mulc(m.albedo * (g.I * att * m.metal), lc);
        return mulc(m.albedo * m.metal, irr);
    }
    return dc3(mk(0.f, 0.f, 0.f));
}

// hybridHit.rchit:92-171: the term one light adds to Lo (shadowFactor 1 or 2 is fixed)
__device__ __forceinline__ Dg3 d_hit_term(int smode, const DMat& m, f3 N, f3 V, float NdotV, const DLight& g,
                                          float shadowFactor, f3 lc, f3 irr) {
    const Dg att = d_atten(g);
    if (smode == 0) {
        const Dg s = g.I * att * shadowFactor;
        const Dg3 radiance{s * lc.x, s * lc.y, s * lc.z};
        const Dg3 H = dnormalize(dc3(V) + g.L);
        const Dg NdotH = dclamp(dotc(N, H), 0.f, 1.f);
        const Dg3 F = d_fresnel(NdotH, m.F0);
        const Dg D = d_ggx(N, H, m.rough);
        const Dg G = d_smith(N, V, g.L, m.rough);
        const Dg3 numerator = F * (D * G);
        const Dg denominator = dmax((4.0f * NdotV) * g.NdotL, 0.000001f);
        const Dg3 specular = div3(numerator, denominator);
        const Dg3 kD = one_minus(F) * (1.0f - m.metal);
        const Dg3 brdf = kD * m.albedo * (1.0f / PI) + specular;
        return brdf * radiance * g.NdotL;
    }
    if (smode == 3) {
        if (g.NdotL.v > 0.f && g.I.v > 0.f) return mulc(m.albedo * (g.I * att * m.metal), lc);
        return mulc(m.albedo * m.metal, irr);
    }
    if (smode == 4) {
        if (g.I.v > 0.f) return mulc(m.albedo * (g.I * att * m.metal), lc);
        return mulc(m.albedo * m.metal, irr);
    }
    return dc3(mk(0.f, 0.f, 0.f));
}

// kD * albedo * irradiance with kD from FresnelSchlick(NdotV, F0)
__device__ __forceinline__ Dg3 d_ambient(const DMat& m, float NdotV, f3 irr) {
    const Dg3 F = d_fresnel(dconst<KG>(NdotV), m.F0);
    const Dg3 kD = one_minus(F) * (1.0f - m.metal);
    return mulc(kD * m.albedo, irr);
}

__device__ __forceinline__ void contract(const Dg3& t, f3 w, float c[KG]) {
#pragma unroll
    for (int j = 0; j < KG; j++) c[j] = w.x * t.x.d[j] + w.y * t.y.d[j] + w.z * t.z.d[j];
}

__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// warp-collective: add the warp's sum of c[0..3] to acc[base..base+3]
__device__ __forceinline__ void scatter_light(float* acc, uint32_t base, const float* c) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const float s = warp_sum(c[q]);
        if ((threadIdx.x & 31) == 0 && s != 0.f) atomicAdd(acc + base + q, s);
    }
}

// warp-collective: add each lane's v[0..4] to material `mat`'s five slots,
// one warp sum per distinct material among the lanes with `has`
__device__ __forceinline__ void scatter_material(float* acc, int mat, bool has, const float* v) {
    const uint32_t lane = threadIdx.x & 31;
    uint32_t pending = __ballot_sync(0xffffffffu, has);
    while (pending) {
        const int leader = __ffs(pending) - 1;
        const int m = __shfl_sync(0xffffffffu, mat, leader);
        const bool mine = has && mat == m;
        pending &= ~__ballot_sync(0xffffffffu, mine);
#pragma unroll
        for (int q = 0; q < 5; q++) {
            const float s = warp_sum(mine ? v[q] : 0.f);
            if (lane == (uint32_t)leader && s != 0.f) atomicAdd(acc + (size_t)m * 5 + q, s);
        }
    }
}

// ---- one pixel (all 32 lanes of the warp call this together) ----
__device__ __forceinline__ void grad_pixel(const SceneDev& S, const GradParams& G, uint32_t x, uint32_t y, bool valid,
                                           float* acc, LaneStats& ls) {
    const PassParams& P = G.P;
    const size_t plane = (size_t)P.W * P.H;
    const size_t pix = valid ? (size_t)y * P.W + x : 0;
    bool active = valid;
    float4 g0 = make_float4(0.f, 0.f, 0.f, 0.f), g1 = g0, g2 = g0, g4 = g0, up = g0;
    if (active) {
        g0 = fetch_texel(P.plane[0], P.fmt[0], pix);
        g1 = fetch_texel(P.plane[1], P.fmt[1], pix);
        up = __ldg(G.grad + pix);
        // background texels copy the G-buffer albedo: no scene parameter
        active = !(g0.w == 0.f && g1.w == 0.f) && (up.x != 0.f || up.y != 0.f || up.z != 0.f);
    }
    const int mi = active ? mat_index(g0.w, S.num_mats) : -1;
    const f3 gup = mk(up.x, up.y, up.z);

    // ---- geometry of the pixel (constants) ----
    f3 position = mk(0.f, 0.f, 0.f), N = mk(0.f, 0.f, 1.f), V = N, irr = mk(0.f, 0.f, 0.f);
    float NdotV = 0.f;
    int smode = 0;
    f3 origin = mk(0.f, 0.f, 0.f), direction = mk(0.f, 0.f, 0.f);
    if (active) {
        g2 = fetch_texel(P.plane[2], P.fmt[2], pix);
        g4 = fetch_texel(P.plane[4], P.fmt[4], pix);
        position = mk(g0.x, g0.y, g0.z);
        const f3 normal = mk(__fsub_rn(__fmul_rn(g1.x, 2.0f), 1.0f), __fsub_rn(__fmul_rn(g1.y, 2.0f), 1.0f),
                             __fsub_rn(__fmul_rn(g1.z, 2.0f), 1.0f));
        N = normalize_rn(normal);
        smode = mi >= 0 ? (int)S.mats[mi].smr[0] : 0;
        const float ior = mi >= 0 ? S.mats[mi].diffuse[3] : 1.f;
        V = normalize(P.cam_pos - position);
        NdotV = clampf(dot(N, V), 0.f, 1.f);
        irr = irradiance_at(S, N);
        // hybridRaygen.rgen sets the bounce ray inside the light loop; it
        // depends on the geometry only
        if (P.num_lights > 0 && smode == 3) {
            direction = reflect(normalize(-V), N);
            origin = position;
        }
        if (P.num_lights > 0 && smode == 4) {
            origin = position;
            const float cosAlpha = dot(N, V);
            const f3 Iv = -V;
            const float NdotI = dot(N, Iv);
            const f3 refrN = NdotI > 0.f ? -N : N;
            const float eta = NdotI > 0.f ? 1.0f / ior : ior;
            const float radicand = 1.0f + powf(eta, 2.0f) * (cosAlpha * cosAlpha - 1.0f);
            direction = radicand < 0.f ? reflect(Iv, N) : refract(Iv, refrN, eta);
        }
    }

    // ---- 1. the bounce chain, re-traced (hybridRaygen.rgen:151-170) ----
    Hit hits[kGradMaxBounces];
    f3 ros[kGradMaxBounces], rds[kGradMaxBounces], pcs[kGradMaxBounces];
    unsigned long long vis[kGradMaxBounces];
    int nb = 0;
    if (active && smode != 0) {
        uint32_t seed = tea(y * P.W + x, P.frame_u);
        // the forward's GGX-sampled first bounce (a constant here: visibility is held fixed)
        if ((P.flags & HY_FLAG_GGX_REFLECTION) && smode == 3 && P.max_bounces > 0) {
            const float u1 = rnd(seed), u2 = rnd(seed);
            direction = ggx_reflect(N, V, g4.y, u1, u2);
        }
        for (uint32_t depth = 0; depth < P.max_bounces && depth < (uint32_t)kGradMaxBounces; depth++) {
            const f3 ro = origin + direction * 1e-2f;
            const Hit h = trace<false, false>(S, ro, direction, 0.001f, 1000.0f, ls, P.status);
            ls.refl++;
            f3 pc, pdir = direction, porg = origin;
            float pt, pw = 0.f;
            unsigned long long vb = 0ull;
            if (h.id == HY_NO_HIT) {
                pc = miss_color(S, direction);
                pt = -1.f;
            } else {
                const Payload p = closest_hit<false, true>(S, P, h, ro, direction, seed, ls, &vb);
                pc = p.color; pt = p.t; pdir = p.dir; pw = p.scattered; porg = p.origin;
            }
            hits[nb] = h; ros[nb] = ro; rds[nb] = direction; pcs[nb] = pc; vis[nb] = vb;
            nb++;
            if (pt < 0.f || !(pw > 0.f)) break;
            origin = porg;
            direction = pdir;
        }
    }
    f3 chain = mk(1.f, 1.f, 1.f);
    for (int k = 0; k < nb; k++) chain = chain * pcs[k];

    // ---- 2. primary lights (hybridRaygen.rgen:73-149) ----
    // a texel whose material samples a texture holds the texture's value, not a parameter
    const bool var_alb = mi >= 0 && !(S.mats[mi].textures[0] > -1.f);
    const bool var_rm = mi >= 0 && !(S.mats[mi].textures[3] > -1.f);
    const DMat m = dmat(g2.x, g2.y, g2.z, g4.y, g4.z, var_alb, var_rm);
    const f3 w_rc = gup * chain;  // dLoss/d(rayColor before the bounces)
    f3 rc0 = mk(0.f, 0.f, 0.f);
    float macc[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    // attenuation carried between lights: value, the light it came from
    // (-1: a constant) and its gradient with respect to that light's position
    float att_v = 1.0f, pend = 0.f;
    int att_src = -1;
    f3 att_dp = mk(0.f, 0.f, 0.f);
    for (uint32_t i = 0; i < P.num_lights; i++) {
        float c[KG];
#pragma unroll
        for (int j = 0; j < KG; j++) c[j] = 0.f;
        if (active) {
            const HyLight lt = S.lights[i];
            const DLight g = d_light(lt, position, N);
            Dg att;
            if (g.NdotL.v > 0.f) {
                // a fresh attenuation: hand the stale one's gradient to its light
                if (att_src >= 0 && pend != 0.f) {
                    float* dst = acc + G.light_off + (size_t)att_src * 4;
                    atomicAdd(dst + 0, pend * att_dp.x);
                    atomicAdd(dst + 1, pend * att_dp.y);
                    atomicAdd(dst + 2, pend * att_dp.z);
                }
                pend = 0.f;
                att = d_atten(g);
                att_v = att.v;
                att_dp = mk(att.d[S_LPOS + 0], att.d[S_LPOS + 1], att.d[S_LPOS + 2]);
                att_src = (g.I.v == 0.f || g.isDir) ? -1 : (int)i;
            } else {
                att = att_src >= 0 ? dvar<KG>(att_v, S_ATT) : dconst<KG>(att_v);
            }
            const float sfac = accum_load(P.accum_fmt, P.hist, i * plane + pix);
            const f3 lc = mk(lt.color[0], lt.color[1], lt.color[2]);
            const Dg3 t = d_primary_term(smode, m, N, V, NdotV, g, att, sfac, lc, irr);
            rc0 = rc0 + val3(t);
            contract(t, w_rc, c);
            pend += c[S_ATT];
        }
#pragma unroll
        for (int q = 0; q < 5; q++) macc[q] += c[q];
        scatter_light(acc, G.light_off + i * 4, c + S_LPOS);
    }
    if (active && att_src >= 0 && pend != 0.f) {
        float* dst = acc + G.light_off + (size_t)att_src * 4;
        atomicAdd(dst + 0, pend * att_dp.x);
        atomicAdd(dst + 1, pend * att_dp.y);
        atomicAdd(dst + 2, pend * att_dp.z);
    }
    if (active) {
        float c[KG];
        contract(d_ambient(m, NdotV, irr), gup, c);
#pragma unroll
        for (int q = 0; q < 5; q++) macc[q] += c[q];
    }
    scatter_material(acc, mi, active && mi >= 0, macc);

    // ---- 3. bounce hits (hybridHit.rchit) ----
    const int kmax = (int)__reduce_max_sync(0xffffffffu, (uint32_t)nb);
    for (int k = 0; k < kmax; k++) {
        const bool has = k < nb && hits[k].id != HY_NO_HIT;
        DMat hm = m;
        f3 Nh = N, Vh = V, wp = position, irr_h = irr, wk = mk(0.f, 0.f, 0.f);
        float NdotV_h = 0.f;
        int hsm = 0, hmat = 0;
        unsigned long long vb = 0ull;
        if (has) {
            wk = gup * rc0;
            for (int j = 0; j < nb; j++)
                if (j != k) wk = wk * pcs[j];
            const HitAttr a = hit_attributes(S, hits[k]);
            Nh = a.N;
            Vh = normalize(-rds[k]);
            NdotV_h = clampf(dot(Nh, Vh), 0.f, 1.f);
            wp = ros[k] + rds[k] * hits[k].t;
            hmat = (int)S.prims[a.prim].material_id;
            const HyMaterial mat = S.mats[hmat];
            hsm = (int)mat.smr[0];
            const MatSample ms = material_at_hit(S, mat, hits[k]);
            hm = dmat(ms.albedo.x, ms.albedo.y, ms.albedo.z, ms.rm.y, ms.rm.z, !(mat.textures[0] > -1.f),
                      !(mat.textures[3] > -1.f));
            irr_h = irradiance_at(S, Nh);
            vb = vis[k];
        }
        float hacc[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
        for (uint32_t i = 0; i < P.num_lights; i++) {
            float c[KG];
#pragma unroll
            for (int j = 0; j < KG; j++) c[j] = 0.f;
            if (has) {
                const HyLight lt = S.lights[i];
                const DLight g = d_light(lt, wp, Nh);
                const float sf = ((vb >> i) & 1ull) ? 2.0f : 1.0f;
                const f3 lc = mk(lt.color[0], lt.color[1], lt.color[2]);
                contract(d_hit_term(hsm, hm, Nh, Vh, NdotV_h, g, sf, lc, irr_h), wk, c);
            }
#pragma unroll
            for (int q = 0; q < 5; q++) hacc[q] += c[q];
            scatter_light(acc, G.light_off + i * 4, c + S_LPOS);
        }
        if (has) {
            float c[KG];
            contract(d_ambient(hm, NdotV_h, irr_h), wk, c);
#pragma unroll
            for (int q = 0; q < 5; q++) hacc[q] += c[q];
        }
        scatter_material(acc, hmat, has, hacc);
    }
}

template <bool SMEM>
__global__ void __launch_bounds__(128) k_shade_grad(const SceneDev S, const GradParams G) {
    extern __shared__ float s_acc[];
    float* acc = SMEM ? s_acc : G.out;
    if (SMEM) {
        for (uint32_t j = threadIdx.x; j < G.nparam; j += blockDim.x) s_acc[j] = 0.f;
        __syncthreads();
    }
    const PassParams& P = G.P;
    LaneStats ls;
    const uint32_t lane = threadIdx.x & 31;
    for (;;) {
        uint32_t t0 = 0;
        if (lane == 0) t0 = atomicAdd(P.queue, P.chunk);
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        if (t0 >= P.ntiles) break;
        const uint32_t t1 = min(t0 + P.chunk, P.ntiles);
        for (uint32_t t = t0; t < t1; t++) {
            const uint32_t tx = t % P.tiles_x, ty = t / P.tiles_x;
            const uint32_t x = tx * 8 + (lane & 7), y = ty * 4 + (lane >> 3);
            grad_pixel(S, G, x, y, x < P.W && y < P.H, acc, ls);
        }
    }
    flush_stats(ls, P.stats);
    if (SMEM) {
        __syncthreads();
        float* row = G.out + (size_t)blockIdx.x * G.nparam;
        for (uint32_t j = threadIdx.x; j < G.nparam; j += blockDim.x) row[j] = s_acc[j];
    }
}

// sum of `rows` partial vectors; block (32, 8): 32 parameters x 8 row phases
__global__ void __launch_bounds__(256) k_grad_reduce(const float* __restrict__ partial, uint32_t rows,
                                                     uint32_t nparam, uint32_t light_off, float* out_mat,
                                                     float* out_light) {
    __shared__ float s[8][33];
    const uint32_t j = blockIdx.x * 32 + threadIdx.x;
    float sum = 0.f;
    if (j < nparam)
        for (uint32_t r = threadIdx.y; r < rows; r += 8) sum += partial[(size_t)r * nparam + j];
    s[threadIdx.y][threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.y == 0 && j < nparam) {
        float tot = 0.f;
#pragma unroll
        for (int q = 0; q < 8; q++) tot += s[q][threadIdx.x];
        if (j < light_off) {
            if (out_mat) out_mat[j] = tot;
        } else if (out_light) {
            out_light[j - light_off] = tot;
        }
    }
}

constexpr size_t kGradSmemMax = 64 * 1024;

}  // namespace

cudaError_t grad_launch_shape(uint32_t nparam, int num_sms, uint32_t ntiles, int* grid, bool* smem,
                              size_t* smem_bytes) {
    const size_t bytes = (size_t)nparam * 4;
    *smem = bytes <= kGradSmemMax;
    *smem_bytes = *smem ? bytes : 0;
    int per = 0;
    cudaError_t e;
    if (*smem) {
        e = cudaFuncSetAttribute(k_shade_grad<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmemMax);
        if (e != cudaSuccess) return e;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_shade_grad<true>, 128, *smem_bytes);
    } else {
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_shade_grad<false>, 128, 0);
    }
    if (e != cudaSuccess) return e;
    if (per <= 0) per = 1;
    long long g = (long long)per * num_sms;
    const long long need = ((long long)ntiles * 32 + 127) / 128;
    if (g > need) g = need;
    *grid = (int)(g > 0 ? g : 1);
    return cudaSuccess;
}

cudaError_t launch_shade_grad(const SceneDev& S, const GradParams& G, int grid, bool smem, size_t smem_bytes,
                              float* out_mat, float* out_light, cudaStream_t s) {
    cudaError_t e;
    if (smem) {
        k_shade_grad<true><<<grid, 128, smem_bytes, s>>>(S, G);
    } else {
        e = cudaMemsetAsync(G.out, 0, (size_t)G.nparam * 4, s);
        if (e != cudaSuccess) return e;
        k_shade_grad<false><<<grid, 128, 0, s>>>(S, G);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const uint32_t rows = smem ? (uint32_t)grid : 1u;
    k_grad_reduce<<<(G.nparam + 31) / 32, dim3(32, 8), 0, s>>>(G.out, rows, G.nparam, G.light_off, out_mat,
                                                                out_light);
    return cudaGetLastError();
}

}  // namespace hy
