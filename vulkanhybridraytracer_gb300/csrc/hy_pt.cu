// Path-traced mode on sm_103a: the reference's full ray-tracing pipeline
// (Renderer::raytrace, src/renderer.cpp:465-501) — raygen.rgen:20-81 camera
// rays and running mean, closesthit.rchit:26-186 shading with shadow rays at
// every hit, miss.rmiss sky, shadow.rmiss — over the same BVH8 traversal as
// the hybrid pass.  One lane per pixel; persistent warps pull 8x4 tiles.
#include <cuda_runtime.h>

#include "hy_shade.cuh"
#include "hy_stream.cuh"

namespace hy {

namespace {

// closesthit.rchit:26-186.  Unlike hybridHit.rchit every shading model casts
// the shadow rays, the shadow factor is the unoccluded fraction of
// samplesBuffer.samples rays, the attenuation has no directional special case
// and glass refracts the unnormalised ray direction.  Split in three so the
// warp-cooperative kernel can trace each light's shadow rays as a tile stream
// between the set-up and the shading: pt_hit (the hit's state), pt_light (one
// light's geometry), pt_shade_light (its contribution given the shadow factor).
struct PtHit {
    f3 N, V, worldPos, rd, albedo, F0, irradiance, emissive;
    float NdotV, roughness, metallic, ior, t;
    int smode;
};

__device__ __forceinline__ PtHit pt_hit(const SceneDev& S, const Hit& h, f3 ro, f3 rd) {
    PtHit c;
    HitAttr a = hit_attributes(S, h);
    c.N = a.N;
    c.V = normalize(-rd);
    c.NdotV = clampf(dot(c.N, c.V), 0.f, 1.f);
    // the shadow and bounce rays start here: single-rounded ops, as the CPU restatement
    c.worldPos = add_rn(ro, scale_rn(rd, h.t));
    c.rd = rd;
    c.t = h.t;
    const HyMaterial mat = S.mats[S.prims[a.prim].material_id];
    c.smode = (int)mat.smr[0];
    c.ior = mat.diffuse[3];
    const MatSample ms = material_at_hit(S, mat, h);
    c.albedo = pow3(ms.albedo, 2.2f);
    c.roughness = ms.rm.y;
    c.metallic = ms.rm.z;
    c.emissive = ms.emissive;
    c.F0 = mix3(splat(0.04f), c.albedo, c.metallic);
    c.irradiance = irradiance_at(S, c.N);
    return c;
}

struct PtLight {
    f3 L, H, lc;
    float dist, maxd, I, NdotL, NdotH;
};

__device__ __forceinline__ PtLight pt_light(const HyLight& lt, const PtHit& c) {
    PtLight g;
    const bool isDir = lt.pos[3] < 0.f;
    const f3 lp = mk(lt.pos[0], lt.pos[1], lt.pos[2]);
    f3 L = isDir ? lp : sub_rn(lp, c.worldPos);
    g.maxd = lt.pos[3];
    g.dist = length_rn(L);
    g.L = normalize_rn(L);
    g.I = isDir ? 1.0f : (lt.color[3] / (g.dist * g.dist));
    g.H = normalize(c.V + g.L);
    g.NdotL = clampf(dot_rn(c.N, g.L), 0.f, 1.f);
    g.NdotH = clampf(dot(c.N, g.H), 0.f, 1.f);
    g.lc = mk(lt.color[0], lt.color[1], lt.color[2]);
    return g;
}

// one light's term (closesthit.rchit:112-176); attenuation carries over to the
// next light as in the shader
__device__ __forceinline__ void pt_shade_light(const PtHit& c, const PtLight& g, float shadowFactor, f3& Lo,
                                               f3& direction, float& dirw, float& attenuation) {
    if (g.I == 0.f) attenuation = 0.f;
    else {
        attenuation = g.maxd - g.dist;
        attenuation /= g.maxd;
        attenuation = fmaxf(attenuation, 0.f);
        attenuation = attenuation * attenuation;
    }
    if (c.smode == 0) {
        f3 radiance = g.I * g.lc * attenuation * shadowFactor;
        f3 F = FresnelSchlick(g.NdotH, c.F0);
        float D = DistributionGGX(c.N, g.H, c.roughness);
        float G = GeometrySmith(c.N, c.V, g.L, c.roughness);
        f3 numerator = D * G * F;
        float denominator = fmaxf(4.0f * clampf(dot(c.N, c.V), 0.f, 1.f) * g.NdotL, 0.000001f);
        f3 specular = numerator / denominator;
        f3 kD = (splat(1.0f) - F) * (1.0f - c.metallic);
        Lo = Lo + (kD * c.albedo / PI + specular) * radiance * g.NdotL;
        direction = mk(1.f, 1.f, 1.f);
        dirw = 0.f;
    } else if (c.smode == 3) {
        f3 reflected = reflect(normalize(c.rd), c.N);
        bool sc = dot(reflected, c.N) > 0.f;
        Lo = Lo + ((g.NdotL > 0.f && g.I > 0.f) ? g.I * g.lc * attenuation * shadowFactor * c.metallic * c.albedo
                                                : c.irradiance * c.albedo * c.metallic);
        direction = reflected;
        dirw = sc ? 1.f : 0.f;
    } else if (c.smode == 4) {
        float NdV = dot(c.N, normalize(c.rd));
        f3 refrN = NdV > 0.f ? -c.N : c.N;
        float eta = NdV > 0.f ? 1.0f / c.ior : c.ior;
        Lo = Lo + ((g.I > 0.f) ? g.I * g.lc * attenuation * c.albedo * c.metallic : c.irradiance * c.albedo * c.metallic);
        float radicand = 1.0f + powf(eta, 2.0f) * (NdV * NdV - 1.0f);
        direction = radicand < 0.f ? reflect(c.rd, c.N) : refract(c.rd, refrN, eta);
        dirw = 1.f;
    }
}

__device__ __forceinline__ Payload pt_finish(const PtHit& c, f3 Lo, f3 direction, float dirw) {
    f3 F = FresnelSchlick(c.NdotV, c.F0);
    f3 kD = (splat(1.0f) - F) * (1.0f - c.metallic);
    Payload p;
    p.color = Lo + kD * c.albedo * c.irradiance + c.emissive;
    p.t = c.t;
    p.dir = direction;
    p.scattered = dirw;
    p.origin = c.worldPos;
    return p;
}

// the whole hit on one lane, its shadow rays traced in turn
template <bool COUNT>
__device__ Payload closest_hit_pt(const SceneDev& S, const PassParams& P, const Hit& h, f3 ro, f3 rd,
                                  uint32_t& seed, LaneStats& ls) {
    const PtHit c = pt_hit(S, h, ro, rd);
    f3 direction = mk(1.f, 1.f, 1.f), Lo = mk(0.f, 0.f, 0.f);
    float dirw = 0.f, attenuation = 1.0f;
    const float spp = (float)P.spp;
    for (uint32_t i = 0; i < P.num_lights; i++) {
        const HyLight lt = S.lights[i];
        const PtLight g = pt_light(lt, c);
        float shadowFactor = 0.f;
        if (g.NdotL > 0.f) {
            if (g.dist < g.maxd && P.rng_mode == HY_RNG_REFERENCE) {
                // sampleDisk takes the seed by value: every sample is this one ray
                uint32_t sd = seed;
                f3 dir = sampleDisk(lt.radius, c.worldPos, g.L, sd);
                Hit sh = trace<true, COUNT>(S, add_rn(c.worldPos, scale_rn(dir, 1e-2f)), dir, 0.001f,
                                            __fadd_rn(g.dist, 1.0f), ls, P.status);
                ls.shadow++;
                shadowFactor = sh.id == HY_NO_HIT ? spp : 0.f;
            } else {
                for (uint32_t k = 0; k < P.spp; k++) {
                    bool shadowed = true;
                    if (g.dist < g.maxd) {
                        f3 dir = sampleDisk(lt.radius, c.worldPos, g.L, seed);
                        Hit sh = trace<true, COUNT>(S, add_rn(c.worldPos, scale_rn(dir, 1e-2f)), dir, 0.001f,
                                                    __fadd_rn(g.dist, 1.0f), ls, P.status);
                        ls.shadow++;
                        shadowed = sh.id != HY_NO_HIT;
                    }
                    if (!shadowed) shadowFactor += 1.0f;
                }
            }
            shadowFactor /= spp;
        }
        pt_shade_light(c, g, shadowFactor, Lo, direction, dirw, attenuation);
    }
    return pt_finish(c, Lo, direction, dirw);
}

__device__ __forceinline__ f3 mat_vec3_rn(const float* m, float x, float y, float z, float w) {
    float r[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float a = __fmul_rn(m[0 * 4 + i], x);
        a = __fadd_rn(a, __fmul_rn(m[1 * 4 + i], y));
        a = __fadd_rn(a, __fmul_rn(m[2 * 4 + i], z));
        a = __fadd_rn(a, __fmul_rn(m[3 * 4 + i], w));
        r[i] = a;
    }
    return mk(r[0], r[1], r[2]);
}

// raygen.rgen:20-81: the camera ray of a pixel (NSAMPLES = 1, helpers.glsl:6:
// the pixel centre, but r1 and r2 are drawn)
__device__ __forceinline__ void pt_camera(const PtParams& T, uint32_t x, uint32_t y, uint32_t& seed, f3& origin,
                                          f3& direction) {
    const PassParams& P = T.P;
    seed = tea(y * P.W + x, (uint32_t)T.frame);
    rnd(seed);
    rnd(seed);
    const float ux = __fdiv_rn(__fadd_rn((float)x, 0.5f), (float)P.W);
    const float uy = __fdiv_rn(__fadd_rn((float)y, 0.5f), (float)P.H);
    const float dx = __fsub_rn(__fmul_rn(ux, 2.0f), 1.0f), dy = __fsub_rn(__fmul_rn(uy, 2.0f), 1.0f);
    origin = mat_vec3_rn(T.inv_view, 0.f, 0.f, 0.f, 1.f);
    const f3 tgt = mat_vec3_rn(T.inv_proj, dx, dy, 1.f, 1.f);
    const f3 tn = normalize_rn(tgt);
    direction = mat_vec3_rn(T.inv_view, tn.x, tn.y, tn.z, 0.f);
}

// raygen.rgen:69-80: the frame's colour, and the running mean against the
// 8-bit image
__device__ __forceinline__ void pt_output(const PtParams& T, size_t pix, f3 fc) {
    const PassParams& P = T.P;
    if (P.out_f) reinterpret_cast<float4*>(P.out_f)[pix] = make_float4(fc.x, fc.y, fc.z, 1.f);
    if (P.out_8) {
        uchar4* img = reinterpret_cast<uchar4*>(P.out_8);
        if (T.frame >= 0) {
            // mix(lastColor, finalColor, 1 / (1 + frame)) against the 8-bit image
            const uchar4 q = img[pix];
            const float a = __fdiv_rn(1.0f, __fadd_rn(1.0f, (float)T.frame));
            const float na = __fsub_rn(1.0f, a);
            const f3 last = mk(__fdiv_rn((float)q.z, 255.f), __fdiv_rn((float)q.y, 255.f), __fdiv_rn((float)q.x, 255.f));
            fc = mk(__fadd_rn(__fmul_rn(last.x, na), __fmul_rn(fc.x, a)),
                    __fadd_rn(__fmul_rn(last.y, na), __fmul_rn(fc.y, a)),
                    __fadd_rn(__fmul_rn(last.z, na), __fmul_rn(fc.z, a)));
        }
        img[pix] = make_uchar4(quant8(fc.z), quant8(fc.y), quant8(fc.x), 255);
    }
}

// raygen.rgen:20-81 for one pixel on one lane
template <bool COUNT>
__device__ __forceinline__ void pt_pixel(const SceneDev& S, const PtParams& T, uint32_t x, uint32_t y,
                                         LaneStats& ls) {
    const PassParams& P = T.P;
    uint32_t seed;
    f3 origin, direction;
    pt_camera(T, x, y, seed, origin, direction);
    f3 rayColor = mk(1.f, 1.f, 1.f);
    for (uint32_t depth = 0; depth < P.max_bounces; depth++) {
        const f3 ro = add_rn(origin, scale_rn(direction, 1e-2f));
        const Hit h = trace<false, COUNT>(S, ro, direction, 0.001f, 10000.0f, ls, P.status);
        ls.refl++;
        if (h.id == HY_NO_HIT) {
            rayColor = rayColor * miss_color(S, direction);
            break;
        }
        const Payload p = closest_hit_pt<COUNT>(S, P, h, ro, direction, seed, ls);
        rayColor = rayColor * p.color;
        if (!(p.scattered > 0.f)) break;
        origin = p.origin;
        direction = p.dir;
    }
    pt_output(T, (size_t)y * P.W + x, rayColor);
}

// One lane per pixel, each hit's shadow rays traced in turn on its lane
// (HY_FLAG_PIXEL_PARALLEL).
template <bool COUNT>
__global__ void __launch_bounds__(128) k_pathtrace(const SceneDev S, const PtParams T) {
    const PassParams& P = T.P;
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
            if (x < P.W && y < P.H) pt_pixel<COUNT>(S, T, x, y, ls);
        }
    }
    flush_stats(ls, P.stats);
}

// The default: a warp per 8x4 tile, one lane per pixel for the camera and
// bounce rays and the shading, each hit's shadow rays (lights in order) traced
// by the whole warp as tile streams (hy_stream.cuh).  Sample k of light l at a
// hit starts from the hit's RNG state advanced 2 (rays_before + k) LCG steps,
// exactly the state the per-lane loop reaches, and the per-light shading runs
// in the same order, so the image equals k_pathtrace's.
template <bool COUNT, bool TWO, int MINB>
__global__ void __launch_bounds__(128, MINB) k_pathtrace_stream(const SceneDev S, const PtParams T) {
    __shared__ StreamSlots sm;
    const PassParams& P = T.P;
    LaneStats ls;
    const uint32_t lane = threadIdx.x & 31, wb = threadIdx.x & ~31u;
    const bool reference = P.rng_mode == HY_RNG_REFERENCE;
    const uint32_t nrays = reference ? 1u : P.spp;
    const float spp = (float)P.spp;
    uint2 stk[kStackMax];
    Trav t;
    RayPre r;
    uint32_t nn = 0, nt = 0;
    for (;;) {
        uint32_t t0 = 0;
        if (lane == 0) t0 = atomicAdd(P.queue, P.chunk);
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        if (t0 >= P.ntiles) break;
        const uint32_t t1 = min(t0 + P.chunk, P.ntiles);
        for (uint32_t tile = t0; tile < t1; tile++) {
            const uint32_t x = (tile % P.tiles_x) * 8 + (lane & 7), y = (tile / P.tiles_x) * 4 + (lane >> 3);
            const bool present = x < P.W && y < P.H;
            uint32_t seed = 0;
            f3 origin = mk(0.f, 0.f, 0.f), direction = mk(0.f, 0.f, 1.f), rayColor = mk(1.f, 1.f, 1.f);
            if (present) pt_camera(T, x, y, seed, origin, direction);
            bool active = present;
            for (uint32_t depth = 0; depth < P.max_bounces; depth++) {
                if (__ballot_sync(0xffffffffu, active) == 0) break;
                bool hit = false;
                PtHit c;
                if (active) {
                    const f3 ro = add_rn(origin, scale_rn(direction, 1e-2f));
                    const Hit h = trace<false, COUNT>(S, ro, direction, 0.001f, 10000.0f, ls, P.status);
                    ls.refl++;
                    if (h.id == HY_NO_HIT) {
                        rayColor = rayColor * miss_color(S, direction);
                        active = false;
                    } else {
                        hit = true;
                        c = pt_hit(S, h, ro, direction);
                    }
                }
                f3 Lo = mk(0.f, 0.f, 0.f), dirv = mk(1.f, 1.f, 1.f);
                float dirw = 0.f, attenuation = 1.0f;
                uint32_t rays_before = 0;
                for (uint32_t i = 0; i < P.num_lights; i++) {
                    const HyLight lt = S.lights[i];
                    PtLight g;
                    bool traced = false;
                    if (hit) {
                        g = pt_light(lt, c);
                        traced = g.NdotL > 0.f && g.dist < g.maxd;
                    }
                    stream_publish(sm, traced, traced ? c.worldPos : mk(0.f, 0.f, 0.f), traced ? g.L : mk(0.f, 1.f, 0.f),
                                   traced ? g.dist : 0.f, !traced || reference ? seed : lcg_jump(seed, 2u * rays_before));
                    // closesthit.rchit: origin worldPos + 0.01 dir, tmax distance + 1
                    if (__ballot_sync(0xffffffffu, traced) != 0)
                        stream_light<COUNT, TWO>(S, P, sm, nrays, lt.radius, 1e-2f, stk, t, r, ls, nn, nt, nullptr, 0);
                    if (hit) {
                        float sf = 0.f;
                        if (g.NdotL > 0.f) {
                            const uint32_t cnt = traced ? *unocc_count(sm, wb + lane) : 0u;
                            sf = reference ? (cnt ? spp : 0.f) : (float)cnt;
                            sf /= spp;
                        }
                        pt_shade_light(c, g, sf, Lo, dirv, dirw, attenuation);
                    }
                    if (traced && !reference) rays_before += P.spp;
                    __syncwarp();  // the slots are rewritten by the next light
                }
                if (hit) {
                    const Payload p = pt_finish(c, Lo, dirv, dirw);
                    rayColor = rayColor * p.color;
                    if (!reference) seed = lcg_jump(seed, 2u * rays_before);
                    if (!(p.scattered > 0.f)) active = false;
                    origin = p.origin;
                    direction = p.dir;
                }
            }
            if (present) pt_output(T, (size_t)y * P.W + x, rayColor);
        }
    }
    if (COUNT) { ls.nodes += nn; ls.tris += nt; }
    flush_stats(ls, P.stats);
}

template <bool COUNT, int MINB>
static void* pt_stream_kernel(bool two) {
    return two ? (void*)k_pathtrace_stream<COUNT, true, MINB> : (void*)k_pathtrace_stream<COUNT, false, MINB>;
}
template <bool COUNT>
static void* pt_kernel(bool stream, bool two, int minb) {
    if (!stream) return (void*)k_pathtrace<COUNT>;
    if (minb >= 8) return pt_stream_kernel<COUNT, 8>(two);
    if (minb >= 6) return pt_stream_kernel<COUNT, 6>(two);
    if (minb == 5) return pt_stream_kernel<COUNT, 5>(two);
    if (minb == 4) return pt_stream_kernel<COUNT, 4>(two);
    if (minb == 3) return pt_stream_kernel<COUNT, 3>(two);
    return pt_stream_kernel<COUNT, 1>(two);
}

}  // namespace

cudaError_t pathtrace_occupancy(bool count, bool stream, bool two, int minb, int* blocks_per_sm) {
    void* k = count ? pt_kernel<true>(stream, two, minb) : pt_kernel<false>(stream, two, minb);
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k, 128, 0);
}

cudaError_t launch_pathtrace(bool count, bool stream, int minb, const SceneDev& S, const PtParams& T, int grid,
                             cudaStream_t s) {
    void* k = count ? pt_kernel<true>(stream, S.two_level != 0, minb) : pt_kernel<false>(stream, S.two_level != 0, minb);
    void* args[] = {(void*)&S, (void*)&T};
    return cudaLaunchKernel(k, dim3(grid), dim3(128), args, 0, s);
}

}  // namespace hy
