// Path-traced mode on sm_103a: the reference's full ray-tracing pipeline
// (Renderer::raytrace, src/renderer.cpp:465-501) — raygen.rgen:20-81 camera
// rays and running mean, closesthit.rchit:26-186 shading with shadow rays at
// every hit, miss.rmiss sky, shadow.rmiss — over the same BVH8 traversal as
// the hybrid pass.  One lane per pixel; persistent warps pull 8x4 tiles.
#include <cuda_runtime.h>

#include "hy_shade.cuh"

namespace hy {

namespace {

// closesthit.rchit:26-186.  Unlike hybridHit.rchit every shading model casts
// the shadow rays, the shadow factor is the unoccluded fraction of
// samplesBuffer.samples rays, the attenuation has no directional special case
// and glass refracts the unnormalised ray direction.
template <bool COUNT>
__device__ Payload closest_hit_pt(const SceneDev& S, const PassParams& P, const Hit& h, f3 ro, f3 rd,
                                  uint32_t& seed, LaneStats& ls) {
    HitAttr a = hit_attributes(S, h);
    f3 N = a.N;
    f3 V = normalize(-rd);
    float NdotV = clampf(dot(N, V), 0.f, 1.f);
    // the shadow and bounce rays start here: single-rounded ops, as the CPU restatement
    f3 worldPos = add_rn(ro, scale_rn(rd, h.t));
    const HyMaterial mat = S.mats[S.prims[a.prim].material_id];
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
    const float spp = (float)P.spp;
    for (uint32_t i = 0; i < P.num_lights; i++) {
        const HyLight lt = S.lights[i];
        bool isDir = lt.pos[3] < 0.f;
        f3 lp = mk(lt.pos[0], lt.pos[1], lt.pos[2]);
        f3 L = isDir ? lp : sub_rn(lp, worldPos);
        float maxd = lt.pos[3];
        float dist = length_rn(L);
        L = normalize_rn(L);
        float I = isDir ? 1.0f : (lt.color[3] / (dist * dist));
        f3 H = normalize(V + L);
        float NdotL = clampf(dot_rn(N, L), 0.f, 1.f);
        float NdotH = clampf(dot(N, H), 0.f, 1.f);
        float shadowFactor = 0.f;
        if (NdotL > 0.f) {
            if (dist < maxd && P.rng_mode == HY_RNG_REFERENCE) {
                // sampleDisk takes the seed by value: every sample is this one ray
                uint32_t sd = seed;
                f3 dir = sampleDisk(lt.radius, worldPos, L, sd);
                Hit sh = trace<true, COUNT>(S, add_rn(worldPos, scale_rn(dir, 1e-2f)), dir, 0.001f,
                                            __fadd_rn(dist, 1.0f), ls, P.status);
                ls.shadow++;
                shadowFactor = sh.id == HY_NO_HIT ? spp : 0.f;
            } else {
                for (uint32_t k = 0; k < P.spp; k++) {
                    bool shadowed = true;
                    if (dist < maxd) {
                        f3 dir = sampleDisk(lt.radius, worldPos, L, seed);
                        Hit sh = trace<true, COUNT>(S, add_rn(worldPos, scale_rn(dir, 1e-2f)), dir, 0.001f,
                                                    __fadd_rn(dist, 1.0f), ls, P.status);
                        ls.shadow++;
                        shadowed = sh.id != HY_NO_HIT;
                    }
                    if (!shadowed) shadowFactor += 1.0f;
                }
            }
            shadowFactor /= spp;
        }
        if (I == 0.f) attenuation = 0.f;
        else {
            attenuation = maxd - dist;
            attenuation /= maxd;
            attenuation = fmaxf(attenuation, 0.f);
            attenuation = attenuation * attenuation;
        }
        f3 lc = mk(lt.color[0], lt.color[1], lt.color[2]);
        if (smode == 0) {
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
            Lo = Lo + ((NdotL > 0.f && I > 0.f) ? I * lc * attenuation * shadowFactor * metallic * albedo
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
            direction = radicand < 0.f ? reflect(rd, N) : refract(rd, refrN, eta);
            dirw = 1.f;
        }
    }
    f3 F = FresnelSchlick(NdotV, F0);
    f3 kD = (splat(1.0f) - F) * (1.0f - metallic);
    Payload p;
    p.color = Lo + kD * albedo * irradiance + ms.emissive;
    p.t = h.t;
    p.dir = direction;
    p.scattered = dirw;
    p.origin = worldPos;
    return p;
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

// raygen.rgen:20-81 for one pixel
template <bool COUNT>
__device__ __forceinline__ void pt_pixel(const SceneDev& S, const PtParams& T, uint32_t x, uint32_t y,
                                         LaneStats& ls) {
    const PassParams& P = T.P;
    const size_t pix = (size_t)y * P.W + x;
    uint32_t seed = tea(y * P.W + x, (uint32_t)T.frame);
    // NSAMPLES = 1 (helpers.glsl:6): the pixel centre, but r1 and r2 are drawn
    rnd(seed);
    rnd(seed);
    const float ux = __fdiv_rn(__fadd_rn((float)x, 0.5f), (float)P.W);
    const float uy = __fdiv_rn(__fadd_rn((float)y, 0.5f), (float)P.H);
    const float dx = __fsub_rn(__fmul_rn(ux, 2.0f), 1.0f), dy = __fsub_rn(__fmul_rn(uy, 2.0f), 1.0f);
    f3 origin = mat_vec3_rn(T.inv_view, 0.f, 0.f, 0.f, 1.f);
    const f3 tgt = mat_vec3_rn(T.inv_proj, dx, dy, 1.f, 1.f);
    const f3 tn = normalize_rn(tgt);
    f3 direction = mat_vec3_rn(T.inv_view, tn.x, tn.y, tn.z, 0.f);
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
    f3 fc = rayColor;
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

}  // namespace

cudaError_t pathtrace_occupancy(bool count, int* blocks_per_sm) {
    return count ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_pathtrace<true>, 128, 0)
                 : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k_pathtrace<false>, 128, 0);
}

cudaError_t launch_pathtrace(bool count, const SceneDev& S, const PtParams& T, int grid, cudaStream_t s) {
    if (count) k_pathtrace<true><<<grid, 128, 0, s>>>(S, T);
    else k_pathtrace<false><<<grid, 128, 0, s>>>(S, T);
    return cudaGetLastError();
}

}  // namespace hy
