// The hybrid pass on sm_103a.
//
// Kernels of the three reference programs:
//   k_shadow_stream<ACCUM=false>  shadowRaygen.rgen:28-93 -> raw per-light shadow
//                                 images, as tile streams (hy_stream_kernel.cuh,
//                                 instantiated in hy_stream_{raw,accum,two}.cu; the
//                                 default schedule)
//   k_shadow_stream<ACCUM=true>   the same rays folded straight into the history
//                                 with blur.comp's running mean (frame > 0), so the
//                                 raw images never touch memory in the steady state
//   k_shadow / k_shadow_group / k_shadow_pool
//                                 the same rays on other schedules (one lane per
//                                 pixel, lane groups per pixel-light, a ray pool)
//   k_accumulate                  blur.comp:35-81 for the reset frame (frame <= 0),
//                                 whose 3x3 clamp needs the whole raw image first
//   k_pixels<MODE_SHADE>          hybridRaygen.rgen:27-186 + hybridHit.rchit +
//                                 miss.rmiss, reading the accumulated images
//   k_shadow_batch_stream, k_shadow_batch, k_pixels_batch
//                                 the same over (view, tile) units of a batch
//   k_trace, k_gbuffer            ray queries; the primary-ray G-buffer producer
//
// Work distribution: persistent warps pull 8x4 pixel tiles from a global
// queue (one atomicAdd per `chunk` tiles) until it is drained; grids are
// sized to the resident-block capacity of the GPU.
#include <cuda_runtime.h>

#include "hy_device.cuh"
#include "hy_pass.h"
#include "hy_shade.cuh"
#include "hy_stream.cuh"

namespace hy {

template <int MODE, bool COUNT, int LV = 0>
__device__ __forceinline__ void do_pixel(const SceneDev& S, const PassParams& P, uint32_t x, uint32_t y,
                                         LaneStats& ls) {
    const size_t pix = (size_t)y * P.W + x;
    const size_t plane = (size_t)P.W * P.H;
    const float4 g0 = fetch_texel(P.plane[0], P.fmt[0], pix);
    const float4 g1 = fetch_texel(P.plane[1], P.fmt[1], pix);
    const f3 position = mk(g0.x, g0.y, g0.z);
    const f3 normal = mk(__fsub_rn(__fmul_rn(g1.x, 2.0f), 1.0f), __fsub_rn(__fmul_rn(g1.y, 2.0f), 1.0f),
                         __fsub_rn(__fmul_rn(g1.z, 2.0f), 1.0f));
    const int mi = mat_index(g0.w, S.num_mats);
    const int smode = mi >= 0 ? (int)S.mats[mi].smr[0] : 0;
    const float ior = mi >= 0 ? S.mats[mi].diffuse[3] : 1.f;
    const f3 N = normalize_rn(normal);
    uint32_t seed_h = tea(y * P.W + x, P.frame_u);
    const bool background = g0.w == 0.f && g1.w == 0.f;
    const float4 g2 = fetch_texel(P.plane[2], P.fmt[2], pix);
    const f3 albedo = pow3(mk(g2.x, g2.y, g2.z), 2.2f);
    if (background) {
        // hybridRaygen.rgen:182-183 overwrites everything computed before with albedo
        if (P.out_f) reinterpret_cast<float4*>(P.out_f)[pix] = make_float4(albedo.x, albedo.y, albedo.z, 1.f);
        if (P.out_8)
            reinterpret_cast<uchar4*>(P.out_8)[pix] =
                make_uchar4(quant8(albedo.z), quant8(albedo.y), quant8(albedo.x), 255);
        return;
    }

    // shading state (hybridRaygen.rgen:35-72)
    const float4 g4 = fetch_texel(P.plane[4], P.fmt[4], pix);
    const float4 g5 = fetch_texel(P.plane[5], P.fmt[5], pix);
    const f3 emissive = mk(g5.x, g5.y, g5.z);
    const float roughness = g4.y, metallic = g4.z;
    const f3 F0 = mix3(splat(0.04f), albedo, metallic);
    const f3 V = normalize(P.cam_pos - position);
    const float NdotV = clampf(dot(N, V), 0.f, 1.f);
    const f3 irradiance = irradiance_at(S, N);
    f3 origin = mk(0.f, 0.f, 0.f), direction = mk(0.f, 0.f, 0.f);
    f3 rayColor = mk(0.f, 0.f, 0.f);
    float attenuation = 1.0f;

    for (uint32_t i = 0; i < P.num_lights; i++) {
        const HyLight lt = S.lights[i];
        const LightGeo lg = light_geo(lt, position, N);
        const size_t li = i * plane + pix;
        // the accumulated shadow image (or the raw one without the denoise pass)
        const float sfac = accum_load(P.accum_fmt, (P.flags & HY_FLAG_NO_ACCUM) ? P.shadow : P.hist, li);
        // hybridRaygen.rgen:73-149
        const float I = lg.isDir ? 1.0f : (lt.color[3] / (lg.dist * lg.dist));
        const f3 L = lg.L;
        const float NdotL = lg.NdotL;
        if (NdotL > 0.f) {
            if (I == 0.f) attenuation = 0.f;
            else {
                attenuation = lg.maxd - lg.dist;
                attenuation /= lg.maxd;
                attenuation = fmaxf(attenuation, 0.f);
                attenuation = lg.isDir ? 0.3f : (attenuation * attenuation);
            }
        }
        const f3 lc = mk(lt.color[0], lt.color[1], lt.color[2]);
        if (smode == 0) {
            f3 radiance = lc * I * attenuation * sfac;
            f3 H = normalize(V + L);
            float D = DistributionGGX(N, H, roughness);
            float G = GeometrySmith(N, V, L, roughness);
            f3 F = FresnelSchlick(fmaxf(dot(H, V), 0.f), F0);
            f3 kD = (splat(1.0f) - F) * (1.0f - metallic);
            f3 numerator = D * G * F;
            float denominator = 4.0f * NdotV * NdotL;
            f3 specular = numerator / fmaxf(denominator, 0.001f);
            rayColor = rayColor + (kD * albedo / PI + specular) * radiance * NdotL;
        }
        if (smode == 3) {
            direction = reflect(normalize(-V), N);
            origin = position;
            rayColor = rayColor + ((NdotL > 0.f && I > 0.f) ? lc * I * attenuation * sfac * albedo * metallic
                                                            : irradiance * albedo * metallic);
        }
        if (smode == 4) {
            origin = position;
            float cosAlpha = dot(N, V);
            f3 Iv = -V;
            float NdotI = dot(N, Iv);
            f3 refrN = NdotI > 0.f ? -N : N;
            float eta = NdotI > 0.f ? 1.0f / ior : ior;
            float radicand = 1.0f + powf(eta, 2.0f) * (cosAlpha * cosAlpha - 1.0f);
            direction = radicand < 0.f ? reflect(Iv, N) : refract(Iv, refrN, eta);
            rayColor = rayColor + ((I > 0.f) ? I * lc * attenuation * albedo * metallic : irradiance * albedo * metallic);
        }
    }
    // HY_FLAG_GGX_REFLECTION: the mirror texel's first bounce sampled from its
    // GGX lobe with the texel's own RNG stream
    if ((P.flags & HY_FLAG_GGX_REFLECTION) && smode == 3 && P.max_bounces > 0) {
        const float u1 = rnd(seed_h), u2 = rnd(seed_h);
        direction = ggx_reflect(N, V, roughness, u1, u2);
    }
    // hybridRaygen.rgen:151-170
    for (uint32_t depth = 0; depth < P.max_bounces; depth++) {
        if (smode == 0) break;
        f3 ro = origin + direction * 1e-2f;
        Hit h = trace<false, COUNT, LV>(S, ro, direction, 0.001f, 1000.0f, ls, P.status);
        ls.refl++;
        f3 pc, pdir = direction, porg = origin;
        float pt, pw = 0.f;
        if (h.id == HY_NO_HIT) {
            pc = miss_color(S, direction);
            pt = -1.f;
        } else {
            Payload p = closest_hit<COUNT, false, LV>(S, P, h, ro, direction, seed_h, ls);
            pc = p.color; pt = p.t; pdir = p.dir; pw = p.scattered; porg = p.origin;
        }
        rayColor = rayColor * pc;
        if (pt < 0.f || !(pw > 0.f)) break;
        origin = porg;
        direction = pdir;
    }
    const f3 F = FresnelSchlick(NdotV, F0);
    const f3 kD = (splat(1.0f) - F) * (1.0f - metallic);
    const f3 fc = rayColor + (kD * albedo * irradiance + emissive);  // finalColor += ambient + emissive
    if (P.out_f) reinterpret_cast<float4*>(P.out_f)[pix] = make_float4(fc.x, fc.y, fc.z, 1.f);
    if (P.out_8) reinterpret_cast<uchar4*>(P.out_8)[pix] = make_uchar4(quant8(fc.z), quant8(fc.y), quant8(fc.x), 255);
}

// ---------------------------------------------------------------------------------
// shadowRaygen.rgen:28-93 as a persistent state machine.
//
// Each lane owns one pixel and walks its rays (lights in order, samples in
// order, the RNG advancing exactly as the per-pixel loop would) one BVH node
// per iteration; a lane whose ray ends starts the next one in the same
// iteration, and a lane whose pixel is done takes the next pixel of the
// warp's pool (8x4 tiles pulled from the global queue).  Warps therefore stay
// converged on node visits instead of waiting for each ray's slowest lane.
// ACCUM: fold each light's factor into the history with blur.comp's running
// mean (frame > 0) instead of writing the raw image.
// ---------------------------------------------------------------------------------
template <bool COUNT, bool ACCUM, int MINB, bool TWO = false>
__global__ void __launch_bounds__(128, MINB) k_shadow(const SceneDev S, const PassParams P) {
    LaneStats ls;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const size_t plane = (size_t)P.W * P.H;
    const bool reference = P.rng_mode == HY_RNG_REFERENCE;
    uint2 stk[kStackMax];
    ShadowLane s;
    Trav t;
    RayPre r;
    bool has_px = false, live = false, queue_empty = false;
    uint32_t pool_cur = 0, pool_end = 0;
    uint32_t nn = 0, nt = 0;
    for (;;) {
        // ---- give idle lanes a pixel from the warp's pool ----
        uint32_t need = __ballot_sync(0xffffffffu, !has_px);
        while (need && !queue_empty) {
            if (pool_cur == pool_end) {
                uint32_t t0 = 0;
                if (lane == 0) t0 = atomicAdd(P.queue, P.chunk);
                t0 = __shfl_sync(0xffffffffu, t0, 0);
                if (t0 >= P.ntiles) { queue_empty = true; break; }
                pool_cur = t0 * 32;
                pool_end = min(t0 + P.chunk, P.ntiles) * 32;
            }
            const uint32_t take = min((uint32_t)__popc(need), pool_end - pool_cur);
            const uint32_t rank = __popc(need & lt_mask);
            if (!has_px && rank < take) {
                const uint32_t slot = pool_cur + rank, tile = slot >> 5, l = slot & 31;
                const uint32_t x = (tile % P.tiles_x) * 8 + (l & 7), y = (tile / P.tiles_x) * 4 + (l >> 3);
                if (x < P.W && y < P.H) {
                    has_px = true;
                    s.pix = y * P.W + x;
                    const float4 g0 = fetch_texel(P.plane[0], P.fmt[0], s.pix);
                    const float4 g1 = fetch_texel(P.plane[1], P.fmt[1], s.pix);
                    s.position = mk(g0.x, g0.y, g0.z);
                    s.N = normalize_rn(mk(__fsub_rn(__fmul_rn(g1.x, 2.0f), 1.0f), __fsub_rn(__fmul_rn(g1.y, 2.0f), 1.0f),
                                          __fsub_rn(__fmul_rn(g1.z, 2.0f), 1.0f)));
                    const int mi = mat_index(g0.w, S.num_mats);
                    s.smode = mi >= 0 ? (int)S.mats[mi].smr[0] : 0;
                    s.seed = tea(s.pix, P.frame_u);
                    s.light = 0;
                    s.setup = true;
                    s.in_blur = x < P.blur_w && y < P.blur_h;
                }
            }
            pool_cur += take;
            need = __ballot_sync(0xffffffffu, !has_px);
        }
        if (queue_empty && __ballot_sync(0xffffffffu, has_px) == 0) break;

        // ---- a lane without a ray starts its pixel's next one ----
        if (has_px && !live) {
            for (;;) {
                if (s.setup) {
                    if (s.light >= P.num_lights) { has_px = false; break; }
                    const HyLight lt = S.lights[s.light];
                    const LightGeo lg = light_geo(lt, s.position, s.N);
                    s.L = lg.L;
                    s.dist = lg.dist;
                    s.radius = lt.radius;
                    s.k = 0;
                    s.sf = 0.f;
                    float v = -1.f;
                    if (s.smode == 4) v = 1.0f;                       // glass: fully lit, no rays
                    else if (!(lg.NdotL > 0.f)) v = 0.0f;             // facing away
                    else if (!(lg.dist < lg.maxd)) v = 1.0f;          // out of range / directional: all lit
                    if (v >= 0.f) {
                        shadow_finalize<ACCUM>(P, s, plane, v);
                        s.light++;
                        continue;
                    }
                    s.nrays = reference ? 1u : P.spp;
                    s.setup = false;
                }
                if (s.k < s.nrays) {
                    uint32_t sd = s.seed;
                    const f3 dir = reference ? sampleDisk(s.radius, s.position, s.L, sd)
                                             : sampleDisk(s.radius, s.position, s.L, s.seed);
                    r = ray_pre(add_rn(s.position, scale_rn(dir, 1e-1f)), dir);
                    trav_init(t, r, __fadd_rn(s.dist, 1.0f));
                    s.k++;
                    live = true;
                    ls.shadow++;
                    break;
                }
                // every sample of this light is in: REFERENCE traced the one shared ray
                shadow_finalize<ACCUM>(P, s, plane, reference ? s.sf : __fdiv_rn(s.sf, (float)P.spp));
                s.light++;
                s.setup = true;
            }
        }

        // ---- up to P.inner node visits ----
        if (live) {
            for (uint32_t it = 0, ni = max(P.inner, 1u); it < ni; it++) {
                if (trav_step<true, COUNT, TWO>(S, r, 0.001f, t, stk, nn, nt, P.status)) {
                    live = false;
                    if (t.h.id == HY_NO_HIT) s.sf = __fadd_rn(s.sf, 1.0f);
                    break;
                }
            }
        }
    }
    if (COUNT) { ls.nodes += nn; ls.tris += nt; }
    flush_stats(ls, P.stats);
}

// ---------------------------------------------------------------------------------
// DECORRELATED shadow rays, sample-parallel: a group of G lanes (G = spp
// rounded up to a power of two, at most 32) traces the samples of one
// pixel-light together.  The samples share their origin and fall in the
// light's small cone, so the group walks nearly the same nodes: its node
// loads coalesce into one request and its lanes stay converged.  Sample n of
// a pixel starts from the pixel's TEA seed advanced 2n LCG steps (LCG
// jump-ahead), which is exactly the state the sequential per-pixel loop
// reaches, so the rays equal those of k_shadow.
// ---------------------------------------------------------------------------------

template <bool COUNT, bool ACCUM, int MINB, bool TWO = false>
__global__ void __launch_bounds__(128, MINB) k_shadow_group(const SceneDev S, const PassParams P) {
    LaneStats ls;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t G = P.group;                  // power of two, 2..32
    const uint32_t g = lane & (G - 1), base = lane & ~(G - 1);
    const uint32_t gmask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << base;
    const uint32_t lt_mask = (1u << lane) - 1u;
    const size_t plane = (size_t)P.W * P.H;
    const uint32_t spp = P.spp;
    uint2 stk[kStackMax];
    ShadowLane s;
    Trav t;
    RayPre r;
    bool has_px = false, live = false, queue_empty = false;
    uint32_t pool_cur = 0, pool_end = 0, rays_before = 0, seed0 = 0;
    uint32_t nn = 0, nt = 0;
    for (;;) {
        // ---- idle groups take the next pixel of the warp's pool ----
        uint32_t need = __ballot_sync(0xffffffffu, g == 0 && !has_px);
        while (need && !queue_empty) {
            if (pool_cur == pool_end) {
                uint32_t t0 = 0;
                if (lane == 0) t0 = atomicAdd(P.queue, P.chunk);
                t0 = __shfl_sync(0xffffffffu, t0, 0);
                if (t0 >= P.ntiles) { queue_empty = true; break; }
                pool_cur = t0 * 32;
                pool_end = min(t0 + P.chunk, P.ntiles) * 32;
            }
            const uint32_t take = min((uint32_t)__popc(need), pool_end - pool_cur);
            const uint32_t rank = __popc(need & lt_mask);
            const uint32_t my_slot = (g == 0 && !has_px && rank < take) ? pool_cur + rank : 0xffffffffu;
            const uint32_t slot = __shfl_sync(0xffffffffu, my_slot, base);
            if (slot != 0xffffffffu) {
                const uint32_t tile = slot >> 5, l = slot & 31;
                const uint32_t x = (tile % P.tiles_x) * 8 + (l & 7), y = (tile / P.tiles_x) * 4 + (l >> 3);
                if (x < P.W && y < P.H) {
                    has_px = true;
                    s.pix = y * P.W + x;
                    const float4 g0 = fetch_texel(P.plane[0], P.fmt[0], s.pix);
                    const float4 g1 = fetch_texel(P.plane[1], P.fmt[1], s.pix);
                    s.position = mk(g0.x, g0.y, g0.z);
                    s.N = normalize_rn(mk(__fsub_rn(__fmul_rn(g1.x, 2.0f), 1.0f), __fsub_rn(__fmul_rn(g1.y, 2.0f), 1.0f),
                                          __fsub_rn(__fmul_rn(g1.z, 2.0f), 1.0f)));
                    const int mi = mat_index(g0.w, S.num_mats);
                    s.smode = mi >= 0 ? (int)S.mats[mi].smr[0] : 0;
                    seed0 = tea(s.pix, P.frame_u);
                    rays_before = 0;
                    s.light = 0;
                    s.setup = true;
                    s.in_blur = x < P.blur_w && y < P.blur_h;
                }
            }
            pool_cur += take;
            need = __ballot_sync(0xffffffffu, g == 0 && !has_px);
        }
        if (queue_empty && __ballot_sync(0xffffffffu, has_px) == 0) break;

        // ---- light set-up (group-uniform) ----
        if (has_px && s.setup) {
            for (;;) {
                if (s.light >= P.num_lights) { has_px = false; break; }
                const HyLight lt = S.lights[s.light];
                const LightGeo lg = light_geo(lt, s.position, s.N);
                float v = -1.f;
                if (s.smode == 4) v = 1.0f;
                else if (!(lg.NdotL > 0.f)) v = 0.0f;
                else if (!(lg.dist < lg.maxd)) v = 1.0f;
                if (v >= 0.f) {
                    if (g == 0) shadow_finalize<ACCUM>(P, s, plane, v);
                    s.light++;
                    continue;
                }
                s.L = lg.L;
                s.dist = lg.dist;
                s.radius = lt.radius;
                s.k = g;
                s.sf = 0.f;
                s.setup = false;
                break;
            }
        }
        // ---- start this lane's next sample of the current light ----
        if (has_px && !s.setup && !live && s.k < spp) {
            uint32_t sd = lcg_jump(seed0, 2u * (rays_before + s.k));
            const f3 dir = sampleDisk(s.radius, s.position, s.L, sd);
            r = ray_pre(add_rn(s.position, scale_rn(dir, 1e-1f)), dir);
            trav_init(t, r, __fadd_rn(s.dist, 1.0f));
            s.k += G;
            live = true;
            ls.shadow++;
        }
        // ---- up to P.inner node visits ----
        if (live) {
            for (uint32_t it = 0, ni = max(P.inner, 1u); it < ni; it++) {
                if (trav_step<true, COUNT, TWO>(S, r, 0.001f, t, stk, nn, nt, P.status)) {
                    live = false;
                    if (t.h.id == HY_NO_HIT) s.sf = __fadd_rn(s.sf, 1.0f);
                    break;
                }
            }
        }
        // ---- a group whose samples are all in folds them into the light's factor ----
        const uint32_t busy = __ballot_sync(0xffffffffu, has_px && !s.setup && (live || s.k < spp));
        if (has_px && !s.setup && (busy & gmask) == 0) {
            const uint32_t unocc = __reduce_add_sync(gmask, (uint32_t)s.sf);
            if (g == 0) shadow_finalize<ACCUM>(P, s, plane, __fdiv_rn((float)unocc, (float)spp));
            rays_before += spp;
            s.light++;
            s.setup = true;
        }
    }
    if (COUNT) { ls.nodes += nn; ls.tris += nt; }
    flush_stats(ls, P.stats);
}

template <int MODE, bool COUNT, int MINB = 1, int LV = 0>
__global__ void __launch_bounds__(128, MINB) k_pixels(const SceneDev S, const PassParams P) {
    LaneStats ls;
    const uint32_t lane = threadIdx.x & 31;
    uint32_t* queue = P.queue;
    for (;;) {
        uint32_t t0 = 0;
        if (lane == 0) t0 = atomicAdd(queue, P.chunk);
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        if (t0 >= P.ntiles) break;
        uint32_t t1 = min(t0 + P.chunk, P.ntiles);
        for (uint32_t t = t0; t < t1; t++) {
            uint32_t tx = t % P.tiles_x, ty = t / P.tiles_x;
            uint32_t x = tx * 8 + (lane & 7), y = ty * 4 + (lane >> 3);
            if (x < P.W && y < P.H) do_pixel<MODE, COUNT, LV>(S, P, x, y, ls);
        }
    }
    flush_stats(ls, P.stats);
}

// postFragment.frag:9-20: rgb = pow(max(rgb, 0.001), 1/2.2) per pixel of the final
// image (a full-screen quad sampling it NEAREST at texel centres), alpha kept
__global__ void __launch_bounds__(256) k_post(const uint8_t* __restrict__ in8, const float4* __restrict__ inf,
                                              uint32_t n, uchar4* __restrict__ out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 c;
    if (in8) {
        const uchar4 q = reinterpret_cast<const uchar4*>(in8)[i];  // B, G, R, A bytes
        c = make_float4(__fdiv_rn((float)q.z, 255.f), __fdiv_rn((float)q.y, 255.f), __fdiv_rn((float)q.x, 255.f),
                        __fdiv_rn((float)q.w, 255.f));
    } else {
        c = inf[i];
    }
    const float gamma = 1.0f / 2.2f;
    const float r = powf(fmaxf(c.x, 0.001f), gamma), g = powf(fmaxf(c.y, 0.001f), gamma),
                b = powf(fmaxf(c.z, 0.001f), gamma);
    out[i] = make_uchar4(quant8(b), quant8(g), quant8(r), quant8(c.w));
}

cudaError_t launch_post(const uint8_t* in8, const float* inf, uint32_t n, uint8_t* out, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_post<<<(n + 255) / 256, 256, 0, s>>>(in8, reinterpret_cast<const float4*>(inf), n,
                                            reinterpret_cast<uchar4*>(out));
    return cudaGetLastError();
}

// blur.comp:35-81, reset-frame branch and running mean, one texel per thread
__global__ void k_accumulate(const AccumParams A) {
    uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= A.blur_w || y >= A.blur_h) return;
    const size_t plane = (size_t)A.W * A.H, pix = (size_t)y * A.W + x;
    float rx = 0.f;
    if (A.frame <= 0) {
        float4 mo = fetch_texel(A.motion, A.motion_fmt, pix);
        rx = __fsub_rn(__fmul_rn(mo.x, 2.0f), 1.0f);
    }
    for (uint32_t l = 0; l < A.num_lights; l++) {
        const size_t o = l * plane;
        const float center = accum_load(A.fmt, A.shadow, o + pix);
        float out;
        if (A.frame > 0) {
            const float old = accum_load(A.fmt, A.hist, o + pix);
            const float a = __fdiv_rn(1.0f, __fadd_rn((float)A.frame, 1.0f));
            out = __fadd_rn(__fmul_rn(old, __fsub_rn(1.0f, a)), __fmul_rn(center, a));
        } else {
            // blur.comp:53: the y term reuses the x motion (vec2(float, vec2) constructor)
            const float lx = __fadd_rn((float)x, __fmul_rn(rx, (float)A.W));
            const float ly = __fadd_rn((float)y, __fmul_rn(rx, (float)A.H));
            float mn = center, mx = center;
            for (int dy = -1; dy <= 1; dy++)
                for (int dx = -1; dx <= 1; dx++) {
                    if (dx == 0 && dy == 0) continue;
                    int xx = (int)x + dx, yy = (int)y + dy;
                    float c = 0.f;
                    if (xx >= 0 && yy >= 0 && xx < (int)A.W && yy < (int)A.H)
                        c = accum_load(A.fmt, A.shadow, o + (size_t)yy * A.W + xx);
                    mn = fminf(mn, c);
                    mx = fmaxf(mx, c);
                }
            float old = 0.f;
            if (lx > -2147483648.f && lx < 2147483647.f && ly > -2147483648.f && ly < 2147483647.f) {
                int ix = (int)lx, iy = (int)ly;
                if (ix >= 0 && iy >= 0 && ix < (int)A.W && iy < (int)A.H)
                    old = accum_load(A.fmt, A.hist_prev, o + (size_t)iy * A.W + ix);
            }
            old = fmaxf(mn, old);
            old = fminf(mx, old);
            out = __fadd_rn(__fmul_rn(old, __fsub_rn(1.0f, 0.4f)), __fmul_rn(center, 0.4f));
        }
        accum_store(A.fmt, A.hist, o + pix, out);
    }
}

// generic ray queries (32 B ray in, 16 B hit out)
template <bool ANY, bool COUNT>
__global__ void __launch_bounds__(128) k_trace(const SceneDev S, const HyRay* __restrict__ rays, uint32_t n,
                                               HyHit* __restrict__ hits, unsigned long long* stats, uint32_t* status) {
    LaneStats ls;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i - threadIdx.x < n; i += gridDim.x * blockDim.x) {
        if (i < n) {
            HyRay r = rays[i];
            Hit h = trace<ANY, COUNT>(S, mk(r.org[0], r.org[1], r.org[2]), mk(r.dir[0], r.dir[1], r.dir[2]), r.tmin,
                                      r.tmax, ls, status);
            ls.shadow++;
            HyHit o;
            o.t = h.id == HY_NO_HIT ? 0.f : h.t;
            o.tri_id = h.id;
            o.b1 = h.id == HY_NO_HIT ? 0.f : h.b1;
            o.b2 = h.id == HY_NO_HIT ? 0.f : h.b2;
            hits[i] = o;
        }
    }
    flush_stats(ls, stats);
}

// primary-ray G-buffer (raygen.rgen:29-40 camera, geometry_shader.frag:54-76 encoding)
__device__ __forceinline__ f3 mat_vec3(const float* m, float x, float y, float z, float w) {
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

__global__ void __launch_bounds__(128) k_gbuffer(const SceneDev S, const GbufParams G) {
    uint32_t x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= G.W || y >= G.H) return;
    size_t i = (size_t)y * G.W + x;
    float ux = __fdiv_rn(__fadd_rn((float)x, 0.5f), (float)G.W), uy = __fdiv_rn(__fadd_rn((float)y, 0.5f), (float)G.H);
    float dx = __fsub_rn(__fmul_rn(ux, 2.0f), 1.0f), dy = __fsub_rn(__fmul_rn(uy, 2.0f), 1.0f);
    f3 org = mat_vec3(G.inv_view, 0.f, 0.f, 0.f, 1.f);
    f3 tgt = mat_vec3(G.inv_proj, dx, dy, 1.f, 1.f);
    f3 tn = normalize_rn(tgt);
    f3 dir = mat_vec3(G.inv_view, tn.x, tn.y, tn.z, 0.f);
    f3 o = add_rn(org, scale_rn(dir, 1e-2f));
    LaneStats ls;
    Hit h = trace<false, false>(S, o, dir, 0.001f, 10000.0f, ls, G.status);
    float4* p0 = (float4*)G.planes[0]; float4* p1 = (float4*)G.planes[1]; float4* p2 = (float4*)G.planes[2];
    float2* p3 = (float2*)G.planes[3]; float4* p4 = (float4*)G.planes[4]; float4* p5 = (float4*)G.planes[5];
    if (h.id == HY_NO_HIT) {
        float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        p0[i] = z; p1[i] = z; p2[i] = z; p3[i] = make_float2(0.f, 0.f); p4[i] = z; p5[i] = z;
        return;
    }
    HitAttr a = hit_attributes(S, h);
    const HyMaterial m = S.mats[S.prims[a.prim].material_id];
    f3 wp = add_rn(o, scale_rn(dir, h.t));
    p0[i] = make_float4(wp.x, wp.y, wp.z, m.smr[3]);
    p1[i] = make_float4(__fadd_rn(__fmul_rn(a.N.x, 0.5f), 0.5f), __fadd_rn(__fmul_rn(a.N.y, 0.5f), 0.5f),
                        __fadd_rn(__fmul_rn(a.N.z, 0.5f), 0.5f), 1.f);
    // geometry_shader.frag:56-59: textures, a diffuse texture modulated by the vertex colour
    f3 alb = mk(m.diffuse[0], m.diffuse[1], m.diffuse[2]), emis = mk(0.f, 0.f, 0.f), rm = mk(0.f, m.smr[2], m.smr[1]);
    if (has_textures(m)) {
        float u, v;
        f3 col;
        hit_uv_color(S, h, u, v, col);
        const MatSample ms = material_at(S, m, u, v);
        alb = m.textures[0] > -1.f ? mk(__fmul_rn(ms.albedo.x, col.x), __fmul_rn(ms.albedo.y, col.y),
                                        __fmul_rn(ms.albedo.z, col.z))
                                   : ms.albedo;
        emis = ms.emissive;
        rm = ms.rm;
    }
    p2[i] = make_float4(alb.x, alb.y, alb.z, 1.f);
    p3[i] = make_float2(0.5f, 0.5f);
    p4[i] = make_float4(rm.x, rm.y, rm.z, 1.f);
    p5[i] = make_float4(emis.x, emis.y, emis.z, 1.f);
}

// ---------------------------------------------------------------------------------
// Batches: many views of several scenes in one persistent launch.  The global
// queue hands out (view, 8x4 tile) units; a warp finishes its tile before it
// takes the next one, so lane-group size (from the view's spp), scene and
// G-buffer stay uniform across the warp while different warps work on
// different views.  REFERENCE views run with one lane per pixel (their
// samples are one ray), DECORRELATED views with spp lanes per pixel-light.
// ---------------------------------------------------------------------------------
template <bool COUNT, int MINB>
__global__ void __launch_bounds__(128, MINB) k_shadow_batch(const BatchParams B) {
    __shared__ uint32_t s_begin[kMaxBatchViews + 1];
    for (uint32_t i = threadIdx.x; i <= B.nviews; i += blockDim.x)
        s_begin[i] = i < B.nviews ? B.views[i].tile_begin : B.total_tiles;
    __syncthreads();
    LaneStats ls;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    uint2 stk[kStackMax];
    ShadowLane s;
    Trav t;
    RayPre r;
    bool has_px = false, live = false;
    uint32_t rays_before = 0, seed0 = 0, nn = 0, nt = 0;
    // warp-uniform: the current unit and its view's parameters
    uint32_t slot_cur = 0, slot_end = 0, chunk_cur = 0, chunk_end = 0;
    uint32_t G = 1, g = 0, base = lane, gmask = 1u << lane, spp = 1, nrays = 1;
    uint32_t cur_view = 0xffffffffu, pending = 0xffffffffu;
    bool reference = true, accum = false, queue_empty = false;
    size_t plane = 0;
    const PassParams* P = B.views;
    const SceneDev* S = B.scenes;
    for (;;) {
        // ---- the next unit once the current tile is handed out and every lane is
        //      idle: a warp's lanes stay on one 8x4 tile (coherent rays), and group
        //      size and G-buffer may change with the view.  (Letting a warp run
        //      into its next tile early measured 4 % slower: with one tile per
        //      pull that tile lies far away in the image.) ----
        if (slot_cur == slot_end && __ballot_sync(0xffffffffu, has_px) == 0) {
            if (pending == 0xffffffffu && !queue_empty) {
                if (chunk_cur == chunk_end) {
                    uint32_t t0 = 0;
                    if (lane == 0) t0 = atomicAdd(B.queue, B.chunk);
                    t0 = __shfl_sync(0xffffffffu, t0, 0);
                    if (t0 >= B.total_tiles) queue_empty = true;
                    else { chunk_cur = t0; chunk_end = min(t0 + B.chunk, B.total_tiles); }
                }
                if (!queue_empty) pending = chunk_cur++;
            }
            const bool idle = __ballot_sync(0xffffffffu, has_px) == 0;
            if (pending == 0xffffffffu) {
                if (idle) break;  // queue drained, every lane done
            } else {
                const uint32_t v = view_of_tile(s_begin, B.nviews, pending);
                if (v != cur_view && idle) {
                    cur_view = v;
                    P = B.views + v;
                    S = B.scenes + P->scene;
                    reference = P->rng_mode == HY_RNG_REFERENCE;
                    spp = P->spp;
                    nrays = reference ? 1u : spp;
                    G = P->group;
                    g = lane & (G - 1);
                    base = lane & ~(G - 1);
                    gmask = (G == 32 ? 0xffffffffu : ((1u << G) - 1u)) << base;
                    accum = !(P->flags & HY_FLAG_NO_ACCUM) && P->accum_frame > 0;
                    plane = (size_t)P->W * P->H;
                }
                if (v == cur_view) {
                    slot_cur = (pending - P->tile_begin) * 32;
                    slot_end = slot_cur + 32;
                    pending = 0xffffffffu;
                }
            }
        }
        // ---- idle groups take the tile's next pixel ----
        uint32_t need = __ballot_sync(0xffffffffu, g == 0 && !has_px);
        while (need && slot_cur < slot_end) {
            const uint32_t take = min((uint32_t)__popc(need), slot_end - slot_cur);
            const uint32_t rank = __popc(need & lt_mask);
            const uint32_t my_slot = (g == 0 && !has_px && rank < take) ? slot_cur + rank : 0xffffffffu;
            const uint32_t slot = __shfl_sync(0xffffffffu, my_slot, base);
            if (slot != 0xffffffffu) {
                const uint32_t tl = slot >> 5, l = slot & 31;
                const uint32_t x = (tl % P->tiles_x) * 8 + (l & 7), y = (tl / P->tiles_x) * 4 + (l >> 3);
                if (x < P->W && y < P->H) {
                    has_px = true;
                    s.pix = y * P->W + x;
                    const float4 g0 = fetch_texel(P->plane[0], P->fmt[0], s.pix);
                    const float4 g1 = fetch_texel(P->plane[1], P->fmt[1], s.pix);
                    s.position = mk(g0.x, g0.y, g0.z);
                    s.N = normalize_rn(mk(__fsub_rn(__fmul_rn(g1.x, 2.0f), 1.0f), __fsub_rn(__fmul_rn(g1.y, 2.0f), 1.0f),
                                          __fsub_rn(__fmul_rn(g1.z, 2.0f), 1.0f)));
                    const int mi = mat_index(g0.w, S->num_mats);
                    s.smode = mi >= 0 ? (int)S->mats[mi].smr[0] : 0;
                    seed0 = tea(s.pix, P->frame_u);
                    rays_before = 0;
                    s.light = 0;
                    s.setup = true;
                    s.in_blur = x < P->blur_w && y < P->blur_h;
                }
            }
            slot_cur += take;
            need = __ballot_sync(0xffffffffu, g == 0 && !has_px);
        }
        // ---- light set-up (group-uniform) ----
        if (has_px && s.setup) {
            for (;;) {
                if (s.light >= P->num_lights) { has_px = false; break; }
                const HyLight lt = S->lights[s.light];
                const LightGeo lg = light_geo(lt, s.position, s.N);
                float v = -1.f;
                if (s.smode == 4) v = 1.0f;
                else if (!(lg.NdotL > 0.f)) v = 0.0f;
                else if (!(lg.dist < lg.maxd)) v = 1.0f;
                if (v >= 0.f) {
                    if (g == 0) finalize_rt(*P, accum, s, plane, v);
                    s.light++;
                    continue;
                }
                s.L = lg.L;
                s.dist = lg.dist;
                s.radius = lt.radius;
                s.k = g;
                s.sf = 0.f;
                s.setup = false;
                break;
            }
        }
        // ---- this lane's next sample ----
        if (has_px && !s.setup && !live && s.k < nrays) {
            uint32_t sd = reference ? seed0 : lcg_jump(seed0, 2u * (rays_before + s.k));
            const f3 dir = sampleDisk(s.radius, s.position, s.L, sd);
            r = ray_pre(add_rn(s.position, scale_rn(dir, 1e-1f)), dir);
            trav_init(t, r, __fadd_rn(s.dist, 1.0f));
            s.k += G;
            live = true;
            ls.shadow++;
        }
        // ---- up to P->inner node visits ----
        if (live) {
            for (uint32_t it = 0, ni = max(P->inner, 1u); it < ni; it++) {
                if (trav_step<true, COUNT>(*S, r, 0.001f, t, stk, nn, nt, P->status)) {
                    live = false;
                    if (t.h.id == HY_NO_HIT) s.sf = __fadd_rn(s.sf, 1.0f);
                    break;
                }
            }
        }
        // ---- groups whose samples are all in fold them into the light's factor ----
        const uint32_t busy = __ballot_sync(0xffffffffu, has_px && !s.setup && (live || s.k < nrays));
        if (has_px && !s.setup && (busy & gmask) == 0) {
            const uint32_t unocc = __reduce_add_sync(gmask, (uint32_t)s.sf);
            const float v = reference ? (float)unocc : __fdiv_rn((float)unocc, (float)spp);
            if (g == 0) finalize_rt(*P, accum, s, plane, v);
            rays_before += spp;
            s.light++;
            s.setup = true;
        }
    }
    if (COUNT) { ls.nodes += nn; ls.tris += nt; }
    flush_stats(ls, B.stats);
}

template <bool COUNT>
__global__ void __launch_bounds__(128, 8) k_pixels_batch(const BatchParams B);

// ---------------------------------------------------------------------------------
// DECORRELATED shadow rays as a per-warp ray pool.
//
// The warp expands its pixels, in order, into pixel-light entries (at most
// kPoolEntries in flight, in shared memory) and each iteration hands every
// idle lane the next sample of the oldest entry that still has samples to
// start, opening entries as needed.  A lane whose ray ends takes new work in
// the next iteration, whatever pixel-light it belongs to, so no lane waits for
// the slowest sample of its group; the samples of one entry still start
// together on adjacent lanes (nearly the same node path).  Unoccluded samples
// are counted with shared-memory atomics and the lane that ends an entry's
// last sample writes the light's factor.  Same rays, seeds and sums as
// k_shadow_group: the unoccluded count is an integer, so the result does not
// depend on the order the samples end in.
// ---------------------------------------------------------------------------------
constexpr int kPoolEntries = 8;
struct PoolEntry {
    float px, py, pz, Lx, Ly, Lz, dist, radius;
    uint32_t pix, light, seed0, rays_before;
    uint32_t issued;   // samples started (written by the issuing step only)
    uint32_t in_blur;
    int pending;       // started and not finished (shared atomics)
    uint32_t unocc;    // unoccluded samples (shared atomics)
};

template <bool ACCUM>
__device__ __forceinline__ void pool_finalize(const PassParams& P, uint32_t pix, uint32_t light, bool in_blur,
                                              size_t plane, float v) {
    ShadowLane s;
    s.pix = pix;
    s.light = light;
    s.in_blur = in_blur;
    shadow_finalize<ACCUM>(P, s, plane, v);
}

template <bool COUNT, bool ACCUM, int MINB>
__global__ void __launch_bounds__(128, MINB) k_shadow_pool(const SceneDev S, const PassParams P) {
    __shared__ PoolEntry s_pool[4][kPoolEntries];
    __shared__ uint32_t s_freed[4];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t lt_mask = (1u << lane) - 1u;
    PoolEntry* E = s_pool[warp];
    if (lane == 0) s_freed[warp] = 0;
    const size_t plane = (size_t)P.W * P.H;
    const uint32_t spp = P.spp;
    LaneStats ls;
    uint2 stk[kStackMax];
    Trav t;
    RayPre r;
    bool live = false;
    uint32_t my_e = 0, nn = 0, nt = 0;
    // warp-uniform state: entries in flight, the entry still starting samples,
    // the pixel being expanded into entries, the warp's tile pool
    uint32_t used = 0, head_issued = 0;
    int head = -1;
    bool cur_valid = false, cur_in_blur = false, queue_empty = false;
    uint32_t cur_pix = 0, cur_light = 0, cur_rays = 0, cur_seed0 = 0, pool_cur = 0, pool_end = 0;
    int cur_smode = 0;
    f3 cur_pos = mk(0.f, 0.f, 0.f), cur_N = cur_pos;
    for (;;) {
        __syncwarp();
        used &= ~s_freed[warp];
        __syncwarp();
        if (lane == 0) s_freed[warp] = 0;
        // ---- hand the idle lanes their next samples ----
        uint32_t idle = __ballot_sync(0xffffffffu, !live);
        while (idle) {
            if (head < 0) {
                // open the next pixel-light that needs rays
                bool opened = false;
                while (!opened) {
                    if (!cur_valid) {
                        if (pool_cur == pool_end) {
                            if (queue_empty) break;
                            uint32_t t0 = 0;
                            if (lane == 0) t0 = atomicAdd(P.queue, P.chunk);
                            t0 = __shfl_sync(0xffffffffu, t0, 0);
                            if (t0 >= P.ntiles) { queue_empty = true; break; }
                            pool_cur = t0 * 32;
                            pool_end = min(t0 + P.chunk, P.ntiles) * 32;
                        }
                        const uint32_t slot = pool_cur++;
                        const uint32_t tile = slot >> 5, l = slot & 31;
                        const uint32_t x = (tile % P.tiles_x) * 8 + (l & 7), y = (tile / P.tiles_x) * 4 + (l >> 3);
                        if (x < P.W && y < P.H) {
                            cur_valid = true;
                            cur_pix = y * P.W + x;
                            const float4 g0 = fetch_texel(P.plane[0], P.fmt[0], cur_pix);
                            const float4 g1 = fetch_texel(P.plane[1], P.fmt[1], cur_pix);
                            cur_pos = mk(g0.x, g0.y, g0.z);
                            cur_N = normalize_rn(mk(__fsub_rn(__fmul_rn(g1.x, 2.0f), 1.0f),
                                                    __fsub_rn(__fmul_rn(g1.y, 2.0f), 1.0f),
                                                    __fsub_rn(__fmul_rn(g1.z, 2.0f), 1.0f)));
                            const int mi = mat_index(g0.w, S.num_mats);
                            cur_smode = mi >= 0 ? (int)S.mats[mi].smr[0] : 0;
                            cur_seed0 = tea(cur_pix, P.frame_u);
                            cur_light = 0;
                            cur_rays = 0;
                            cur_in_blur = x < P.blur_w && y < P.blur_h;
                        }
                        continue;
                    }
                    if (cur_light >= P.num_lights) { cur_valid = false; continue; }
                    if (__popc(used) == kPoolEntries) break;  // wait for an entry to retire
                    const HyLight lt = S.lights[cur_light];
                    const LightGeo lg = light_geo(lt, cur_pos, cur_N);
                    float v = -1.f;
                    if (cur_smode == 4) v = 1.0f;
                    else if (!(lg.NdotL > 0.f)) v = 0.0f;
                    else if (!(lg.dist < lg.maxd)) v = 1.0f;
                    if (v >= 0.f) {  // no rays: the factor is known
                        if (lane == 0) pool_finalize<ACCUM>(P, cur_pix, cur_light, cur_in_blur, plane, v);
                        cur_light++;
                        continue;
                    }
                    const int e = __ffs(~used & ((1u << kPoolEntries) - 1u)) - 1;
                    if (lane == 0) {
                        PoolEntry& q = E[e];
                        q.px = cur_pos.x; q.py = cur_pos.y; q.pz = cur_pos.z;
                        q.Lx = lg.L.x; q.Ly = lg.L.y; q.Lz = lg.L.z;
                        q.dist = lg.dist;
                        q.radius = lt.radius;
                        q.pix = cur_pix;
                        q.light = cur_light;
                        q.seed0 = cur_seed0;
                        q.rays_before = cur_rays;
                        q.issued = 0;
                        q.in_blur = cur_in_blur ? 1u : 0u;
                        q.pending = 0;
                        q.unocc = 0;
                    }
                    used |= 1u << e;
                    head = e;
                    head_issued = 0;
                    cur_rays += spp;
                    cur_light++;
                    opened = true;
                }
                if (!opened) break;
                __syncwarp();
            }
            const uint32_t n = min((uint32_t)__popc(idle), spp - head_issued);
            const uint32_t rank = __popc(idle & lt_mask);
            if (!live && rank < n) {
                const PoolEntry& q = E[head];
                const uint32_t k = head_issued + rank;
                uint32_t sd = lcg_jump(q.seed0, 2u * (q.rays_before + k));
                const f3 pos = mk(q.px, q.py, q.pz);
                const f3 dir = sampleDisk(q.radius, pos, mk(q.Lx, q.Ly, q.Lz), sd);
                r = ray_pre(add_rn(pos, scale_rn(dir, 1e-1f)), dir);
                trav_init(t, r, __fadd_rn(q.dist, 1.0f));
                my_e = (uint32_t)head;
                live = true;
                ls.shadow++;
            }
            __syncwarp();
            head_issued += n;
            if (lane == 0) {
                E[head].issued = head_issued;
                E[head].pending += (int)n;
            }
            if (head_issued == spp) head = -1;
            idle = __ballot_sync(0xffffffffu, !live);
        }
        if (queue_empty && !cur_valid && used == 0 && __ballot_sync(0xffffffffu, live) == 0) break;
        __syncwarp();
        // ---- one node visit ----
        if (live) {
            if (trav_step<true, COUNT>(S, r, 0.001f, t, stk, nn, nt, P.status)) {
                live = false;
                PoolEntry& q = E[my_e];
                if (t.h.id == HY_NO_HIT) atomicAdd(&q.unocc, 1u);
                __threadfence_block();
                if (atomicSub(&q.pending, 1) == 1 && q.issued == spp) {
                    __threadfence_block();
                    const uint32_t unocc = atomicAdd(&q.unocc, 0u);
                    pool_finalize<ACCUM>(P, q.pix, q.light, q.in_blur != 0, plane,
                                         __fdiv_rn((float)unocc, (float)spp));
                    atomicOr(&s_freed[warp], 1u << my_e);
                }
            }
        }
    }
    if (COUNT) { ls.nodes += nn; ls.tris += nt; }
    flush_stats(ls, P.stats);
}

template <bool COUNT>
__global__ void __launch_bounds__(128, 8) k_pixels_batch(const BatchParams B) {
    __shared__ uint32_t s_begin[kMaxBatchViews + 1];
    for (uint32_t i = threadIdx.x; i <= B.nviews; i += blockDim.x)
        s_begin[i] = i < B.nviews ? B.views[i].tile_begin : B.total_tiles;
    __syncthreads();
    LaneStats ls;
    const uint32_t lane = threadIdx.x & 31;
    for (;;) {
        uint32_t t0 = 0;
        if (lane == 0) t0 = atomicAdd(B.queue, B.chunk);
        t0 = __shfl_sync(0xffffffffu, t0, 0);
        if (t0 >= B.total_tiles) break;
        const uint32_t t1 = min(t0 + B.chunk, B.total_tiles);
        for (uint32_t tile = t0; tile < t1; tile++) {
            const PassParams& P = B.views[view_of_tile(s_begin, B.nviews, tile)];
            const uint32_t tl = tile - P.tile_begin;
            const uint32_t x = (tl % P.tiles_x) * 8 + (lane & 7), y = (tl / P.tiles_x) * 4 + (lane >> 3);
            if (x < P.W && y < P.H) do_pixel<MODE_SHADE, COUNT>(B.scenes[P.scene], P, x, y, ls);
        }
    }
    flush_stats(ls, B.stats);
}

// ---------------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------------
template <bool GROUP, bool ACCUM, int MINB>
static void* shadow_kernel(bool count) {
    if (GROUP) return count ? (void*)k_shadow_group<true, ACCUM, MINB> : (void*)k_shadow_group<false, ACCUM, MINB>;
    return count ? (void*)k_shadow<true, ACCUM, MINB> : (void*)k_shadow<false, ACCUM, MINB>;
}
template <bool GROUP, bool ACCUM>
static void* shadow_kernel(bool count, int minb) {
    if (minb >= 8) return shadow_kernel<GROUP, ACCUM, 8>(count);
    if (GROUP && minb == 7) return shadow_kernel<GROUP, ACCUM, 7>(count);
    if (GROUP && minb == 6) return shadow_kernel<GROUP, ACCUM, 6>(count);
    return shadow_kernel<GROUP, ACCUM, 5>(count);
}
// minb: resident blocks per SM the shadow kernel is compiled for (register cap)
template <bool ACCUM, int MINB>
static void* pool_kernel(bool count) {
    return count ? (void*)k_shadow_pool<true, ACCUM, MINB> : (void*)k_shadow_pool<false, ACCUM, MINB>;
}

// two-level structure: the lane-group shadow kernel (register cap of 5 or 6
// resident blocks), the pixel-parallel one (5) and the shade kernel; nullptr
// for the ray pool
template <bool ACCUM>
static void* shadow_kernel_two(bool count, int minb) {
    if (minb >= 6)
        return count ? (void*)k_shadow_group<true, ACCUM, 6, true> : (void*)k_shadow_group<false, ACCUM, 6, true>;
    return count ? (void*)k_shadow_group<true, ACCUM, 5, true> : (void*)k_shadow_group<false, ACCUM, 5, true>;
}

// the shade kernel (hybridRaygen + hybridHit): resident blocks it is compiled for;
// at 8 (the default) one variant per structure level, each holding one copy of
// the walk, else one variant for either level
template <int MINB>
static void* shade_kernel_m(bool count) {
    return count ? (void*)k_pixels<MODE_SHADE, true, MINB> : (void*)k_pixels<MODE_SHADE, false, MINB>;
}
static void* shade_kernel(bool count, int minb, bool two) {
    if (minb >= 8) {
        if (two) return count ? (void*)k_pixels<MODE_SHADE, true, 8, 2> : (void*)k_pixels<MODE_SHADE, false, 8, 2>;
        return count ? (void*)k_pixels<MODE_SHADE, true, 8, 1> : (void*)k_pixels<MODE_SHADE, false, 8, 1>;
    }
    if (minb >= 6) return shade_kernel_m<6>(count);
    if (minb == 5) return shade_kernel_m<5>(count);
    if (minb == 4) return shade_kernel_m<4>(count);
    return shade_kernel_m<1>(count);
}

static void* pixel_kernel(int mode, bool count, int minb, bool two, bool short_stack = false, int shade_minb = 0) {
    if (mode == MODE_SHADOW_S || mode == MODE_SHADOW_ACCUM_S) {
        const bool accum = mode == MODE_SHADOW_ACCUM_S;
        if (two) return stream_kernel_two(accum, count);
        return accum ? stream_kernel_accum(count, minb, short_stack) : stream_kernel_raw(count, minb, short_stack);
    }
    if (two) {
        switch (mode) {
            case MODE_SHADOW_G: return shadow_kernel_two<false>(count, minb);
            case MODE_SHADOW_ACCUM_G: return shadow_kernel_two<true>(count, minb);
            case MODE_SHADOW:
                return count ? (void*)k_shadow<true, false, 5, true> : (void*)k_shadow<false, false, 5, true>;
            case MODE_SHADOW_ACCUM:
                return count ? (void*)k_shadow<true, true, 5, true> : (void*)k_shadow<false, true, 5, true>;
            case MODE_SHADE: return shade_kernel(count, shade_minb, true);
            default: return nullptr;
        }
    }
    switch (mode) {
        case MODE_SHADOW: return shadow_kernel<false, false>(count, minb);
        case MODE_SHADOW_ACCUM: return shadow_kernel<false, true>(count, minb);
        case MODE_SHADOW_G: return shadow_kernel<true, false>(count, minb);
        case MODE_SHADOW_ACCUM_G: return shadow_kernel<true, true>(count, minb);
        case MODE_SHADOW_P: return minb >= 8 ? pool_kernel<false, 8>(count) : pool_kernel<false, 5>(count);
        case MODE_SHADOW_ACCUM_P: return minb >= 8 ? pool_kernel<true, 8>(count) : pool_kernel<true, 5>(count);
        default: return shade_kernel(count, shade_minb, false);
    }
}

cudaError_t launch_pixels(int mode, bool count, int minb, const SceneDev& S, const PassParams& P, int grid, int block,
                          cudaStream_t s) {
    void* args[] = {(void*)&S, (void*)&P};
    void* k = pixel_kernel(mode, count, minb, S.two_level != 0, P.short_stack != 0, (int)P.shade_minb);
    if (!k) return cudaErrorNotSupported;
    return cudaLaunchKernel(k, dim3(grid), dim3(block), args, 0, s);
}

cudaError_t pixel_occupancy(int mode, bool count, int minb, bool two, bool short_stack, int shade_minb, int block,
                            int* blocks_per_sm) {
    void* k = pixel_kernel(mode, count, minb, two, short_stack, shade_minb);
    if (!k) return cudaErrorNotSupported;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k, block, 0);
}

cudaError_t launch_accumulate(const AccumParams& A, cudaStream_t s) {
    dim3 b(16, 16), g((A.blur_w + 15) / 16, (A.blur_h + 15) / 16);
    if (g.x == 0 || g.y == 0) return cudaSuccess;
    k_accumulate<<<g, b, 0, s>>>(A);
    return cudaGetLastError();
}

cudaError_t launch_trace(const SceneDev& S, const HyRay* rays, uint32_t n, bool any, bool count, HyHit* hits,
                         unsigned long long* stats, uint32_t* status, int grid, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    if (any) {
        if (count) k_trace<true, true><<<grid, 128, 0, s>>>(S, rays, n, hits, stats, status);
        else k_trace<true, false><<<grid, 128, 0, s>>>(S, rays, n, hits, stats, status);
    } else {
        if (count) k_trace<false, true><<<grid, 128, 0, s>>>(S, rays, n, hits, stats, status);
        else k_trace<false, false><<<grid, 128, 0, s>>>(S, rays, n, hits, stats, status);
    }
    return cudaGetLastError();
}

cudaError_t launch_gbuffer(const SceneDev& S, const GbufParams& G, cudaStream_t s) {
    dim3 b(16, 8), g((G.W + 15) / 16, (G.H + 7) / 8);
    k_gbuffer<<<g, b, 0, s>>>(S, G);
    return cudaGetLastError();
}

// the tile-stream batch kernel of a launch shape (hy_batch_*.cu); nullptr where none is compiled
static void* batch_stream_kernel(bool count, int minb, int block, int shortd, bool two) {
    switch (block) {
        case 64: return batch_stream_kernel_64(count, minb, shortd, two);
        case 128: return batch_stream_kernel_128(count, minb, shortd, two);
        case 256: return batch_stream_kernel_256(count, minb, shortd, two);
        default: return nullptr;
    }
}

static void* batch_kernel(bool shade, bool count, int minb, bool stream, bool two, int block, int shortd) {
    if (shade) return count ? (void*)k_pixels_batch<true> : (void*)k_pixels_batch<false>;
    if (stream) return batch_stream_kernel(count, minb, block, shortd, two);
    if (block != 128 || shortd != 0) return nullptr;
    if (minb >= 8) return count ? (void*)k_shadow_batch<true, 8> : (void*)k_shadow_batch<false, 8>;
    return count ? (void*)k_shadow_batch<true, 5> : (void*)k_shadow_batch<false, 5>;
}

// dynamic shared memory of a batch kernel: the shared part of the traversal stacks
static size_t batch_dyn_smem(bool shade, bool stream, int block, int shortd) {
    return (!shade && stream) ? (size_t)shortd * (size_t)block * sizeof(uint2) : 0;
}

cudaError_t launch_batch(bool shade, bool count, int minb, bool stream, bool two, int block, int shortd,
                         const BatchParams& B, int grid, cudaStream_t s) {
    void* k = batch_kernel(shade, count, minb, stream, two, shade ? 128 : block, shortd);
    if (!k) return cudaErrorNotSupported;
    const size_t dyn = batch_dyn_smem(shade, stream, block, shortd);
    if (dyn) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
        if (e != cudaSuccess) return e;
    }
    void* args[] = {(void*)&B};
    return cudaLaunchKernel(k, dim3(grid), dim3(shade ? 128 : block), args, dyn, s);
}

cudaError_t batch_occupancy(bool shade, bool count, int minb, bool stream, bool two, int block, int shortd,
                            int* blocks_per_sm) {
    void* k = batch_kernel(shade, count, minb, stream, two, shade ? 128 : block, shortd);
    if (!k) return cudaErrorNotSupported;
    const size_t dyn = batch_dyn_smem(shade, stream, block, shortd);
    if (dyn) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
        if (e != cudaSuccess) return e;
    }
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k, shade ? 128 : block, dyn);
}

}  // namespace hy
