// ORACLE — test infrastructure only (see orc_math.hpp).
//
// CPU restatement of the hybrid pass, one function per reference program:
//   gbuffer_primary  raygen.rgen:29-40 camera model + geometry_shader.frag:54-76 encoding
//   shadow_pass      shadowRaygen.rgen:28-93 (+ shadow.rmiss:6-9)
//   accumulate       blur.comp:35-81
//   shade            hybridRaygen.rgen:27-186, hybridHit.rchit:24-183, miss.rmiss:13-18
// Pixels are spread over std::thread workers by rows; each pixel's
// arithmetic is sequential and independent of the thread count.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <thread>

#include "orc_passes.hpp"

namespace orc {

static int g_threads = 0;
void set_threads(int n) { g_threads = n; }
int get_threads() {
    if (g_threads > 0) return g_threads;
    unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 1;
}

// ---- texel access --------------------------------------------------------------
static inline float half_to_float(uint16_t h) {
    uint32_t s = (uint32_t)(h >> 15) << 31, e = (h >> 10) & 0x1f, m = h & 0x3ff;
    uint32_t u;
    if (e == 0) {
        if (m == 0) u = s;
        else {  // subnormal
            int k = 0;
            while (!(m & 0x400)) { m <<= 1; k++; }
            m &= 0x3ff;
            u = s | ((uint32_t)(127 - 15 - k + 1) << 23) | (m << 13);
        }
    } else if (e == 31) u = s | 0x7f800000u | (m << 13);
    else u = s | ((e - 15 + 127) << 23) | (m << 13);
    return bitsf(u);
}

static inline uint32_t fmt_bytes(uint32_t f) {
    switch (f) {
        case HY_FMT_RGBA32F: return 16;
        case HY_FMT_RG32F: return 8;
        case HY_FMT_RGBA16F: return 8;
        case HY_FMT_RG16F: return 4;
        default: return 4;
    }
}

// NEAREST fetch at the pixel centre == texel (x, y) (the samplers of
// src/renderer.cpp:822 are NEAREST / CLAMP_TO_EDGE)
void fetch(const GBufHost& g, int p, uint32_t x, uint32_t y, float out[4]) {
    size_t i = (size_t)y * g.w + x;
    const uint8_t* base = (const uint8_t*)g.plane[p] + i * fmt_bytes(g.fmt[p]);
    out[0] = out[1] = out[2] = out[3] = 0.f;
    switch (g.fmt[p]) {
        case HY_FMT_RGBA32F: std::memcpy(out, base, 16); break;
        case HY_FMT_RG32F: std::memcpy(out, base, 8); break;
        case HY_FMT_RGBA16F:
        case HY_FMT_RG16F: {
            int nc = g.fmt[p] == HY_FMT_RGBA16F ? 4 : 2;
            for (int c = 0; c < nc; c++) {
                uint16_t h;
                std::memcpy(&h, base + 2 * c, 2);
                out[c] = half_to_float(h);
            }
            break;
        }
        case HY_FMT_RGBA8:
            for (int c = 0; c < 4; c++) out[c] = (float)base[c] / 255.0f;
            break;
    }
}

static inline uint8_t quant8(float v) {
    float c = std::fmin(std::fmax(v, 0.f), 1.f) * 255.0f;
    return (uint8_t)std::nearbyint(c);
}

float accum_load(uint32_t fmt, const void* buf, size_t i) {
    if (fmt == HY_ACCUM_U8) return (float)((const uint8_t*)buf)[i] / 255.0f;
    return ((const float*)buf)[i];
}
void accum_store(uint32_t fmt, void* buf, size_t i, float v) {
    if (fmt == HY_ACCUM_U8) ((uint8_t*)buf)[i] = quant8(v);
    else ((float*)buf)[i] = v;
}

// equirect NEAREST/REPEAT lookup of an RGBA8 environment map
static V3<float> env_lookup(const Env& e, float u, float v) {
    if (e.w == 0 || e.h == 0) return v3(0.f, 0.f, 0.f);
    if (!(u == u)) u = 0.f;
    if (!(v == v)) v = 0.f;
    float fx = std::floor(u * (float)e.w), fy = std::floor(v * (float)e.h);
    fx = std::fmin(std::fmax(fx, -1e9f), 1e9f);
    fy = std::fmin(std::fmax(fy, -1e9f), 1e9f);
    long ix = (long)fx % (long)e.w, iy = (long)fy % (long)e.h;
    if (ix < 0) ix += e.w;
    if (iy < 0) iy += e.h;
    const uint8_t* p = &e.px[((size_t)iy * e.w + (size_t)ix) * 4];
    return v3((float)p[0] / 255.0f, (float)p[1] / 255.0f, (float)p[2] / 255.0f);
}

V3<float> tex_lookup(const Scene& s, float id, float u, float v) {
    const int i = (int)id;
    if (i < 0 || (size_t)i >= s.tex.size()) return v3(0.f, 0.f, 0.f);
    return env_lookup(s.tex[i], u, v);
}

// a material's inputs at a surface point: hybridHit.rchit:62-66 / closesthit.rchit:74-81
// (textures ids in mat.textures: x diffuse, z emissive, w metallic-roughness)
MatSample material_at(const Scene& s, const HyMaterial& m, float u, float v) {
    MatSample r;
    r.albedo = m.textures[0] > -1.f ? tex_lookup(s, m.textures[0], u, v) : v3(m.diffuse[0], m.diffuse[1], m.diffuse[2]);
    r.emissive = m.textures[2] > -1.f ? tex_lookup(s, m.textures[2], u, v) : v3(0.f, 0.f, 0.f);
    r.rm = m.textures[3] > -1.f ? tex_lookup(s, m.textures[3], u, v) : v3(0.f, m.smr[2], m.smr[1]);
    return r;
}

// hybridRaygen.rgen:59-60 / hybridHit.rchit:272-273
V3<float> irradiance_at(const Scene& s, V3<float> N) {
    const float PI = K<float>::PI;
    float u = 0.5f + std::atan2(N.x, N.z) / (2.0f * PI);
    float v = 0.5f - std::asin(N.y) / PI;
    return env_lookup(s.env[1], u, v);
}
// miss.rmiss:13-18
V3<float> miss_color(const Scene& s, V3<float> d) {
    const float PI = K<float>::PI_MISS;
    V3<float> dir = normalize(d);
    float u = 0.5f + std::atan2(dir.x, dir.z) / (2.0f * PI);
    float v = 0.5f - std::asin(dir.y) / PI;
    return pow3(env_lookup(s.env[0], u, v), 2.2f);
}

// int(materialIdx) of a G-buffer texel; -1 when it names no material
int mat_index(float f, size_t n) {
    if (!(f > -1.f && f < (float)n)) return -1;
    return (int)f;
}
static inline int material_mode(const Scene& s, float matIdx) {
    int mi = mat_index(matIdx, s.mats.size());
    return mi < 0 ? 0 : (int)s.mats[mi].smr[0];
}

// ---- G-buffer producer ---------------------------------------------------------------
static inline V3<float> mat_vec3(const float* m, float x, float y, float z, float w) {
    V3<float> r;
    for (int i = 0; i < 3; i++) {
        float a = m[0 * 4 + i] * x;
        a = a + m[1 * 4 + i] * y;
        a = a + m[2 * 4 + i] * z;
        a = a + m[3 * 4 + i] * w;
        (&r.x)[i] = a;
    }
    return r;
}

void primary_ray(const HyCamera& cam, uint32_t W, uint32_t H, uint32_t x, uint32_t y, float o[3], float d[3]) {
    float ux = ((float)x + 0.5f) / (float)W, uy = ((float)y + 0.5f) / (float)H;
    float dx = ux * 2.0f - 1.0f, dy = uy * 2.0f - 1.0f;
    V3<float> org = mat_vec3(cam.inv_view, 0.f, 0.f, 0.f, 1.f);
    V3<float> tgt = mat_vec3(cam.inv_proj, dx, dy, 1.f, 1.f);
    V3<float> tn = normalize(tgt);
    V3<float> dir = mat_vec3(cam.inv_view, tn.x, tn.y, tn.z, 0.f);
    V3<float> oo = org + dir * 1e-2f;
    o[0] = oo.x; o[1] = oo.y; o[2] = oo.z;
    d[0] = dir.x; d[1] = dir.y; d[2] = dir.z;
}

HitAttr hit_attributes(const Scene& s, const Hit& h) {
    uint32_t p = s.tri_prim[h.id];
    const HyPrimitive& pr = s.prims[p];
    uint32_t local = h.id - s.prim_tri0[p];
    float b0 = 1.0f - h.b1 - h.b2;
    V3<float> n = v3(0.f, 0.f, 0.f), col = v3(0.f, 0.f, 0.f);
    float u = 0.f, v = 0.f;
    float bw[3] = {b0, h.b1, h.b2};
    for (int k = 0; k < 3; k++) {
        const HyVertex& vx = s.verts[s.idx[pr.first_index + 3 * local + k] + pr.vertex_offset];
        n = n + v3(vx.normal[0], vx.normal[1], vx.normal[2]) * bw[k];
        u = u + vx.uv[0] * bw[k];
        v = v + vx.uv[1] * bw[k];
        col = col + v3(vx.color[0], vx.color[1], vx.color[2]) * bw[k];
    }
    const float* nm = &s.nrm[(size_t)pr.transform_id * 9];
    V3<float> tn;
    tn.x = nm[0] * n.x + nm[3] * n.y + nm[6] * n.z;
    tn.y = nm[1] * n.x + nm[4] * n.y + nm[7] * n.z;
    tn.z = nm[2] * n.x + nm[5] * n.y + nm[8] * n.z;
    return HitAttr{normalize(tn), u, v, p, col};
}

void gbuffer_primary(const Scene& s, const HyCamera& cam, uint32_t W, uint32_t H, float* planes[6], int mode) {
    parallel_rows(H, [&](uint32_t y, int) {
        for (uint32_t x = 0; x < W; x++) {
            size_t i = (size_t)y * W + x;
            float o[3], d[3];
            primary_ray(cam, W, H, x, y, o, d);
            Hit h = trace(s, o, d, 0.001f, 10000.0f, false, mode, nullptr);
            float* p0 = planes[0] + i * 4; float* p1 = planes[1] + i * 4; float* p2 = planes[2] + i * 4;
            float* p3 = planes[3] + i * 2; float* p4 = planes[4] + i * 4; float* p5 = planes[5] + i * 4;
            if (h.id == HY_NO_HIT) {
                std::memset(p0, 0, 16); std::memset(p1, 0, 16); std::memset(p2, 0, 16);
                std::memset(p3, 0, 8); std::memset(p4, 0, 16); std::memset(p5, 0, 16);
                continue;
            }
            HitAttr a = hit_attributes(s, h);
            const HyMaterial& m = s.mats[s.prims[a.prim].material_id];
            V3<float> wp = v3(o[0], o[1], o[2]) + v3(d[0], d[1], d[2]) * h.t;
            p0[0] = wp.x; p0[1] = wp.y; p0[2] = wp.z; p0[3] = m.smr[3];
            p1[0] = a.N.x * 0.5f + 0.5f; p1[1] = a.N.y * 0.5f + 0.5f; p1[2] = a.N.z * 0.5f + 0.5f; p1[3] = 1.f;
            // geometry_shader.frag:56-59: a diffuse texture is modulated by the vertex colour
            const MatSample ms = material_at(s, m, a.u, a.v);
            const V3<float> alb = m.textures[0] > -1.f ? ms.albedo * a.color : ms.albedo;
            p2[0] = alb.x; p2[1] = alb.y; p2[2] = alb.z; p2[3] = 1.f;
            p3[0] = 0.5f; p3[1] = 0.5f;  // static camera: ndc - ndcPrev = 0
            p4[0] = ms.rm.x; p4[1] = ms.rm.y; p4[2] = ms.rm.z; p4[3] = 1.f;
            p5[0] = ms.emissive.x; p5[1] = ms.emissive.y; p5[2] = ms.emissive.z; p5[3] = 1.f;
        }
    });
}

// ---- shadow pass (shadowRaygen.rgen:28-93) -----------------------------------------
void shadow_pass(const Scene& s, const GBufHost& g, const HyCamera& cam, const HyPassConfig& cfg, uint32_t fmt,
                 void* shadow, int mode, PassStats* st) {
    const uint32_t W = g.w, H = g.h, NL = (uint32_t)s.lights.size();
    const size_t plane = (size_t)W * H;
    int nt = get_threads();
    std::vector<PassStats> loc(nt);
    parallel_rows(H, [&](uint32_t y, int tid) {
        PassStats& ls = loc[tid];
        for (uint32_t x = 0; x < W; x++) {
            size_t pix = (size_t)y * W + x;
            int frame = (int)cam.frame[0];
            uint32_t seed = tea(y * W + x, (uint32_t)frame);
            float g0[4], g1[4];
            fetch(g, 0, x, y, g0);
            fetch(g, 1, x, y, g1);
            V3<float> position = v3(g0[0], g0[1], g0[2]);
            V3<float> normal = v3(g1[0] * 2.0f - 1.0f, g1[1] * 2.0f - 1.0f, g1[2] * 2.0f - 1.0f);
            int smode = material_mode(s, g0[3]);
            V3<float> N = normalize(normal);
            if (smode == 4) {
                for (uint32_t i = 0; i < NL; i++) accum_store(fmt, shadow, i * plane + pix, 1.0f);
                continue;
            }
            for (uint32_t i = 0; i < NL; i++) {
                const HyLight& lt = s.lights[i];
                bool isDir = lt.pos[3] < 0.f;
                V3<float> L = isDir ? v3(lt.pos[0], lt.pos[1], lt.pos[2])
                                    : v3(lt.pos[0], lt.pos[1], lt.pos[2]) - position;
                float maxd = lt.pos[3];
                float dist = length(L);
                L = normalize(L);
                float NdotL = clampv(dot(N, L), 0.f, 1.f);
                float sf = 0.f;
                int spp = (int)cfg.shadow_spp;
                if (NdotL > 0.f) {
                    if (dist < maxd && cfg.rng_mode == HY_RNG_REFERENCE) {
                        // every sample is the same ray (by-value seed): trace it once
                        uint32_t sd = seed;
                        V3<float> dir = sampleDisk<float>(lt.radius, position, L, sd);
                        V3<float> o = position + dir * 1e-1f;
                        float oo[3] = {o.x, o.y, o.z}, dd[3] = {dir.x, dir.y, dir.z};
                        Hit h = trace(s, oo, dd, 0.001f, dist + 1.0f, true, mode, st ? &ls.cnt : nullptr);
                        ls.shadow_rays++;
                        sf = (h.id == HY_NO_HIT) ? (float)spp : 0.f;
                    } else {
                        for (int k = 0; k < spp; k++) {
                            bool shadowed;
                            if (dist < maxd) {
                                V3<float> dir = sampleDisk<float>(lt.radius, position, L, seed);
                                V3<float> o = position + dir * 1e-1f;
                                float oo[3] = {o.x, o.y, o.z}, dd[3] = {dir.x, dir.y, dir.z};
                                Hit h = trace(s, oo, dd, 0.001f, dist + 1.0f, true, mode, st ? &ls.cnt : nullptr);
                                ls.shadow_rays++;
                                shadowed = h.id != HY_NO_HIT;
                            } else {
                                shadowed = false;
                            }
                            if (!shadowed) sf += 1.f;
                        }
                    }
                    sf /= (float)spp;
                }
                accum_store(fmt, shadow, i * plane + pix, sf);
            }
        }
    });
    if (st) for (auto& l : loc) st->add(l);
}

// ---- accumulation (blur.comp:35-81) -----------------------------------------------
void accumulate(const GBufHost& g, const HyPassConfig& cfg, uint32_t fmt, const void* shadow, void* hist,
                uint32_t NL) {
    const uint32_t W = g.w, H = g.h;
    const size_t plane = (size_t)W * H;
    const size_t esz = fmt == HY_ACCUM_U8 ? 1 : 4;
    std::vector<uint8_t> prev((const uint8_t*)hist, (const uint8_t*)hist + plane * NL * esz);
    uint32_t XW = W, YH = H;
    if (!(cfg.flags & HY_FLAG_FULL_BLUR_DISPATCH)) { XW = (W / 16) * 16; YH = (H / 16) * 16; }
    int frame = cfg.accum_frame;
    parallel_rows(YH, [&](uint32_t y, int) {
        for (uint32_t x = 0; x < XW; x++) {
            size_t pix = (size_t)y * W + x;
            for (uint32_t l = 0; l < NL; l++) {
                const size_t o = l * plane;
                float out;
                if (frame > 0) {
                    float center = accum_load(fmt, shadow, o + pix);
                    float old = accum_load(fmt, prev.data(), o + pix);
                    float a = 1.0f / ((float)frame + 1.0f);
                    out = mixv(old, center, a);
                } else {
                    float mo[4];
                    fetch(g, 3, x, y, mo);
                    float rx = mo[0] * 2.0f - 1.0f;
                    // blur.comp:53: the y term reuses the x motion (vec2(float, vec2) constructor)
                    float lx = (float)x + rx * (float)W;
                    float ly = (float)y + rx * (float)H;
                    float center = accum_load(fmt, shadow, o + pix);
                    float mn = center, mx = center;
                    for (int dy = -1; dy <= 1; dy++)
                        for (int dx = -1; dx <= 1; dx++) {
                            if (dx == 0 && dy == 0) continue;
                            int xx = (int)x + dx, yy = (int)y + dy;
                            float c = 0.f;
                            if (xx >= 0 && yy >= 0 && xx < (int)W && yy < (int)H)
                                c = accum_load(fmt, shadow, o + (size_t)yy * W + xx);
                            mn = std::fmin(mn, c);
                            mx = std::fmax(mx, c);
                        }
                    int ix = (int)lx, iy = (int)ly;  // ivec2(): truncation toward zero
                    float old = 0.f;
                    if (lx > -2147483648.f && lx < 2147483647.f && ly > -2147483648.f && ly < 2147483647.f &&
                        ix >= 0 && iy >= 0 && ix < (int)W && iy < (int)H)
                        old = accum_load(fmt, prev.data(), o + (size_t)iy * W + ix);
                    old = std::fmax(mn, old);
                    old = std::fmin(mx, old);
                    out = mixv(old, center, 0.4f);
                }
                accum_store(fmt, hist, o + pix, out);
            }
        }
    });
}

// ---- hybrid shading (hybridRaygen.rgen, hybridHit.rchit, miss.rmiss) ----------------------
Payload closest_hit(const Scene& s, const Hit& h, V3<float> ro, V3<float> rd, uint32_t& seed,
                    const HyPassConfig& cfg, int mode, PassStats& ls, uint64_t* vis) {
    const float PI = K<float>::PI;
    HitAttr a = hit_attributes(s, h);
    V3<float> N = a.N;
    V3<float> V = normalize(-rd);
    float NdotV = clampv(dot(N, V), 0.f, 1.f);
    V3<float> worldPos = ro + rd * h.t;
    const HyMaterial& mat = s.mats[s.prims[a.prim].material_id];
    int smode = (int)mat.smr[0];
    const MatSample ms = material_at(s, mat, a.u, a.v);  // hybridHit.rchit:62-66
    V3<float> albedo = ms.albedo;
    V3<float> emissive = ms.emissive;
    float roughness = ms.rm.y, metallic = ms.rm.z;
    albedo = pow3(albedo, 2.2f);
    V3<float> F0 = mix3(splat(0.04f), albedo, metallic);
    V3<float> irradiance = irradiance_at(s, N);
    V3<float> direction = v3(1.f, 1.f, 1.f);
    float dirw = 0.f;
    V3<float> Lo = v3(0.f, 0.f, 0.f);
    float attenuation = 1.0f;
    if (vis) *vis = 0;
    for (size_t i = 0; i < s.lights.size(); i++) {
        const HyLight& lt = s.lights[i];
        bool isDir = lt.pos[3] < 0.f;
        V3<float> L = isDir ? v3(lt.pos[0], lt.pos[1], lt.pos[2]) : v3(lt.pos[0], lt.pos[1], lt.pos[2]) - worldPos;
        float maxd = lt.pos[3];
        float dist = length(L);
        L = normalize(L);
        float I = isDir ? 1.0f : (lt.color[3] / (dist * dist));
        V3<float> H = normalize(V + L);
        float NdotL = clampv(dot(N, L), 0.f, 1.f);
        float NdotH = clampv(dot(N, H), 0.f, 1.f);
        float shadowFactor = 1.0f;
        if (I == 0.f) attenuation = 0.f;
        else {
            attenuation = maxd - dist;
            attenuation /= maxd;
            attenuation = std::fmax(attenuation, 0.f);
            attenuation = isDir ? 0.3f : attenuation * attenuation;
        }
        V3<float> lc = v3(lt.color[0], lt.color[1], lt.color[2]);
        if (smode == 0) {
            if (NdotL > 0.f) {
                bool shadowed = true;
                if (dist < maxd) {
                    uint32_t sd = seed;
                    V3<float> dir = sampleDisk<float>(lt.radius, worldPos, L,
                                                      cfg.rng_mode == HY_RNG_REFERENCE ? sd : seed);
                    V3<float> o = worldPos + dir * 1e-2f;
                    float oo[3] = {o.x, o.y, o.z}, dd[3] = {dir.x, dir.y, dir.z};
                    Hit sh = trace(s, oo, dd, 0.001f, dist + 1.0f, true, mode, &ls.cnt);
                    ls.hit_shadow_rays++;
                    shadowed = sh.id != HY_NO_HIT;
                }
                if (!shadowed) {
                    shadowFactor += 1.0f;
                    if (vis && i < 64) *vis |= 1ull << i;
                }
            }
            V3<float> radiance = I * lc * attenuation * shadowFactor;
            V3<float> F = FresnelSchlick(NdotH, F0);
            float D = DistributionGGX(N, H, roughness);
            float G = GeometrySmith(N, V, L, roughness);
            V3<float> numerator = D * G * F;
            float denominator = std::fmax(4.0f * clampv(dot(N, V), 0.f, 1.f) * NdotL, 0.000001f);
            V3<float> specular = numerator / denominator;
            V3<float> kD = (splat(1.0f) - F) * (1.0f - metallic);
            Lo = Lo + (kD * albedo / PI + specular) * radiance * NdotL;
            direction = v3(1.f, 1.f, 1.f);
            dirw = 0.f;
        } else if (smode == 3) {
            V3<float> reflected = reflect(normalize(rd), N);
            bool sc = dot(reflected, N) > 0.f;
            Lo = Lo + ((NdotL > 0.f && I > 0.f) ? I * lc * attenuation * albedo * metallic
                                                : irradiance * albedo * metallic);
            direction = reflected;
            dirw = sc ? 1.f : 0.f;
        } else if (smode == 4) {
            float ior = mat.diffuse[3];
            float NdV = dot(N, normalize(rd));
            V3<float> refrN = NdV > 0.f ? -N : N;
            float eta = NdV > 0.f ? 1.0f / ior : ior;
            Lo = Lo + ((I > 0.f) ? I * lc * attenuation * albedo * metallic : irradiance * albedo * metallic);
            float radicand = 1.0f + std::pow(eta, 2.0f) * (NdV * NdV - 1.0f);
            direction = radicand < 0.f ? reflect(rd, N) : refract(normalize(rd), refrN, eta);
            dirw = 1.f;
        }
    }
    V3<float> F = FresnelSchlick(NdotV, F0);
    V3<float> kD = (splat(1.0f) - F) * (1.0f - metallic);
    V3<float> ambient = kD * albedo * irradiance;
    Payload p;
    p.color = Lo + ambient + emissive;
    p.t = h.t;
    p.dir = direction;
    p.scattered = dirw;
    p.origin = worldPos;
    return p;
}

void shade(const Scene& s, const GBufHost& g, const HyCamera& cam, const HyPassConfig& cfg, uint32_t fmt,
           const void* hist, float* out_rgba32f, uint8_t* out_bgra8, int mode, PassStats* st) {
    const uint32_t W = g.w, H = g.h, NL = (uint32_t)s.lights.size();
    const size_t plane = (size_t)W * H;
    const float PI = K<float>::PI;
    int nt = get_threads();
    std::vector<PassStats> loc(nt);
    parallel_rows(H, [&](uint32_t y, int tid) {
        PassStats& ls = loc[tid];
        for (uint32_t x = 0; x < W; x++) {
            size_t pix = (size_t)y * W + x;
            uint32_t frame = (uint32_t)(int)cam.frame[0];
            uint32_t seed = tea(y * W + x, frame);
            float g0[4], g1[4], g2[4], g4[4], g5[4];
            fetch(g, 0, x, y, g0); fetch(g, 1, x, y, g1); fetch(g, 2, x, y, g2);
            fetch(g, 4, x, y, g4); fetch(g, 5, x, y, g5);
            int mi = mat_index(g0[3], s.mats.size());
            bool mat_ok = mi >= 0;
            int smode = mat_ok ? (int)s.mats[mi].smr[0] : 0;
            float ior = mat_ok ? s.mats[mi].diffuse[3] : 1.f;
            V3<float> position = v3(g0[0], g0[1], g0[2]);
            V3<float> normal = v3(g1[0] * 2.0f - 1.0f, g1[1] * 2.0f - 1.0f, g1[2] * 2.0f - 1.0f);
            V3<float> albedo = pow3(v3(g2[0], g2[1], g2[2]), 2.2f);
            V3<float> emissive = v3(g5[0], g5[1], g5[2]);
            bool background = g0[3] == 0.f && g1[3] == 0.f;
            V3<float> fc;
            if (background) {
                fc = albedo;  // hybridRaygen.rgen:182-183 overwrites everything computed before
            } else {
                float roughness = g4[1], metallic = g4[2];
                V3<float> F0 = mix3(splat(0.04f), albedo, metallic);
                V3<float> camPos = mat_vec3(cam.inv_view, 0.f, 0.f, 0.f, 1.f);
                V3<float> V = normalize(camPos - position);
                V3<float> N = normalize(normal);
                float NdotV = clampv(dot(N, V), 0.f, 1.f);
                V3<float> irradiance = irradiance_at(s, N);
                V3<float> origin = v3(0.f, 0.f, 0.f), direction = v3(0.f, 0.f, 0.f);
                float attenuation = 1.0f;
                V3<float> rayColor = v3(0.f, 0.f, 0.f);
                for (uint32_t i = 0; i < NL; i++) {
                    const HyLight& lt = s.lights[i];
                    bool isDir = lt.pos[3] < 0.f;
                    V3<float> L = isDir ? v3(lt.pos[0], lt.pos[1], lt.pos[2])
                                        : v3(lt.pos[0], lt.pos[1], lt.pos[2]) - position;
                    float maxd = lt.pos[3];
                    float dist = length(L);
                    float I = isDir ? 1.0f : (lt.color[3] / (dist * dist));
                    L = normalize(L);
                    float NdotL = clampv(dot(N, L), 0.f, 1.f);
                    float shadowFactor = accum_load(fmt, hist, i * plane + pix);
                    if (NdotL > 0.f) {
                        if (I == 0.f) attenuation = 0.f;
                        else {
                            attenuation = maxd - dist;
                            attenuation /= maxd;
                            attenuation = std::fmax(attenuation, 0.f);
                            attenuation = isDir ? 0.3f : (attenuation * attenuation);
                        }
                    }
                    V3<float> lc = v3(lt.color[0], lt.color[1], lt.color[2]);
                    if (smode == 0) {
                        V3<float> radiance = lc * I * attenuation * shadowFactor;
                        V3<float> Hh = normalize(V + L);
                        float D = DistributionGGX(N, Hh, roughness);
                        float G = GeometrySmith(N, V, L, roughness);
                        V3<float> F = FresnelSchlick(std::fmax(dot(Hh, V), 0.f), F0);
                        V3<float> kD = splat(1.0f) - F;
                        kD = kD * (1.0f - metallic);
                        V3<float> numerator = D * G * F;
                        float denominator = 4.0f * NdotV * NdotL;
                        V3<float> specular = numerator / std::fmax(denominator, 0.001f);
                        rayColor = rayColor + (kD * albedo / PI + specular) * radiance * NdotL;
                    }
                    if (smode == 3) {
                        direction = reflect(normalize(-V), N);
                        origin = position;
                        rayColor = rayColor + ((NdotL > 0.f && I > 0.f)
                                                   ? lc * I * attenuation * shadowFactor * albedo * metallic
                                                   : irradiance * albedo * metallic);
                    }
                    if (smode == 4) {
                        origin = position;
                        float cosAlpha = dot(N, V);
                        V3<float> Iv = -V;
                        float NdotI = dot(N, Iv);
                        V3<float> refrN = NdotI > 0.f ? -N : N;
                        float eta = NdotI > 0.f ? 1.0f / ior : ior;
                        float radicand = 1.0f + std::pow(eta, 2.0f) * (cosAlpha * cosAlpha - 1.0f);
                        direction = radicand < 0.f ? reflect(Iv, N) : refract(Iv, refrN, eta);
                        rayColor = rayColor + ((I > 0.f) ? I * lc * attenuation * albedo * metallic
                                                         : irradiance * albedo * metallic);
                    }
                }
                // HY_FLAG_GGX_REFLECTION: the mirror texel's first bounce from its GGX lobe
                if ((cfg.flags & HY_FLAG_GGX_REFLECTION) && smode == 3 && cfg.max_bounces > 0) {
                    const float u1 = rnd(seed), u2 = rnd(seed);
                    direction = ggx_reflect<float>(N, V, roughness, u1, u2);
                }
                for (uint32_t depth = 0; depth < cfg.max_bounces; depth++) {
                    if (smode == 0) break;
                    V3<float> ro = origin + direction * 1e-2f;
                    float oo[3] = {ro.x, ro.y, ro.z}, dd[3] = {direction.x, direction.y, direction.z};
                    Hit h = trace(s, oo, dd, 0.001f, 1000.0f, false, mode, st ? &ls.cnt : nullptr);
                    ls.reflection_rays++;
                    V3<float> pc;
                    float pt, pw = 0.f;
                    V3<float> pdir = direction, porg = origin;
                    if (h.id == HY_NO_HIT) {
                        pc = miss_color(s, direction);
                        pt = -1.f;
                    } else {
                        Payload p = closest_hit(s, h, ro, direction, seed, cfg, mode, ls);
                        pc = p.color; pt = p.t; pdir = p.dir; pw = p.scattered; porg = p.origin;
                    }
                    rayColor = rayColor * pc;
                    if (pt < 0.f || !(pw > 0.f)) break;
                    origin = porg;
                    direction = pdir;
                }
                V3<float> F = FresnelSchlick(NdotV, F0);
                V3<float> kD = (splat(1.0f) - F) * (1.0f - metallic);
                V3<float> ambient = kD * albedo * irradiance;
                fc = rayColor + (ambient + emissive);  // finalColor += ambient + emissive (hybridRaygen.rgen:180)
            }
            if (out_rgba32f) {
                float* o = out_rgba32f + pix * 4;
                o[0] = fc.x; o[1] = fc.y; o[2] = fc.z; o[3] = 1.f;
            }
            if (out_bgra8) {
                uint8_t* o = out_bgra8 + pix * 4;
                o[0] = quant8(fc.z); o[1] = quant8(fc.y); o[2] = quant8(fc.x); o[3] = 255;
            }
        }
    });
    if (st) for (auto& l : loc) st->add(l);
}

// ---- post (postFragment.frag:9-20) ---------------------------------------------------
void post_resolve(uint32_t n, const uint8_t* in_bgra8, const float* in_rgba32f, uint8_t* out_bgra8) {
    const float gamma = 1.0f / 2.2f;
    for (size_t i = 0; i < n; i++) {
        float c[4];
        if (in_bgra8) {
            const uint8_t* q = in_bgra8 + i * 4;
            c[0] = (float)q[2] / 255.0f; c[1] = (float)q[1] / 255.0f; c[2] = (float)q[0] / 255.0f;
            c[3] = (float)q[3] / 255.0f;
        } else {
            for (int k = 0; k < 4; k++) c[k] = in_rgba32f[i * 4 + k];
        }
        float rgb[3];
        for (int k = 0; k < 3; k++) rgb[k] = std::pow(std::fmax(c[k], 0.001f), gamma);
        uint8_t* o = out_bgra8 + i * 4;
        o[0] = quant8(rgb[2]); o[1] = quant8(rgb[1]); o[2] = quant8(rgb[0]); o[3] = quant8(c[3]);
    }
}

// ---- path-traced mode (raygen.rgen:20-81, closesthit.rchit:26-186, miss.rmiss) ----------
static Payload closest_hit_pt(const Scene& s, const Hit& h, V3<float> ro, V3<float> rd, uint32_t& seed,
                              const HyPassConfig& cfg, int mode, PassStats& ls) {
    const float PI = K<float>::PI;
    HitAttr a = hit_attributes(s, h);
    V3<float> N = a.N;
    V3<float> V = normalize(-rd);
    float NdotV = clampv(dot(N, V), 0.f, 1.f);
    V3<float> worldPos = ro + rd * h.t;
    const HyMaterial& mat = s.mats[s.prims[a.prim].material_id];
    int smode = (int)mat.smr[0];
    const MatSample ms = material_at(s, mat, a.u, a.v);  // closesthit.rchit:74-81
    V3<float> albedo = pow3(ms.albedo, 2.2f);
    float roughness = ms.rm.y, metallic = ms.rm.z;
    V3<float> F0 = mix3(splat(0.04f), albedo, metallic);
    V3<float> irradiance = irradiance_at(s, N);
    V3<float> direction = v3(1.f, 1.f, 1.f);
    float dirw = 0.f;
    V3<float> Lo = v3(0.f, 0.f, 0.f);
    float attenuation = 1.0f;
    const int samples = (int)cfg.shadow_spp;
    for (size_t i = 0; i < s.lights.size(); i++) {
        const HyLight& lt = s.lights[i];
        bool isDir = lt.pos[3] < 0.f;
        V3<float> L = isDir ? v3(lt.pos[0], lt.pos[1], lt.pos[2]) : v3(lt.pos[0], lt.pos[1], lt.pos[2]) - worldPos;
        float maxd = lt.pos[3];
        float dist = length(L);
        L = normalize(L);
        float I = isDir ? 1.0f : (lt.color[3] / (dist * dist));
        V3<float> H = normalize(V + L);
        float NdotL = clampv(dot(N, L), 0.f, 1.f);
        float NdotH = clampv(dot(N, H), 0.f, 1.f);
        float shadowFactor = 0.f;
        // every shading model casts the shadow rays; sampleDisk's seed is by value,
        // so in REFERENCE mode all samples are one ray
        if (NdotL > 0.f) {
            if (dist < maxd && cfg.rng_mode == HY_RNG_REFERENCE) {
                uint32_t sd = seed;
                V3<float> dir = sampleDisk<float>(lt.radius, worldPos, L, sd);
                V3<float> o = worldPos + dir * 1e-2f;
                float oo[3] = {o.x, o.y, o.z}, dd[3] = {dir.x, dir.y, dir.z};
                Hit sh = trace(s, oo, dd, 0.001f, dist + 1.0f, true, mode, &ls.cnt);
                ls.shadow_rays++;
                shadowFactor = sh.id == HY_NO_HIT ? (float)samples : 0.f;
            } else {
                for (int k = 0; k < samples; k++) {
                    bool shadowed = true;
                    if (dist < maxd) {
                        V3<float> dir = sampleDisk<float>(lt.radius, worldPos, L, seed);
                        V3<float> o = worldPos + dir * 1e-2f;
                        float oo[3] = {o.x, o.y, o.z}, dd[3] = {dir.x, dir.y, dir.z};
                        Hit sh = trace(s, oo, dd, 0.001f, dist + 1.0f, true, mode, &ls.cnt);
                        ls.shadow_rays++;
                        shadowed = sh.id != HY_NO_HIT;
                    }
                    if (!shadowed) shadowFactor += 1.0f;
                }
            }
            shadowFactor /= (float)samples;
        }
        // closesthit.rchit:109-117: no directional special case here
        if (I == 0.f) attenuation = 0.f;
        else {
            attenuation = maxd - dist;
            attenuation /= maxd;
            attenuation = std::fmax(attenuation, 0.f);
            attenuation = attenuation * attenuation;
        }
        V3<float> lc = v3(lt.color[0], lt.color[1], lt.color[2]);
        if (smode == 0) {
            V3<float> radiance = I * lc * attenuation * shadowFactor;
            V3<float> F = FresnelSchlick(NdotH, F0);
            float D = DistributionGGX(N, H, roughness);
            float G = GeometrySmith(N, V, L, roughness);
            V3<float> numerator = D * G * F;
            float denominator = std::fmax(4.0f * clampv(dot(N, V), 0.f, 1.f) * NdotL, 0.000001f);
            V3<float> specular = numerator / denominator;
            V3<float> kD = (splat(1.0f) - F) * (1.0f - metallic);
            Lo = Lo + (kD * albedo / PI + specular) * radiance * NdotL;
            direction = v3(1.f, 1.f, 1.f);
            dirw = 0.f;
        } else if (smode == 3) {
            V3<float> reflected = reflect(normalize(rd), N);
            bool sc = dot(reflected, N) > 0.f;
            Lo = Lo + ((NdotL > 0.f && I > 0.f) ? I * lc * attenuation * shadowFactor * metallic * albedo
                                                : irradiance * albedo * metallic);
            direction = reflected;
            dirw = sc ? 1.f : 0.f;
        } else if (smode == 4) {
            float ior = mat.diffuse[3];
            float NdV = dot(N, normalize(rd));
            V3<float> refrN = NdV > 0.f ? -N : N;
            float eta = NdV > 0.f ? 1.0f / ior : ior;
            Lo = Lo + ((I > 0.f) ? I * lc * attenuation * albedo * metallic : irradiance * albedo * metallic);
            float radicand = 1.0f + std::pow(eta, 2.0f) * (NdV * NdV - 1.0f);
            direction = radicand < 0.f ? reflect(rd, N) : refract(rd, refrN, eta);
            dirw = 1.f;
        }
    }
    V3<float> F = FresnelSchlick(NdotV, F0);
    V3<float> kD = (splat(1.0f) - F) * (1.0f - metallic);
    Payload p;
    p.color = Lo + kD * albedo * irradiance + ms.emissive;
    p.t = h.t;
    p.dir = direction;
    p.scattered = dirw;
    p.origin = worldPos;
    return p;
}

void pathtrace(const Scene& s, const HyCamera& cam, uint32_t W, uint32_t H, const HyPassConfig& cfg,
               uint8_t* image_bgra8, float* out_rgba32f, int mode, PassStats* st) {
    int nt = get_threads();
    std::vector<PassStats> loc(nt);
    const int frame = (int)cam.frame[0];
    parallel_rows(H, [&](uint32_t y, int tid) {
        PassStats& ls = loc[tid];
        for (uint32_t x = 0; x < W; x++) {
            const size_t pix = (size_t)y * W + x;
            uint32_t seed = tea(y * W + x, (uint32_t)frame);
            // NSAMPLES = 1 (helpers.glsl:6): the offset is the pixel centre, r1/r2 are still drawn
            rnd(seed);
            rnd(seed);
            float o[3], d[3];
            primary_ray(cam, W, H, x, y, o, d);  // the camera ray of raygen.rgen:35-44
            V3<float> origin = mat_vec3(cam.inv_view, 0.f, 0.f, 0.f, 1.f);  // the loop adds the 1e-2 offset
            V3<float> direction = v3(d[0], d[1], d[2]);
            V3<float> rayColor = v3(1.f, 1.f, 1.f);
            for (uint32_t depth = 0; depth < cfg.max_bounces; depth++) {
                V3<float> ro = origin + direction * 1e-2f;
                float oo[3] = {ro.x, ro.y, ro.z}, dd[3] = {direction.x, direction.y, direction.z};
                Hit h = trace(s, oo, dd, 0.001f, 10000.0f, false, mode, &ls.cnt);
                ls.reflection_rays++;
                if (h.id == HY_NO_HIT) {
                    rayColor = rayColor * miss_color(s, direction);
                    break;
                }
                Payload p = closest_hit_pt(s, h, ro, direction, seed, cfg, mode, ls);
                rayColor = rayColor * p.color;
                if (!(p.scattered > 0.f)) break;
                origin = p.origin;
                direction = p.dir;
            }
            V3<float> fc = rayColor;  // finalColor / NSAMPLES with NSAMPLES = 1
            if (out_rgba32f) {
                float* q = out_rgba32f + pix * 4;
                q[0] = fc.x; q[1] = fc.y; q[2] = fc.z; q[3] = 1.f;
            }
            if (image_bgra8) {
                uint8_t* q = image_bgra8 + pix * 4;
                if (frame >= 0) {
                    const float a = 1.0f / (1.0f + (float)frame);
                    V3<float> last = v3((float)q[2] / 255.0f, (float)q[1] / 255.0f, (float)q[0] / 255.0f);
                    fc = mix3(last, fc, a);
                }
                q[0] = quant8(fc.z); q[1] = quant8(fc.y); q[2] = quant8(fc.x); q[3] = 255;
            }
        }
    });
    if (st) for (auto& l : loc) st->add(l);
}

}  // namespace orc
