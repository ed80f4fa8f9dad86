// ORACLE PIN — test infrastructure only.  Runs the reference's own shader
// sources (rewritten into C++ by translate.py, compiled from the reference
// checkout by oracle/glsl_ref/Makefile into oracle/_ref/) on the CPU, playing
// the part of the Vulkan ray-tracing pipeline:
//
//   shadow pipeline  raygen shadowRaygen, miss 0 shadow.rmiss, hit skipped
//                    (src/renderer.cpp:2319-2387, TerminateOnFirstHit |
//                    SkipClosestHit rays)
//   hybrid pipeline  raygen hybridRaygen, miss 0 miss.rmiss, miss 1
//                    shadow.rmiss, hit group hybridHit
//   compute          blur.comp over the W/16 x H/16 workgroups of
//                    src/renderer.cpp:2672
//
// Descriptor contents follow create_shadow_descriptors /
// create_hybrid_descriptors (src/renderer.cpp:1919-2090, 2917-3129).
// Traversal is the oracle's brute-force closest/any hit over all triangles
// (the driver's BVH is not part of the reference's code).  Samplers are
// NEAREST; G-buffer samplers clamp, environment samplers repeat.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../orc_scene.hpp"
#include "glsl.hpp"

namespace glsl {
uvec3 gl_LaunchIDEXT, gl_LaunchSizeEXT, gl_GlobalInvocationID;
vec3 gl_WorldRayOriginEXT, gl_WorldRayDirectionEXT;
float gl_HitTEXT = 0.f;
int gl_PrimitiveID = 0, gl_InstanceCustomIndexEXT = 0;

vec4 texture(const sampler2D& s, const vec2& uv) {
    if (!s.texels || s.w == 0 || s.h == 0) return vec4(0.f);
    float u = uv.x, v = uv.y;
    if (!(u == u)) u = 0.f;
    if (!(v == v)) v = 0.f;
    float fx = std::floor(u * (float)s.w), fy = std::floor(v * (float)s.h);
    fx = std::fmin(std::fmax(fx, -1e9f), 1e9f);
    fy = std::fmin(std::fmax(fy, -1e9f), 1e9f);
    long ix = (long)fx, iy = (long)fy;
    if (s.repeat) {
        ix %= s.w; iy %= s.h;
        if (ix < 0) ix += s.w;
        if (iy < 0) iy += s.h;
    } else {
        ix = ix < 0 ? 0 : (ix >= s.w ? s.w - 1 : ix);
        iy = iy < 0 ? 0 : (iy >= s.h ? s.h - 1 : iy);
    }
    const float* t = s.texels + ((size_t)iy * s.w + ix) * 4;
    return vec4(t[0], t[1], t[2], t[3]);
}

vec4 imageLoad(const image2D& im, const ivec2& p) {
    if (!im.data || p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return vec4(0.f);
    size_t i = (size_t)p.y * im.w + p.x;
    if (im.unorm8 && im.bgra8) {
        const uint8_t* q = (const uint8_t*)im.data + i * 4;
        return vec4((float)q[2] / 255.0f, (float)q[1] / 255.0f, (float)q[0] / 255.0f, (float)q[3] / 255.0f);
    }
    if (im.unorm8) return vec4((float)((const uint8_t*)im.data)[i] / 255.0f, 0.f, 0.f, 1.f);
    const float* f = (const float*)im.data + i * 4;
    return vec4(f[0], f[1], f[2], f[3]);
}

void imageStore(image2D& im, const ivec2& p, const vec4& v) {
    if (!im.data || p.x < 0 || p.y < 0 || p.x >= im.w || p.y >= im.h) return;
    size_t i = (size_t)p.y * im.w + p.x;
    auto u8 = [](float x) { return (uint8_t)std::nearbyint(std::fmin(std::fmax(x, 0.f), 1.f) * 255.0f); };
    if (im.unorm8 && im.bgra8) {
        uint8_t* q = (uint8_t*)im.data + i * 4;
        q[0] = u8(v.z); q[1] = u8(v.y); q[2] = u8(v.x); q[3] = u8(v.w);
        return;
    }
    if (im.unorm8) {
        float c = std::fmin(std::fmax(v.x, 0.f), 1.f) * 255.0f;
        ((uint8_t*)im.data)[i] = (uint8_t)std::nearbyint(c);
    } else {
        float* f = (float*)im.data + i * 4;
        f[0] = v.x; f[1] = v.y; f[2] = v.z; f[3] = v.w;
    }
}

mat4 inverse(const mat4& m) {
    double a[16], inv[16];
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) a[c * 4 + r] = m.c[c].e[r];
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    double det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    double rr = 1.0 / det;
    mat4 o;
    for (int c = 0; c < 4; c++)
        for (int r = 0; r < 4; r++) o.c[c].e[r] = (float)(inv[c * 4 + r] * rr);
    return o;
}

using TraceFn = void (*)(uint flags, uint miss, const vec3& o, float tmin, const vec3& d, float tmax, int payload);
static TraceFn g_trace = nullptr;
void traceRayEXT(const accelerationStructureEXT&, uint flags, uint, uint, uint, uint miss_index, const vec3& origin,
                 float tmin, const vec3& dir, float tmax, int payload) {
    g_trace(flags, miss_index, origin, tmin, dir, tmax, payload);
}
}  // namespace glsl

#include "shadowRaygen.rgen.hpp"
#include "shadow.rmiss.hpp"
#include "hybridRaygen.rgen.hpp"
#include "hybridHit.rchit.hpp"
#include "miss.rmiss.hpp"
#include "blur.comp.hpp"
#include "raygen.rgen.hpp"
#include "closesthit.rchit.hpp"
#include "postFragment.frag.hpp"
namespace sh_helpers {
using namespace glsl;
#include "helpers.glsl.hpp"
}  // namespace sh_helpers

using namespace glsl;

namespace {

struct RefScene {
    orc::Scene os;
    std::vector<int> indices;
    std::vector<float> env[2];
    int env_w[2] = {0, 0}, env_h[2] = {0, 0};
    std::vector<std::vector<float>> tex;   // Texture::_textures, RGBA8 UNORM as floats
    std::vector<int> tex_w, tex_h;
};

// binding 7 / 9 of the hybrid / path-traced sets: the material textures with
// the NEAREST + REPEAT sampler of src/renderer.cpp:3059
void bind_textures(Array<sampler2D>& arr, RefScene& s) {
    arr.v.assign(s.tex.size(), sampler2D());
    for (size_t k = 0; k < s.tex.size(); k++) {
        arr.v[k].texels = s.tex[k].data();
        arr.v[k].w = s.tex_w[k];
        arr.v[k].h = s.tex_h[k];
        arr.v[k].repeat = true;
    }
}

template <class LightT> std::vector<LightT> make_lights(const std::vector<HyLight>& in) {
    std::vector<LightT> v(in.size());
    for (size_t i = 0; i < in.size(); i++) {
        v[i].pos = vec4(in[i].pos[0], in[i].pos[1], in[i].pos[2], in[i].pos[3]);
        v[i].color = vec4(in[i].color[0], in[i].color[1], in[i].color[2], in[i].color[3]);
        v[i].radius = in[i].radius;
    }
    return v;
}
template <class MatT> std::vector<MatT> make_mats(const std::vector<HyMaterial>& in) {
    std::vector<MatT> v(in.size());
    for (size_t i = 0; i < in.size(); i++) {
        v[i].diffuse = vec4(in[i].diffuse[0], in[i].diffuse[1], in[i].diffuse[2], in[i].diffuse[3]);
        v[i].textures = vec4(in[i].textures[0], in[i].textures[1], in[i].textures[2], in[i].textures[3]);
        v[i].shadingMetallicRoughness = vec4(in[i].smr[0], in[i].smr[1], in[i].smr[2], in[i].smr[3]);
    }
    return v;
}
mat4 mat_of(const float* m) {
    mat4 o;
    for (int c = 0; c < 4; c++) o.c[c] = vec4(m[c * 4 + 0], m[c * 4 + 1], m[c * 4 + 2], m[c * 4 + 3]);
    return o;
}

sampler2D plane_sampler(const float* data, int w, int h) {
    sampler2D s;
    s.texels = data;
    s.w = w;
    s.h = h;
    s.repeat = false;
    return s;
}

// ---- pipeline state for the trace hook ----
RefScene* g_scene = nullptr;
int g_pipeline = 0;  // 0 = shadow, 1 = hybrid, 2 = path traced (raygen + closesthit)
std::vector<PayloadTable*> g_callers;

// the closest-hit program of the bound pipeline
struct HitProgram {
    PayloadTable* payloads;
    vec3* attribs;
    void (*main)();
};
HitProgram hit_program() {
    if (g_pipeline == 2) return {&sh_closesthit::g_payloads, &sh_closesthit::attribs, sh_closesthit::main};
    return {&sh_hybridHit::g_payloads, &sh_hybridHit::attribs, sh_hybridHit::main};
}

template <class T> void copy_in(PayloadTable& callee, PayloadTable& caller, int loc) {
    (void)sizeof(T);
    std::memcpy(callee.in_ptr, caller.ptr[loc], caller.size[loc]);
}

void run_miss(PayloadTable& callee, void (*fn)(), PayloadTable& caller, int loc, const vec3& o, const vec3& d) {
    std::memcpy(callee.in_ptr, caller.ptr[loc], caller.size[loc]);
    vec3 so = gl_WorldRayOriginEXT, sd = gl_WorldRayDirectionEXT;
    gl_WorldRayOriginEXT = o;
    gl_WorldRayDirectionEXT = d;
    fn();
    gl_WorldRayOriginEXT = so;
    gl_WorldRayDirectionEXT = sd;
    std::memcpy(caller.ptr[loc], callee.in_ptr, caller.size[loc]);
}

void trace_hook(uint flags, uint miss, const vec3& o, float tmin, const vec3& d, float tmax, int payload) {
    const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    const bool any = (flags & gl_RayFlagsTerminateOnFirstHitEXT) != 0;
    orc::Hit h = orc::trace(g_scene->os, oo, dd, tmin, tmax, any, 0, nullptr);
    PayloadTable& caller = *g_callers.back();
    if (h.id == HY_NO_HIT) {
        if (g_pipeline == 0 || miss == 1) run_miss(sh_shadowMiss::g_payloads, sh_shadowMiss::main, caller, payload, o, d);
        else run_miss(sh_miss::g_payloads, sh_miss::main, caller, payload, o, d);
        return;
    }
    if (flags & gl_RayFlagsSkipClosestHitShaderEXT) return;
    // closest hit: hybridHit.rchit or closesthit.rchit
    const HitProgram hp = hit_program();
    const uint32_t p = g_scene->os.tri_prim[h.id];
    PayloadTable& callee = *hp.payloads;
    std::memcpy(callee.in_ptr, caller.ptr[payload], caller.size[payload]);
    vec3 so = gl_WorldRayOriginEXT, sd = gl_WorldRayDirectionEXT;
    float st = gl_HitTEXT;
    int sp = gl_PrimitiveID, si = gl_InstanceCustomIndexEXT;
    vec3 sa = *hp.attribs;
    gl_WorldRayOriginEXT = o;
    gl_WorldRayDirectionEXT = d;
    gl_HitTEXT = h.t;
    gl_PrimitiveID = (int)(h.id - g_scene->os.prim_tri0[p]);
    gl_InstanceCustomIndexEXT = (int)p;
    *hp.attribs = vec3(h.b1, h.b2, 0.f);
    g_callers.push_back(&callee);
    hp.main();
    g_callers.pop_back();
    std::memcpy(caller.ptr[payload], callee.in_ptr, caller.size[payload]);
    gl_WorldRayOriginEXT = so;
    gl_WorldRayDirectionEXT = sd;
    gl_HitTEXT = st;
    gl_PrimitiveID = sp;
    gl_InstanceCustomIndexEXT = si;
    *hp.attribs = sa;
}

void bind_env(Array<sampler2D>& arr, RefScene& s) {
    arr.v.assign(2, sampler2D());
    for (int k = 0; k < 2; k++) {
        arr.v[k].texels = s.env[k].empty() ? nullptr : s.env[k].data();
        arr.v[k].w = s.env_w[k];
        arr.v[k].h = s.env_h[k];
        arr.v[k].repeat = true;
    }
}

}  // namespace

extern "C" {

void* ref_scene_create() { return new RefScene(); }
void ref_scene_destroy(void* s) { delete (RefScene*)s; }

int ref_scene_set(void* sp, const HyVertex* verts, uint32_t nv, const uint32_t* idx, uint32_t ni,
                  const HyPrimitive* prims, uint32_t np, const float* xf, uint32_t nx, const HyMaterial* mats,
                  uint32_t nm, const HyLight* lights, uint32_t nl) {
    RefScene& s = *(RefScene*)sp;
    s.os.verts.assign(verts, verts + nv);
    s.os.idx.assign(idx, idx + ni);
    s.os.prims.assign(prims, prims + np);
    s.os.xf.assign(xf, xf + (size_t)nx * 16);
    s.os.mats.assign(mats, mats + nm);
    s.os.lights.assign(lights, lights + nl);
    orc::scene_derive(s.os);
    s.indices.assign(idx, idx + ni);
    return 0;
}

int ref_scene_set_texture(void* sp, const uint8_t* px, uint32_t w, uint32_t h) {
    RefScene& s = *(RefScene*)sp;
    std::vector<float> t((size_t)w * h * 4);
    for (size_t i = 0; i < t.size(); i++) t[i] = (float)px[i] / 255.0f;
    s.tex.push_back(std::move(t));
    s.tex_w.push_back((int)w);
    s.tex_h.push_back((int)h);
    return (int)s.tex.size() - 1;
}

int ref_scene_set_env(void* sp, int slot, const uint8_t* px, uint32_t w, uint32_t h) {
    RefScene& s = *(RefScene*)sp;
    s.env[slot].resize((size_t)w * h * 4);
    for (size_t i = 0; i < (size_t)w * h * 4; i++) s.env[slot][i] = (float)px[i] / 255.0f;
    s.env_w[slot] = (int)w;
    s.env_h[slot] = (int)h;
    return 0;
}

// ---- the reference's helper functions ----
uint32_t ref_tea(uint32_t a, uint32_t b) { return sh_helpers::tea(a, b); }
void ref_rnd_seq(uint32_t seed, uint32_t n, uint32_t* states, float* vals) {
    for (uint32_t i = 0; i < n; i++) {
        float v = sh_helpers::rnd(seed);
        if (states) states[i] = seed;
        if (vals) vals[i] = v;
    }
}
void ref_sample_disk(float radius, const float* pos, const float* L, uint32_t seed, float* out) {
    sh_helpers::Light l;
    l.radius = radius;
    vec3 d = sh_helpers::sampleDisk(l, vec3(pos[0], pos[1], pos[2]), vec3(L[0], L[1], L[2]), seed);
    out[0] = d.x; out[1] = d.y; out[2] = d.z;
}
void ref_brdf(const float* N, const float* V, const float* L, float roughness, const float* F0, float cosTheta,
              float* out) {
    vec3 n(N[0], N[1], N[2]), v(V[0], V[1], V[2]), l(L[0], L[1], L[2]);
    vec3 h = normalize(v + l);
    out[0] = sh_helpers::DistributionGGX(n, h, roughness);
    out[1] = sh_helpers::GeometrySmith(n, v, l, roughness);
    vec3 F = sh_helpers::FresnelSchlick(cosTheta, vec3(F0[0], F0[1], F0[2]));
    out[2] = F.x; out[3] = F.y; out[4] = F.z;
}

// ---- shadow pipeline: shadowRaygen.rgen over W x H; out: L images, u8 ----
int ref_shadow_pass(void* sp, uint32_t W, uint32_t H, const float* const* planes, const float* cam36, int samples,
                    uint8_t* out) {
    RefScene& s = *(RefScene*)sp;
    namespace sh = sh_shadowRaygen;
    const uint32_t L = (uint32_t)s.os.lights.size();
    if (L > 3) return -1;  // shadowImage[3] (shadowRaygen.rgen:9)
    std::vector<float> motion4((size_t)W * H * 4, 0.f);
    for (size_t i = 0; i < (size_t)W * H; i++) { motion4[i * 4] = planes[3][i * 2]; motion4[i * 4 + 1] = planes[3][i * 2 + 1]; }
    sh::gbuffers.v = {plane_sampler(planes[0], W, H), plane_sampler(planes[1], W, H),
                      plane_sampler(motion4.data(), W, H)};
    sh::shadowImage.v.assign(3, image2D());
    for (uint32_t l = 0; l < L; l++) {
        sh::shadowImage.v[l].data = out + (size_t)l * W * H;
        sh::shadowImage.v[l].w = (int)W;
        sh::shadowImage.v[l].h = (int)H;
        sh::shadowImage.v[l].unorm8 = true;
    }
    sh::cam.viewInverse = mat_of(cam36);
    sh::cam.projInverse = mat_of(cam36 + 16);
    sh::cam.frame = cam36[32];
    std::vector<sh::Light> lights = make_lights<sh::Light>(s.os.lights);
    std::vector<sh::Material> mats = make_mats<sh::Material>(s.os.mats);
    sh::lightsBuffer.lights.data = lights.data();
    sh::lightsBuffer.lights.n = (int)L;
    sh::materials.mat.data = mats.data();
    sh::materials.mat.n = (int)mats.size();
    sh::samplesBuffer.samples = samples;
    g_scene = &s;
    g_pipeline = 0;
    g_trace = trace_hook;
    g_callers.assign(1, &sh::g_payloads);
    gl_LaunchSizeEXT = uvec3(W, H, 1);
    for (uint32_t y = 0; y < H; y++)
        for (uint32_t x = 0; x < W; x++) {
            gl_LaunchIDEXT = uvec3(x, y, 0);
            sh::main();
        }
    return 0;
}

// ---- blur.comp over the W/16 x H/16 workgroups (WIDTH/HEIGHT/NLIGHTS are 1700/900/3 in the shader) ----
int ref_blur(uint32_t W, uint32_t H, int frame, const float* motion_rg, uint8_t* in3, uint8_t* hist3) {
    namespace sh = sh_blur;
    std::vector<float> motion4((size_t)W * H * 4, 0.f);
    for (size_t i = 0; i < (size_t)W * H; i++) { motion4[i * 4] = motion_rg[i * 2]; motion4[i * 4 + 1] = motion_rg[i * 2 + 1]; }
    sh::motionTexture = plane_sampler(motion4.data(), W, H);
    sh::inputImage.v.assign(3, image2D());
    sh::outputImage.v.assign(3, image2D());
    for (int l = 0; l < 3; l++) {
        sh::inputImage.v[l] = image2D{in3 + (size_t)l * W * H, (int)W, (int)H, true};
        sh::outputImage.v[l] = image2D{hist3 + (size_t)l * W * H, (int)W, (int)H, true};
    }
    sh::frameBuffer.frame = frame;
    for (uint32_t gy = 0; gy < H / 16; gy++)
        for (uint32_t gx = 0; gx < W / 16; gx++)
            for (uint32_t ly = 0; ly < 16; ly++)
                for (uint32_t lx = 0; lx < 16; lx++) {
                    gl_GlobalInvocationID = uvec3(gx * 16 + lx, gy * 16 + ly, 0);
                    sh::main();
                }
    return 0;
}

// ---- hybrid pipeline: hybridRaygen.rgen over W x H; shadow: L denoised u8 images; out: rgba float ----
int ref_hybrid_pass(void* sp, uint32_t W, uint32_t H, const float* const* planes, const float* cam36,
                    uint8_t* shadow, float* out_rgba) {
    RefScene& s = *(RefScene*)sp;
    namespace sh = sh_hybridRaygen;
    namespace hh = sh_hybridHit;
    const uint32_t L = (uint32_t)s.os.lights.size();
    std::vector<float> motion4((size_t)W * H * 4, 0.f);
    for (size_t i = 0; i < (size_t)W * H; i++) { motion4[i * 4] = planes[3][i * 2]; motion4[i * 4 + 1] = planes[3][i * 2 + 1]; }
    sh::gbuffers.v = {plane_sampler(planes[0], W, H), plane_sampler(planes[1], W, H), plane_sampler(planes[2], W, H),
                      plane_sampler(motion4.data(), W, H), plane_sampler(planes[4], W, H),
                      plane_sampler(planes[5], W, H)};
    sh::image = image2D{out_rgba, (int)W, (int)H, false};
    sh::shadowImage.v.assign(L, image2D());
    for (uint32_t l = 0; l < L; l++) sh::shadowImage.v[l] = image2D{shadow + (size_t)l * W * H, (int)W, (int)H, true};
    sh::cam.viewInverse = mat_of(cam36);
    sh::cam.projInverse = mat_of(cam36 + 16);
    sh::cam.frame = vec4(cam36[32], cam36[33], cam36[34], cam36[35]);
    std::vector<sh::Light> lights = make_lights<sh::Light>(s.os.lights);
    std::vector<sh::Material> mats = make_mats<sh::Material>(s.os.mats);
    sh::lightsBuffer.lights = RuntimeArray<sh::Light>{lights.data(), (int)L};
    sh::materials.mat = RuntimeArray<sh::Material>{mats.data(), (int)mats.size()};
    bind_env(sh::environmentTexture, s);
    // closest-hit resources (create_hybrid_descriptors, src/renderer.cpp:3015-3048)
    std::vector<hh::Light> hlights = make_lights<hh::Light>(s.os.lights);
    std::vector<hh::Material> hmats = make_mats<hh::Material>(s.os.mats);
    hh::lightsBuffer.lights = RuntimeArray<hh::Light>{hlights.data(), (int)L};
    hh::materials.mat = RuntimeArray<hh::Material>{hmats.data(), (int)hmats.size()};
    bind_env(hh::environmentTexture, s);
    bind_textures(hh::textures, s);
    const size_t np = s.os.prims.size();
    std::vector<vec4> ids(np);
    std::vector<std::vector<hh::Vertex>> vbuf(np);
    hh::vertices.v.assign(np, hh::Vertices());
    hh::indices.v.assign(np, hh::Indices());
    for (size_t p = 0; p < np; p++) {
        const HyPrimitive& pr = s.os.prims[p];
        ids[p] = vec4((float)p, (float)pr.material_id, (float)pr.transform_id, (float)pr.first_index);
        // rtVertexAttribute: (normal, 1), (color, 1), (uv, 1, 1)
        const size_t nvx = s.os.verts.size() - pr.vertex_offset;
        vbuf[p].resize(nvx);
        for (size_t k = 0; k < nvx; k++) {
            const HyVertex& v = s.os.verts[pr.vertex_offset + k];
            vbuf[p][k].normal = vec4(v.normal[0], v.normal[1], v.normal[2], 1.f);
            vbuf[p][k].color = vec4(v.color[0], v.color[1], v.color[2], 1.f);
            vbuf[p][k].uv = vec4(v.uv[0], v.uv[1], 1.f, 1.f);
        }
        hh::vertices.v[p].v = RuntimeArray<hh::Vertex>{vbuf[p].data(), (int)nvx};
        hh::indices.v[p].i = RuntimeArray<int>{s.indices.data(), (int)s.indices.size()};
    }
    hh::objIndices.idx = RuntimeArray<vec4>{ids.data(), (int)np};
    std::vector<mat4> m4(s.os.xf.size() / 16);
    for (size_t t = 0; t < m4.size(); t++) m4[t] = mat_of(&s.os.xf[t * 16]);
    hh::matrices.m = RuntimeArray<mat4>{m4.data(), (int)m4.size()};
    bind_env(sh_miss::skybox, s);
    g_scene = &s;
    g_pipeline = 1;
    g_trace = trace_hook;
    g_callers.assign(1, &sh::g_payloads);
    gl_LaunchSizeEXT = uvec3(W, H, 1);
    for (uint32_t y = 0; y < H; y++)
        for (uint32_t x = 0; x < W; x++) {
            gl_LaunchIDEXT = uvec3(x, y, 0);
            sh::main();
        }
    return 0;
}

// ---- post pass: postFragment.frag at every pixel centre of a W x H target, sampling the
//      B8G8R8A8 image with the NEAREST / CLAMP _offscreenSampler (src/renderer.cpp:822,
//      2861); the colour attachment is written as UNORM bytes B, G, R, A ----
int ref_post(uint32_t W, uint32_t H, const uint8_t* in_bgra8, uint8_t* out_bgra8) {
    namespace sh = sh_post;
    std::vector<float> tex((size_t)W * H * 4);
    for (size_t i = 0; i < (size_t)W * H; i++) {
        tex[i * 4 + 0] = (float)in_bgra8[i * 4 + 2] / 255.0f;
        tex[i * 4 + 1] = (float)in_bgra8[i * 4 + 1] / 255.0f;
        tex[i * 4 + 2] = (float)in_bgra8[i * 4 + 0] / 255.0f;
        tex[i * 4 + 3] = (float)in_bgra8[i * 4 + 3] / 255.0f;
    }
    sh::finalTexture = plane_sampler(tex.data(), (int)W, (int)H);
    image2D out{out_bgra8, (int)W, (int)H, true, true};
    for (uint32_t y = 0; y < H; y++)
        for (uint32_t x = 0; x < W; x++) {
            sh::outUV = vec2(((float)x + 0.5f) / (float)W, ((float)y + 0.5f) / (float)H);
            sh::main();
            imageStore(out, ivec2((int)x, (int)y), sh::fragColor);
        }
    return 0;
}

// ---- path-traced pipeline (Renderer::raytrace, src/renderer.cpp:465-501): raygen.rgen over
//      W x H, miss 0 miss.rmiss, miss 1 shadow.rmiss, hit group closesthit.rchit; the image
//      is the B8G8R8A8 _rtImage (src/renderer.cpp:1535), read and written in place ----
int ref_pathtrace_pass(void* sp, uint32_t W, uint32_t H, const float* cam36, int samples, uint8_t* image_bgra8) {
    RefScene& s = *(RefScene*)sp;
    namespace sh = sh_raygen;
    namespace ch = sh_closesthit;
    const uint32_t L = (uint32_t)s.os.lights.size();
    sh::image = image2D{image_bgra8, (int)W, (int)H, true, true};
    sh::cam.viewInverse = mat_of(cam36);
    sh::cam.projInverse = mat_of(cam36 + 16);
    sh::cam.frame = vec4(cam36[32], cam36[33], cam36[34], cam36[35]);
    // closest-hit resources (create_rt_descriptors, src/renderer.cpp:2092-2305)
    std::vector<ch::Light> clights = make_lights<ch::Light>(s.os.lights);
    std::vector<ch::Material> cmats = make_mats<ch::Material>(s.os.mats);
    ch::lightsBuffer.lights = RuntimeArray<ch::Light>{clights.data(), (int)L};
    ch::materials.mat = RuntimeArray<ch::Material>{cmats.data(), (int)cmats.size()};
    bind_env(ch::environment_texture, s);
    bind_textures(ch::textures, s);
    ch::samplesBuffer.samples = samples;
    const size_t np = s.os.prims.size();
    std::vector<vec4> ids(np);
    std::vector<std::vector<ch::Vertex>> vbuf(np);
    ch::vertices.v.assign(np, ch::Vertices());
    ch::indices.v.assign(np, ch::Indices());
    for (size_t p = 0; p < np; p++) {
        const HyPrimitive& pr = s.os.prims[p];
        ids[p] = vec4((float)p, (float)pr.material_id, (float)pr.transform_id, (float)pr.first_index);
        const size_t nvx = s.os.verts.size() - pr.vertex_offset;
        vbuf[p].resize(nvx);
        for (size_t k = 0; k < nvx; k++) {
            const HyVertex& v = s.os.verts[pr.vertex_offset + k];
            vbuf[p][k].normal = vec4(v.normal[0], v.normal[1], v.normal[2], 1.f);
            vbuf[p][k].color = vec4(v.color[0], v.color[1], v.color[2], 1.f);
            vbuf[p][k].uv = vec4(v.uv[0], v.uv[1], 1.f, 1.f);
        }
        ch::vertices.v[p].v = RuntimeArray<ch::Vertex>{vbuf[p].data(), (int)nvx};
        ch::indices.v[p].i = RuntimeArray<int>{s.indices.data(), (int)s.indices.size()};
    }
    ch::objIndices.idx = RuntimeArray<vec4>{ids.data(), (int)np};
    std::vector<mat4> m4(s.os.xf.size() / 16);
    for (size_t t = 0; t < m4.size(); t++) m4[t] = mat_of(&s.os.xf[t * 16]);
    ch::matrices.m = RuntimeArray<mat4>{m4.data(), (int)m4.size()};
    bind_env(sh_miss::skybox, s);
    g_scene = &s;
    g_pipeline = 2;
    g_trace = trace_hook;
    g_callers.assign(1, &sh::g_payloads);
    gl_LaunchSizeEXT = uvec3(W, H, 1);
    for (uint32_t y = 0; y < H; y++)
        for (uint32_t x = 0; x < W; x++) {
            gl_LaunchIDEXT = uvec3(x, y, 0);
            sh::main();
        }
    return 0;
}

}  // extern "C"
