// ORACLE — test infrastructure only (see orc_math.hpp).  C entry points for the
// Python test harness (ctypes).  The scene setters take the same arrays as the
// product's hy_scene_* calls so both sides are fed identical inputs.
#include <cstring>

#include "orc_grad.hpp"
#include "orc_passes.hpp"

using namespace orc;

extern "C" {

void* orc_scene_create() { return new Scene(); }
void orc_scene_destroy(void* s) { delete (Scene*)s; }
void orc_set_threads(int n) { set_threads(n); }
int orc_get_threads() { return get_threads(); }

int orc_scene_set_geometry(void* sp, const HyVertex* verts, uint32_t nv, const uint32_t* idx, uint32_t ni,
                           const HyPrimitive* prims, uint32_t np, const float* xf, uint32_t nx) {
    Scene& s = *(Scene*)sp;
    s.verts.assign(verts, verts + nv);
    s.idx.assign(idx, idx + ni);
    s.prims.assign(prims, prims + np);
    s.xf.assign(xf, xf + (size_t)nx * 16);
    scene_derive(s);
    return 0;
}
int orc_scene_set_materials(void* sp, const HyMaterial* m, uint32_t n) {
    ((Scene*)sp)->mats.assign(m, m + n);
    return 0;
}
int orc_scene_set_lights(void* sp, const HyLight* l, uint32_t n) {
    ((Scene*)sp)->lights.assign(l, l + n);
    return 0;
}
int orc_scene_set_env(void* sp, int slot, const uint8_t* px, uint32_t w, uint32_t h) {
    Env& e = ((Scene*)sp)->env[slot & 1];
    e.w = w; e.h = h;
    e.px.assign(px, px + (size_t)w * h * 4);
    return 0;
}
int orc_scene_set_textures(void* sp, const uint8_t* const* px, const uint32_t* w, const uint32_t* h, uint32_t n) {
    Scene& s = *(Scene*)sp;
    s.tex.assign(n, Env());
    for (uint32_t i = 0; i < n; i++) {
        s.tex[i].w = w[i];
        s.tex[i].h = h[i];
        s.tex[i].px.assign(px[i], px[i] + (size_t)w[i] * h[i] * 4);
    }
    return 0;
}
uint32_t orc_num_tris(void* sp) { return ((Scene*)sp)->ntri; }
void orc_world_tris(void* sp, float* out) {
    Scene& s = *(Scene*)sp;
    std::memcpy(out, s.world.data(), s.world.size() * 4);
}

// BVH build; info = {n, n_bvh2, n_bvh8, depth}
int orc_bvh_build(void* sp, uint32_t* info, float* bounds6) {
    Scene& s = *(Scene*)sp;
    bvh_build(s);
    if (info) {
        info[0] = s.bvh.n;
        info[1] = (uint32_t)s.bvh.bvh2.size();
        info[2] = (uint32_t)s.bvh.bvh8.size();
        info[3] = s.bvh.depth;
    }
    if (bounds6)
        for (int a = 0; a < 3; a++) { bounds6[a] = s.bvh.slo[a]; bounds6[3 + a] = s.bvh.shi[a]; }
    return s.bvh_ok ? 0 : -8;
}
// two-level build (hy_bvh_build_instanced's counterpart); layout = the 8 words
// of HyBvhLayout
static void layout_of(const Scene& s, uint32_t* L) {
    const Bvh2L& T = s.two;
    L[0] = s.two_level ? 1u : 0u;
    L[1] = (uint32_t)T.nodes.size();
    L[2] = (uint32_t)(T.tris.size() / 12);
    L[3] = T.ninst;
    L[4] = T.nblas;
    L[5] = T.tlas_region;
    L[6] = T.tlas_nodes;
    L[7] = T.tlas_depth + T.blas_depth;
}
// any-hit child order (HY_ANYHIT_*), as hy_scene_set_anyhit_order
int orc_scene_set_anyhit_order(void* sp, uint32_t order) {
    if (order > HY_ANYHIT_NEAR_FIRST) return HY_ERR_INVALID_ARG;
    ((Scene*)sp)->anyhit_order = order;
    return HY_OK;
}

int orc_scene_set_build_mode(void* sp, uint32_t mode) {
    if (mode > HY_BUILD_LBVH) return HY_ERR_INVALID_ARG;
    ((Scene*)sp)->build_mode = mode;
    return 0;
}
int orc_bvh_build_instanced(void* sp, uint32_t* layout) {
    Scene& s = *(Scene*)sp;
    bvh_build_instanced(s);
    if (layout) layout_of(s, layout);
    return s.bvh_ok ? 0 : -8;
}
void orc_bvh_download_instanced(void* sp, uint32_t* layout, uint32_t* bvh8, float* tris, float* inst,
                                float* boxes) {
    const Scene& s = *(const Scene*)sp;
    const Bvh2L& T = s.two;
    if (layout) layout_of(s, layout);
    if (bvh8) std::memcpy(bvh8, T.nodes.data(), T.nodes.size() * 80);
    if (tris) std::memcpy(tris, T.tris.data(), T.tris.size() * 4);
    if (inst) std::memcpy(inst, T.inst.data(), T.inst.size() * 4);
    if (boxes) std::memcpy(boxes, T.inst_box.data(), T.inst_box.size() * 4);
}
// new transforms, same topology (hy_bvh_refit's counterpart)
int orc_bvh_refit(void* sp, const float* xf, uint32_t nx) {
    Scene& s = *(Scene*)sp;
    if (!s.bvh_ok || (size_t)nx * 16 != s.xf.size()) return -1;
    s.xf.assign(xf, xf + (size_t)nx * 16);
    derive_world(s);
    bvh_refit(s);
    return 0;
}

void orc_bvh_download(void* sp, uint32_t* morton, uint32_t* order, uint32_t* bvh2, uint32_t* bvh8, float* tris) {
    Bvh& B = ((Scene*)sp)->bvh;
    if (morton) std::memcpy(morton, B.morton.data(), B.morton.size() * 4);
    if (order) std::memcpy(order, B.order.data(), B.order.size() * 4);
    if (bvh2)
        for (size_t i = 0; i < B.bvh2.size(); i++) {
            uint32_t* o = bvh2 + i * 10;
            o[0] = B.bvh2[i].left; o[1] = B.bvh2[i].right; o[2] = B.bvh2[i].first; o[3] = B.bvh2[i].last;
            std::memcpy(o + 4, B.bvh2[i].lo, 12);
            std::memcpy(o + 7, B.bvh2[i].hi, 12);
        }
    if (bvh8) std::memcpy(bvh8, B.bvh8.data(), B.bvh8.size() * 80);
    if (tris) std::memcpy(tris, B.tris.data(), B.tris.size() * 4);
}

// rays: 8 floats (org, tmin, dir, tmax); hits: 4 words (t, id, b1, b2);
// counters: per-ray {nodes, tris} as uint32 pairs (may be NULL)
void orc_trace(void* sp, const float* rays, uint32_t n, int any_hit, int mode, float* hits, uint32_t* counters) {
    Scene& s = *(Scene*)sp;
    for (uint32_t i = 0; i < n; i++) {
        const float* r = rays + (size_t)i * 8;
        Counters c;
        Hit h = trace(s, r, r + 4, r[3], r[7], any_hit != 0, mode, &c);
        float* o = hits + (size_t)i * 4;
        o[0] = h.id == HY_NO_HIT ? 0.f : h.t;
        std::memcpy(o + 1, &h.id, 4);
        o[2] = h.id == HY_NO_HIT ? 0.f : h.b1;
        o[3] = h.id == HY_NO_HIT ? 0.f : h.b2;
        if (counters) { counters[2 * i] = (uint32_t)c.nodes; counters[2 * i + 1] = (uint32_t)c.tris; }
    }
}

// tea / lcg / rnd / sampleDisk known-answer helpers
uint32_t orc_tea(uint32_t a, uint32_t b) { return tea(a, b); }
void orc_rnd_seq(uint32_t seed, uint32_t n, uint32_t* states, float* vals) {
    for (uint32_t i = 0; i < n; i++) {
        float v = rnd(seed);
        if (states) states[i] = seed;
        if (vals) vals[i] = v;
    }
}
void orc_sample_disk(const float* light_radius, const float* pos, const float* L, uint32_t seed, float* out) {
    uint32_t sd = seed;
    V3<float> d = sampleDisk<float>(*light_radius, v3(pos[0], pos[1], pos[2]), v3(L[0], L[1], L[2]), sd);
    out[0] = d.x; out[1] = d.y; out[2] = d.z;
}
// out: D, G, F.rgb for one (N, V, L, roughness, F0) evaluation
// ggx_reflect in float (dbl = 0) or double (dbl = 1); out: the direction (3 floats)
void orc_ggx_reflect(const float* N, const float* V, float roughness, float u1, float u2, int dbl, float* out) {
    if (dbl) {
        const V3<double> d = ggx_reflect<double>(v3<double>(N[0], N[1], N[2]), v3<double>(V[0], V[1], V[2]),
                                                 roughness, u1, u2);
        out[0] = (float)d.x; out[1] = (float)d.y; out[2] = (float)d.z;
    } else {
        const V3<float> d = ggx_reflect<float>(v3(N[0], N[1], N[2]), v3(V[0], V[1], V[2]), roughness, u1, u2);
        out[0] = d.x; out[1] = d.y; out[2] = d.z;
    }
}

void orc_brdf(const float* N, const float* V, const float* L, float roughness, const float* F0, float cosTheta,
              float* out) {
    V3<float> n = v3(N[0], N[1], N[2]), v = v3(V[0], V[1], V[2]), l = v3(L[0], L[1], L[2]);
    V3<float> h = normalize(v + l);
    out[0] = DistributionGGX(n, h, roughness);
    out[1] = GeometrySmith(n, v, l, roughness);
    V3<float> F = FresnelSchlick(cosTheta, v3(F0[0], F0[1], F0[2]));
    out[2] = F.x; out[3] = F.y; out[4] = F.z;
}

static GBufHost gb_of(const HyGBuffer* g) {
    GBufHost h;
    h.w = g->width; h.h = g->height;
    for (int i = 0; i < 6; i++) { h.plane[i] = g->plane[i]; h.fmt[i] = g->format[i]; }
    return h;
}
static void stats_out(const PassStats& p, HyStats* st) {
    if (!st) return;
    st->shadow_rays = p.shadow_rays;
    st->reflection_rays = p.reflection_rays;
    st->hit_shadow_rays = p.hit_shadow_rays;
    st->nodes_visited = p.cnt.nodes;
    st->tris_tested = p.cnt.tris;
    st->error_flags = p.cnt.status;
}

int orc_gbuffer_primary(void* sp, const HyCamera* cam, uint32_t W, uint32_t H, float** planes, int mode) {
    gbuffer_primary(*(Scene*)sp, *cam, W, H, planes, mode);
    return 0;
}
int orc_shadow_pass(void* sp, const HyGBuffer* g, const HyCamera* cam, const HyPassConfig* cfg, uint32_t fmt,
                    void* shadow, int mode, HyStats* st) {
    PassStats p;
    shadow_pass(*(Scene*)sp, gb_of(g), *cam, *cfg, fmt, shadow, mode, &p);
    stats_out(p, st);
    return 0;
}
int orc_accumulate(void* sp, const HyGBuffer* g, const HyPassConfig* cfg, const void* shadow, HyAccum* acc) {
    accumulate(gb_of(g), *cfg, acc->format, shadow, acc->history, acc->num_lights);
    (void)sp;
    return 0;
}
int orc_shade(void* sp, const HyGBuffer* g, const HyCamera* cam, const HyPassConfig* cfg, const HyAccum* acc,
              float* out_rgba32f, uint8_t* out_bgra8, int mode, HyStats* st) {
    PassStats p;
    shade(*(Scene*)sp, gb_of(g), *cam, *cfg, acc->format, acc->history, out_rgba32f, out_bgra8, mode, &p);
    stats_out(p, st);
    return 0;
}

void orc_post_resolve(uint32_t n, const uint8_t* in_bgra8, const float* in_rgba32f, uint8_t* out_bgra8) {
    post_resolve(n, in_bgra8, in_rgba32f, out_bgra8);
}

int orc_pathtrace(void* sp, const HyCamera* cam, uint32_t W, uint32_t H, const HyPassConfig* cfg,
                  uint8_t* image_bgra8, float* out_rgba32f, int mode, HyStats* st) {
    PassStats p;
    pathtrace(*(Scene*)sp, *cam, W, H, *cfg, image_bgra8, out_rgba32f, mode, &p);
    stats_out(p, st);
    return 0;
}

// ---- FP64 shading as a function of the material / light parameters ----
// The record's light count is the scene's (closest_hit shades with every
// scene light); acc->num_lights must equal it.
void* orc_grad_record(void* sp, const HyGBuffer* g, const HyCamera* cam, const HyPassConfig* cfg,
                      const HyAccum* acc, int mode) {
    Scene& s = *(Scene*)sp;
    if (acc->num_lights != s.lights.size() || s.lights.size() > 64) return nullptr;
    GradRecord* R = new GradRecord();
    grad_record(s, gb_of(g), *cam, *cfg, acc->format, acc->history, acc->num_lights, mode, *R);
    return R;
}
void orc_grad_free(void* r) { delete (GradRecord*)r; }
int orc_grad_forward(void* sp, void* r, const double* mats, const double* lights, double* rgb) {
    grad_forward64(*(Scene*)sp, *(GradRecord*)r, mats, lights, rgb);
    return 0;
}
int orc_grad_adjoint(void* sp, void* r, const double* mats, const double* lights, const double* w, double* g_mats,
                     double* g_lights) {
    grad_adjoint64(*(Scene*)sp, *(GradRecord*)r, mats, lights, w, g_mats, g_lights);
    return 0;
}

}  // extern "C"
