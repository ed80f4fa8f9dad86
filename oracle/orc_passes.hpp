// ORACLE — test infrastructure only (see orc_math.hpp).
#pragma once
#include <algorithm>
#include <atomic>
#include <thread>
#include <vector>

#include "orc_scene.hpp"

namespace orc {

struct GBufHost {
    uint32_t w, h;
    const void* plane[6];
    uint32_t fmt[6];
};

struct PassStats {
    uint64_t shadow_rays = 0, reflection_rays = 0, hit_shadow_rays = 0;
    Counters cnt;
    void add(const PassStats& o) {
        shadow_rays += o.shadow_rays;
        reflection_rays += o.reflection_rays;
        hit_shadow_rays += o.hit_shadow_rays;
        cnt.nodes += o.cnt.nodes;
        cnt.tris += o.cnt.tris;
        cnt.status |= o.cnt.status;
    }
};

void set_threads(int n);
int get_threads();

// rows of an image spread over get_threads() workers; f(y, worker)
template <class F> void parallel_rows(uint32_t H, F&& f) {
    int nt = std::min<int>(get_threads(), (int)std::max<uint32_t>(H, 1));
    if (nt <= 1) { for (uint32_t y = 0; y < H; y++) f(y, 0); return; }
    std::atomic<uint32_t> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < nt; t++)
        th.emplace_back([&, t] { for (uint32_t y; (y = next.fetch_add(1)) < H;) f(y, t); });
    for (auto& x : th) x.join();
}

struct HitAttr { V3<float> N; float u, v; uint32_t prim; V3<float> color; };
struct Payload { V3<float> color; float t; V3<float> dir; float scattered; V3<float> origin; };

struct MatSample { V3<float> albedo, emissive, rm; };  // albedo before pow(2.2); rm = (_, roughness, metallic)
V3<float> tex_lookup(const Scene& s, float id, float u, float v);
MatSample material_at(const Scene& s, const HyMaterial& m, float u, float v);
V3<float> irradiance_at(const Scene& s, V3<float> N);
V3<float> miss_color(const Scene& s, V3<float> d);
int mat_index(float f, size_t n);
HitAttr hit_attributes(const Scene& s, const Hit& h);
// hybridHit.rchit; vis (may be NULL) gets bit i set when light i's shadow
// factor came out 2 (lit side, unoccluded)
Payload closest_hit(const Scene& s, const Hit& h, V3<float> ro, V3<float> rd, uint32_t& seed,
                    const HyPassConfig& cfg, int mode, PassStats& ls, uint64_t* vis = nullptr);
void fetch(const GBufHost& g, int p, uint32_t x, uint32_t y, float out[4]);
float accum_load(uint32_t fmt, const void* buf, size_t i);
void accum_store(uint32_t fmt, void* buf, size_t i, float v);
void primary_ray(const HyCamera& cam, uint32_t W, uint32_t H, uint32_t x, uint32_t y, float o[3], float d[3]);

void gbuffer_primary(const Scene& s, const HyCamera& cam, uint32_t W, uint32_t H, float* planes[6], int mode);
void shadow_pass(const Scene& s, const GBufHost& g, const HyCamera& cam, const HyPassConfig& cfg, uint32_t fmt,
                 void* shadow, int mode, PassStats* st);
void accumulate(const GBufHost& g, const HyPassConfig& cfg, uint32_t fmt, const void* shadow, void* hist,
                uint32_t num_lights);
void shade(const Scene& s, const GBufHost& g, const HyCamera& cam, const HyPassConfig& cfg, uint32_t fmt,
           const void* hist, float* out_rgba32f, uint8_t* out_bgra8, int mode, PassStats* st);
// post pass: pow(max(rgb, 0.001), 1/2.2) of n pixels into BGRA8
void post_resolve(uint32_t n, const uint8_t* in_bgra8, const float* in_rgba32f, uint8_t* out_bgra8);
// path-traced mode: camera rays, closesthit.rchit shading, running mean into the
// BGRA8 image (frame >= 0) or a plain store (frame < 0); out_rgba32f gets the
// frame's colour before the mean (either may be NULL)
void pathtrace(const Scene& s, const HyCamera& cam, uint32_t W, uint32_t H, const HyPassConfig& cfg,
               uint8_t* image_bgra8, float* out_rgba32f, int mode, PassStats* st);

}  // namespace orc
