// ORACLE — test infrastructure only (see orc_math.hpp).
#pragma once
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

}  // namespace orc
