// ORACLE — test infrastructure only (see orc_math.hpp).  FP64 restatement of
// the shading pass as a function of the scene's material and light
// parameters, with visibility held fixed, and its derivative.
#pragma once
#include <cstdint>
#include <vector>

#include "orc_passes.hpp"

namespace orc {

constexpr int kGradMaxBounces = 8;

// What the parameters do not move continuously, recorded once in float like
// shade(): each pixel's G-buffer geometry, its bounce rays' hits, the bounce
// hits' shadow-ray outcomes and which side of the surface each light is on.
struct BounceRec {
    bool hit;
    int mat;                        // material of the hit
    V3<float> N, V, wp, irr, miss;  // hit normal, -ray direction, hit point, irradiance / miss colour
    float NdotV;
    uint64_t vis;                   // bit i: light i's shadow factor was 2
    uint64_t ndl;                   // bit i: light i on the lit side of the hit
    bool var_alb, var_rm;           // diffuse / roughness-metallic are parameters (no texture)
    MatSample ms;                   // the material's inputs at the hit (textures sampled)
};
struct PixRec {
    bool active;                    // false: background, the colour is the G-buffer albedo
    int mi, smode;                  // material index (-1: none) and its shading model
    V3<float> pos, N, V, irr, emis, bg;
    float NdotV;
    float gb_mat[5];                // G-buffer diffuse rgb, roughness, metallic (constants where not parameters)
    bool var_alb, var_rm;           // the G-buffer values are the material's parameters
    uint64_t ndl;                   // bit i: light i on the lit side of the pixel
    int nb;
    BounceRec b[kGradMaxBounces];
};
struct GradRecord {
    uint32_t W = 0, H = 0, NL = 0;
    std::vector<PixRec> px;
    std::vector<float> sfac;        // [pix * NL + light]: the shadow images the shading read
};

void grad_record(const Scene& s, const GBufHost& g, const HyCamera& cam, const HyPassConfig& cfg, uint32_t fmt,
                 const void* hist, uint32_t num_lights, int mode, GradRecord& R);
// mats: 5 per material (diffuse rgb, roughness, metallic); lights: 4 per light (position, intensity)
void grad_forward64(const Scene& s, const GradRecord& R, const double* mats, const double* lights, double* rgb);
// gradient of sum(w * image): forward-mode dual numbers, one tangent per parameter a pixel depends on
void grad_adjoint64(const Scene& s, const GradRecord& R, const double* mats, const double* lights, const double* w,
                    double* g_mats, double* g_lights);

}  // namespace orc
