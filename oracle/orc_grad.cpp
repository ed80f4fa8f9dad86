// ORACLE — test infrastructure only (see orc_math.hpp).
//
// FP64 restatement of the shading pass (hybridRaygen.rgen:27-186,
// hybridHit.rchit:24-183, miss.rmiss:13-18) as a function of the material
// parameters (diffuse rgb, roughness, metallic) and the light parameters
// (position xyz, intensity), visibility held fixed, and its derivative:
//   grad_record     one float pass like shade(), keeping what the parameters
//                   do not move continuously (see PixRec)
//   eval_pixel<T>   a pixel's colour from its record, T = double or a
//                   forward-mode dual number
//   grad_forward64  the image in FP64 (central finite differences use it)
//   grad_adjoint64  the gradient of sum(w * image): each pixel is evaluated
//                   with one tangent per parameter it depends on (its
//                   material, every light, each bounce hit's material) and
//                   the tangents are contracted with w and summed
// Branches that switch on a light's side of the surface replay the side
// recorded in float, so the function is smooth in the parameters apart from
// the clamps of the shaders.
#include <cmath>
#include <cstring>
#include <mutex>

#include "orc_grad.hpp"

namespace orc {

namespace {

// ---- forward-mode dual number with KM tangents ----------------------------------
template <int KM> struct Dual {
    double v;
    double d[KM];
    Dual(double x = 0.0) : v(x) { std::memset(d, 0, sizeof(d)); }
    friend Dual operator+(const Dual& a, const Dual& b) {
        Dual r(a.v + b.v);
        for (int i = 0; i < KM; i++) r.d[i] = a.d[i] + b.d[i];
        return r;
    }
    friend Dual operator-(const Dual& a, const Dual& b) {
        Dual r(a.v - b.v);
        for (int i = 0; i < KM; i++) r.d[i] = a.d[i] - b.d[i];
        return r;
    }
    friend Dual operator*(const Dual& a, const Dual& b) {
        Dual r(a.v * b.v);
        for (int i = 0; i < KM; i++) r.d[i] = a.d[i] * b.v + a.v * b.d[i];
        return r;
    }
    friend Dual operator/(const Dual& a, const Dual& b) {
        Dual r(a.v / b.v);
        for (int i = 0; i < KM; i++) r.d[i] = (a.d[i] * b.v - a.v * b.d[i]) / (b.v * b.v);
        return r;
    }
    friend Dual operator-(const Dual& a) {
        Dual r(-a.v);
        for (int i = 0; i < KM; i++) r.d[i] = -a.d[i];
        return r;
    }
};

inline double val(double x) { return x; }
inline double gsqrt(double x) { return std::sqrt(x); }
inline double gpow(double x, double e) { return std::pow(x, e); }
inline double gmax(double a, double b) { return a >= b ? a : b; }
inline double gmin(double a, double b) { return a <= b ? a : b; }

template <int KM> double val(const Dual<KM>& x) { return x.v; }
template <int KM> Dual<KM> gsqrt(const Dual<KM>& a) {
    Dual<KM> r(std::sqrt(a.v));
    const double h = r.v > 0.0 ? 0.5 / r.v : 0.0;
    for (int i = 0; i < KM; i++) r.d[i] = a.d[i] * h;
    return r;
}
template <int KM> Dual<KM> gpow(const Dual<KM>& a, double e) {
    Dual<KM> r(std::pow(a.v, e));
    const double g = a.v > 0.0 ? e * std::pow(a.v, e - 1.0) : (e == 1.0 ? 1.0 : 0.0);
    for (int i = 0; i < KM; i++) r.d[i] = a.d[i] * g;
    return r;
}
// GLSL max/min: the derivative of the selected argument
template <int KM> Dual<KM> gmax(const Dual<KM>& a, double b) { return a.v >= b ? a : Dual<KM>(b); }
template <int KM> Dual<KM> gmin(const Dual<KM>& a, double b) { return a.v <= b ? a : Dual<KM>(b); }

template <class T> T gclamp(const T& a, double lo, double hi) { return gmin(gmax(a, lo), hi); }

template <class T> struct T3 { T x, y, z; };
template <class T> T3<T> t3(V3<float> a) { return {T(a.x), T(a.y), T(a.z)}; }
template <class T> T3<T> operator+(const T3<T>& a, const T3<T>& b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
template <class T> T3<T> operator-(const T3<T>& a, const T3<T>& b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
template <class T> T3<T> operator*(const T3<T>& a, const T3<T>& b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
template <class T> T3<T> scale(const T3<T>& a, const T& s) { return {a.x * s, a.y * s, a.z * s}; }
template <class T> T dot3(const T3<T>& a, const T3<T>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> T3<T> normalize3(const T3<T>& a) {
    const T l = gsqrt(dot3(a, a));
    return {a.x / l, a.y / l, a.z / l};
}
template <class T> T3<T> one_minus(const T3<T>& a) { return {T(1.0) - a.x, T(1.0) - a.y, T(1.0) - a.z}; }

// helpers.glsl:33-80
constexpr double kPI = 3.14159265359;
template <class T> T ggx(const T3<T>& N, const T3<T>& H, const T& rough) {
    const T a = rough * rough;
    const T a2 = a * a;
    const T NdotH = gmax(dot3(N, H), 0.0);
    const T NdotH2 = NdotH * NdotH;
    T denom = NdotH2 * (a2 - T(1.0)) + T(1.0);
    denom = T(kPI) * denom * denom;
    return a2 / denom;
}
template <class T> T schlick_ggx(const T& NdotV, const T& rough) {
    const T r = rough + T(1.0);
    const T k = (r * r) / T(8.0);
    return NdotV / (NdotV * (T(1.0) - k) + k);
}
template <class T> T smith(const T3<T>& N, const T3<T>& V, const T3<T>& L, const T& rough) {
    return schlick_ggx(gmax(dot3(N, V), 0.0), rough) * schlick_ggx(gmax(dot3(N, L), 0.0), rough);
}
template <class T> T3<T> fresnel(const T& cosTheta, const T3<T>& F0) {
    const T p = gpow(T(1.0) - cosTheta, 5.0);
    return F0 + scale(one_minus(F0), p);
}

// one light seen from a point: L (normalised), dist, intensity
template <class T> struct LightT { T3<T> L; T dist, I; bool isDir; double maxd; T3<T> lc; };

template <class T, class LF>
LightT<T> light_at(const HyLight& lt, uint32_t i, const T3<T>& pos, LF&& light) {
    LightT<T> g;
    g.isDir = lt.pos[3] < 0.f;
    g.maxd = lt.pos[3];
    const T3<T> lp{light(i, 0), light(i, 1), light(i, 2)};
    const T3<T> L = g.isDir ? lp : lp - pos;
    g.dist = gsqrt(dot3(L, L));
    g.L = {L.x / g.dist, L.y / g.dist, L.z / g.dist};
    g.I = g.isDir ? T(1.0) : light(i, 3) / (g.dist * g.dist);
    g.lc = {T(lt.color[0]), T(lt.color[1]), T(lt.color[2])};
    return g;
}
template <class T> T fresh_atten(const LightT<T>& g) {
    if (val(g.I) == 0.0) return T(0.0);
    if (g.isDir) return T(0.3);
    const T a = gmax((T(g.maxd) - g.dist) / T(g.maxd), 0.0);
    return a * a;
}

template <class T, class MF, class LF>
T3<T> eval_hit(const Scene& s, const BounceRec& b, uint32_t NL, MF&& mat, LF&& light) {
    const HyMaterial& M = s.mats[b.mat];
    const int smode = (int)M.smr[0];
    T dif[3];
    for (int c = 0; c < 3; c++) dif[c] = b.var_alb ? mat(b.mat, c) : T((&b.ms.albedo.x)[c]);
    const T3<T> albedo{gpow(dif[0], 2.2), gpow(dif[1], 2.2), gpow(dif[2], 2.2)};
    const T rough = b.var_rm ? mat(b.mat, 3) : T(b.ms.rm.y), metal = b.var_rm ? mat(b.mat, 4) : T(b.ms.rm.z);
    const T keep = T(1.0) - metal;
    const T3<T> F0{T(0.04) * keep + albedo.x * metal, T(0.04) * keep + albedo.y * metal,
                   T(0.04) * keep + albedo.z * metal};
    const T3<T> N = t3<T>(b.N), V = t3<T>(b.V), wp = t3<T>(b.wp), irr = t3<T>(b.irr);
    const T NdotV = T(b.NdotV);
    T3<T> Lo{T(0.0), T(0.0), T(0.0)};
    for (uint32_t i = 0; i < NL; i++) {
        const LightT<T> g = light_at<T>(s.lights[i], i, wp, light);
        const T3<T> H = normalize3(V + g.L);
        const T NdotL = gclamp(dot3(N, g.L), 0.0, 1.0);
        const T NdotH = gclamp(dot3(N, H), 0.0, 1.0);
        const T att = fresh_atten(g);
        if (smode == 0) {
            const double sf = ((b.vis >> i) & 1) ? 2.0 : 1.0;
            const T3<T> radiance = scale(g.lc, g.I * att * T(sf));
            const T3<T> F = fresnel(NdotH, F0);
            const T D = ggx(N, H, rough);
            const T G = smith(N, V, g.L, rough);
            const T3<T> numerator = scale(F, D * G);
            const T denominator = gmax(T(4.0) * NdotV * NdotL, 0.000001);
            const T3<T> specular{numerator.x / denominator, numerator.y / denominator, numerator.z / denominator};
            const T3<T> kD = scale(one_minus(F), T(1.0) - metal);
            const T3<T> brdf = scale(kD * albedo, T(1.0 / kPI)) + specular;
            Lo = Lo + scale(brdf * radiance, NdotL);
        } else if (smode == 3) {
            const bool lit = ((b.ndl >> i) & 1) && val(g.I) > 0.0;
            Lo = Lo + (lit ? scale(g.lc * albedo, g.I * att * metal) : scale(irr * albedo, metal));
        } else if (smode == 4) {
            Lo = Lo + (val(g.I) > 0.0 ? scale(g.lc * albedo, g.I * att * metal) : scale(irr * albedo, metal));
        }
    }
    const T3<T> F = fresnel(NdotV, F0);
    const T3<T> kD = scale(one_minus(F), T(1.0) - metal);
    return Lo + kD * albedo * irr + t3<T>(b.ms.emissive);
}

template <class T, class MF, class LF>
T3<T> eval_pixel(const Scene& s, const GradRecord& R, size_t pix, MF&& mat, LF&& light) {
    const PixRec& p = R.px[pix];
    if (!p.active) return t3<T>(p.bg);
    T dif[3], rough, metal;
    for (int c = 0; c < 3; c++) dif[c] = p.var_alb ? mat(p.mi, c) : T(p.gb_mat[c]);
    rough = p.var_rm ? mat(p.mi, 3) : T(p.gb_mat[3]);
    metal = p.var_rm ? mat(p.mi, 4) : T(p.gb_mat[4]);
    const T3<T> albedo{gpow(dif[0], 2.2), gpow(dif[1], 2.2), gpow(dif[2], 2.2)};
    const T keep = T(1.0) - metal;
    const T3<T> F0{T(0.04) * keep + albedo.x * metal, T(0.04) * keep + albedo.y * metal,
                   T(0.04) * keep + albedo.z * metal};
    const T3<T> N = t3<T>(p.N), V = t3<T>(p.V), pos = t3<T>(p.pos), irr = t3<T>(p.irr);
    const T NdotV = T(p.NdotV);
    T3<T> rc{T(0.0), T(0.0), T(0.0)};
    T att = T(1.0);
    for (uint32_t i = 0; i < R.NL; i++) {
        const LightT<T> g = light_at<T>(s.lights[i], i, pos, light);
        const T NdotL = gclamp(dot3(N, g.L), 0.0, 1.0);
        const bool lit = (p.ndl >> i) & 1;
        if (lit) att = fresh_atten(g);  // hybridRaygen.rgen updates it on the lit side only
        const double sfac = R.sfac[pix * R.NL + i];
        if (p.smode == 0) {
            const T3<T> radiance = scale(g.lc, g.I * att * T(sfac));
            const T3<T> H = normalize3(V + g.L);
            const T D = ggx(N, H, rough);
            const T G = smith(N, V, g.L, rough);
            const T3<T> F = fresnel(gmax(dot3(H, V), 0.0), F0);
            const T3<T> kD = scale(one_minus(F), T(1.0) - metal);
            const T3<T> numerator = scale(F, D * G);
            const T denominator = gmax(T(4.0) * NdotV * NdotL, 0.001);
            const T3<T> specular{numerator.x / denominator, numerator.y / denominator, numerator.z / denominator};
            const T3<T> brdf = scale(kD * albedo, T(1.0 / kPI)) + specular;
            rc = rc + scale(brdf * radiance, NdotL);
        } else if (p.smode == 3) {
            rc = rc + ((lit && val(g.I) > 0.0) ? scale(g.lc * albedo, g.I * att * T(sfac) * metal)
                                               : scale(irr * albedo, metal));
        } else if (p.smode == 4) {
            rc = rc + (val(g.I) > 0.0 ? scale(g.lc * albedo, g.I * att * metal) : scale(irr * albedo, metal));
        }
    }
    for (int k = 0; k < p.nb; k++) {
        const BounceRec& b = p.b[k];
        const T3<T> pc = b.hit ? eval_hit<T>(s, b, R.NL, mat, light) : t3<T>(b.miss);
        rc = rc * pc;
    }
    const T3<T> F = fresnel(NdotV, F0);
    const T3<T> kD = scale(one_minus(F), T(1.0) - metal);
    return rc + (kD * albedo * irr + t3<T>(p.emis));
}

template <int KM>
void adjoint_rows(const Scene& s, const GradRecord& R, const double* mats, const double* lights, const double* w,
                  double* g_mats, double* g_lights) {
    const size_t nm5 = s.mats.size() * 5, nl4 = s.lights.size() * 4;
    std::mutex mu;
    parallel_rows(R.H, [&](uint32_t y, int) {
        std::vector<double> gm(nm5, 0.0), gl(nl4, 0.0);
        for (uint32_t x = 0; x < R.W; x++) {
            const size_t pix = (size_t)y * R.W + x;
            const PixRec& p = R.px[pix];
            if (!p.active) continue;
            // tangent slots: the lights, then each distinct material in order of use
            int mslot_mat[1 + kGradMaxBounces];
            int mslot_base[1 + kGradMaxBounces];
            int nms = 0;
            const int light_base = 0;
            int next = (int)(4 * R.NL);
            auto slot_of = [&](int m) {
                for (int j = 0; j < nms; j++)
                    if (mslot_mat[j] == m) return mslot_base[j];
                mslot_mat[nms] = m;
                mslot_base[nms] = next;
                nms++;
                next += 5;
                return next - 5;
            };
            if (p.mi >= 0) slot_of(p.mi);
            for (int k = 0; k < p.nb; k++)
                if (p.b[k].hit) slot_of(p.b[k].mat);
            auto mat = [&](int m, int q) {
                Dual<KM> r(mats[(size_t)m * 5 + q]);
                r.d[slot_of(m) + q] = 1.0;
                return r;
            };
            auto light = [&](uint32_t i, int q) {
                Dual<KM> r(lights[(size_t)i * 4 + q]);
                r.d[light_base + 4 * i + q] = 1.0;
                return r;
            };
            const T3<Dual<KM>> c = eval_pixel<Dual<KM>>(s, R, pix, mat, light);
            const double wx = w[pix * 3 + 0], wy = w[pix * 3 + 1], wz = w[pix * 3 + 2];
            auto contract = [&](int j) { return wx * c.x.d[j] + wy * c.y.d[j] + wz * c.z.d[j]; };
            for (uint32_t i = 0; i < R.NL; i++)
                for (int q = 0; q < 4; q++) gl[(size_t)i * 4 + q] += contract(light_base + 4 * i + q);
            for (int j = 0; j < nms; j++)
                for (int q = 0; q < 5; q++) gm[(size_t)mslot_mat[j] * 5 + q] += contract(mslot_base[j] + q);
        }
        std::lock_guard<std::mutex> lk(mu);
        for (size_t j = 0; j < nm5; j++) g_mats[j] += gm[j];
        for (size_t j = 0; j < nl4; j++) g_lights[j] += gl[j];
    });
}

}  // namespace

// ---- the float record pass: shade() without the colour ------------------------------
void grad_record(const Scene& s, const GBufHost& g, const HyCamera& cam, const HyPassConfig& cfg, uint32_t fmt,
                 const void* hist, uint32_t NL, int mode, GradRecord& R) {
    const uint32_t W = g.w, H = g.h;
    const size_t plane = (size_t)W * H;
    R.W = W;
    R.H = H;
    R.NL = NL;
    R.px.assign(plane, PixRec{});
    R.sfac.assign(plane * NL, 0.f);
    parallel_rows(H, [&](uint32_t y, int) {
        PassStats ls;
        for (uint32_t x = 0; x < W; x++) {
            const size_t pix = (size_t)y * W + x;
            PixRec& p = R.px[pix];
            uint32_t seed = tea(y * W + x, (uint32_t)(int)cam.frame[0]);
            float g0[4], g1[4], g2[4], g4[4], g5[4];
            fetch(g, 0, x, y, g0); fetch(g, 1, x, y, g1); fetch(g, 2, x, y, g2);
            fetch(g, 4, x, y, g4); fetch(g, 5, x, y, g5);
            p.mi = mat_index(g0[3], s.mats.size());
            p.smode = p.mi >= 0 ? (int)s.mats[p.mi].smr[0] : 0;
            const float ior = p.mi >= 0 ? s.mats[p.mi].diffuse[3] : 1.f;
            p.pos = v3(g0[0], g0[1], g0[2]);
            const V3<float> normal = v3(g1[0] * 2.0f - 1.0f, g1[1] * 2.0f - 1.0f, g1[2] * 2.0f - 1.0f);
            p.bg = pow3(v3(g2[0], g2[1], g2[2]), 2.2f);
            p.emis = v3(g5[0], g5[1], g5[2]);
            p.gb_mat[0] = g2[0]; p.gb_mat[1] = g2[1]; p.gb_mat[2] = g2[2];
            p.gb_mat[3] = g4[1]; p.gb_mat[4] = g4[2];
            p.var_alb = p.mi >= 0 && !(s.mats[p.mi].textures[0] > -1.f);
            p.var_rm = p.mi >= 0 && !(s.mats[p.mi].textures[3] > -1.f);
            p.active = !(g0[3] == 0.f && g1[3] == 0.f);
            p.nb = 0;
            p.ndl = 0;
            for (uint32_t i = 0; i < NL; i++) R.sfac[pix * NL + i] = accum_load(fmt, hist, i * plane + pix);
            if (!p.active) continue;
            const V3<float> camPos = v3(cam.inv_view[12], cam.inv_view[13], cam.inv_view[14]);
            p.V = normalize(camPos - p.pos);
            p.N = normalize(normal);
            p.NdotV = clampv(dot(p.N, p.V), 0.f, 1.f);
            p.irr = irradiance_at(s, p.N);
            V3<float> origin = v3(0.f, 0.f, 0.f), direction = v3(0.f, 0.f, 0.f);
            for (uint32_t i = 0; i < NL; i++) {
                const HyLight& lt = s.lights[i];
                const bool isDir = lt.pos[3] < 0.f;
                V3<float> L = isDir ? v3(lt.pos[0], lt.pos[1], lt.pos[2]) : v3(lt.pos[0], lt.pos[1], lt.pos[2]) - p.pos;
                L = normalize(L);
                if (clampv(dot(p.N, L), 0.f, 1.f) > 0.f && i < 64) p.ndl |= 1ull << i;
                if (p.smode == 3) {
                    direction = reflect(normalize(-p.V), p.N);
                    origin = p.pos;
                }
                if (p.smode == 4) {
                    origin = p.pos;
                    const float cosAlpha = dot(p.N, p.V);
                    const V3<float> Iv = -p.V;
                    const float NdotI = dot(p.N, Iv);
                    const V3<float> refrN = NdotI > 0.f ? -p.N : p.N;
                    const float eta = NdotI > 0.f ? 1.0f / ior : ior;
                    const float radicand = 1.0f + std::pow(eta, 2.0f) * (cosAlpha * cosAlpha - 1.0f);
                    direction = radicand < 0.f ? reflect(Iv, p.N) : refract(Iv, refrN, eta);
                }
            }
            if ((cfg.flags & HY_FLAG_GGX_REFLECTION) && p.smode == 3 && cfg.max_bounces > 0) {
                const float u1 = rnd(seed), u2 = rnd(seed);
                direction = ggx_reflect<float>(p.N, p.V, g4[1], u1, u2);
            }
            for (uint32_t depth = 0; depth < cfg.max_bounces && depth < (uint32_t)kGradMaxBounces; depth++) {
                if (p.smode == 0) break;
                const V3<float> ro = origin + direction * 1e-2f;
                const float oo[3] = {ro.x, ro.y, ro.z}, dd[3] = {direction.x, direction.y, direction.z};
                const Hit h = trace(s, oo, dd, 0.001f, 1000.0f, false, mode, nullptr);
                BounceRec& b = p.b[p.nb++];
                b.hit = h.id != HY_NO_HIT;
                b.vis = 0;
                b.ndl = 0;
                float pt, pw = 0.f;
                V3<float> pdir = direction, porg = origin;
                if (!b.hit) {
                    b.miss = miss_color(s, direction);
                    pt = -1.f;
                } else {
                    Payload pl = closest_hit(s, h, ro, direction, seed, cfg, mode, ls, &b.vis);
                    const HitAttr a = hit_attributes(s, h);
                    b.mat = (int)s.prims[a.prim].material_id;
                    b.ms = material_at(s, s.mats[b.mat], a.u, a.v);
                    b.var_alb = !(s.mats[b.mat].textures[0] > -1.f);
                    b.var_rm = !(s.mats[b.mat].textures[3] > -1.f);
                    b.N = a.N;
                    b.V = normalize(-direction);
                    b.wp = ro + direction * h.t;
                    b.NdotV = clampv(dot(b.N, b.V), 0.f, 1.f);
                    b.irr = irradiance_at(s, b.N);
                    for (uint32_t i = 0; i < NL; i++) {
                        const HyLight& lt = s.lights[i];
                        const bool isDir = lt.pos[3] < 0.f;
                        V3<float> L = isDir ? v3(lt.pos[0], lt.pos[1], lt.pos[2])
                                            : v3(lt.pos[0], lt.pos[1], lt.pos[2]) - b.wp;
                        L = normalize(L);
                        if (clampv(dot(b.N, L), 0.f, 1.f) > 0.f && i < 64) b.ndl |= 1ull << i;
                    }
                    pt = pl.t; pdir = pl.dir; pw = pl.scattered; porg = pl.origin;
                }
                if (pt < 0.f || !(pw > 0.f)) break;
                origin = porg;
                direction = pdir;
            }
        }
    });
}

void grad_forward64(const Scene& s, const GradRecord& R, const double* mats, const double* lights, double* rgb) {
    auto mat = [&](int m, int q) { return mats[(size_t)m * 5 + q]; };
    auto light = [&](uint32_t i, int q) { return lights[(size_t)i * 4 + q]; };
    parallel_rows(R.H, [&](uint32_t y, int) {
        for (uint32_t x = 0; x < R.W; x++) {
            const size_t pix = (size_t)y * R.W + x;
            const T3<double> c = eval_pixel<double>(s, R, pix, mat, light);
            rgb[pix * 3 + 0] = c.x;
            rgb[pix * 3 + 1] = c.y;
            rgb[pix * 3 + 2] = c.z;
        }
    });
}

void grad_adjoint64(const Scene& s, const GradRecord& R, const double* mats, const double* lights, const double* w,
                    double* g_mats, double* g_lights) {
    std::memset(g_mats, 0, s.mats.size() * 5 * sizeof(double));
    std::memset(g_lights, 0, s.lights.size() * 4 * sizeof(double));
    int maxb = 0;
    for (const PixRec& p : R.px) maxb = std::max(maxb, p.nb);
    const int need = (int)(4 * R.NL) + 5 * (1 + maxb);
    if (need <= 48) adjoint_rows<48>(s, R, mats, lights, w, g_mats, g_lights);
    else if (need <= 96) adjoint_rows<96>(s, R, mats, lights, w, g_mats, g_lights);
    else adjoint_rows<4 * 64 + 5 * (1 + kGradMaxBounces)>(s, R, mats, lights, w, g_mats, g_lights);
}

}  // namespace orc
