// The C++ host side (include/hybridrt.hpp) driven the way the reference's
// engine drives its renderer: build a scene of Objects / Lights / Materials,
// load it, build the acceleration structure, then per frame update the frame
// counter and call rasterize_hybrid.  The frames must equal, bit for bit, the
// same inputs sent through the C ABI directly; a refit after moving an entity
// must render without errors.  Exit code 0 on success.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "hybridrt.hpp"

using namespace hybridrt;

static Mesh icosahedron() {
    const float t = (1.0f + std::sqrt(5.0f)) / 2.0f;
    const float p[12][3] = {{-1, t, 0}, {1, t, 0}, {-1, -t, 0}, {1, -t, 0}, {0, -1, t}, {0, 1, t},
                            {0, -1, -t}, {0, 1, -t}, {t, 0, -1}, {t, 0, 1}, {-t, 0, -1}, {-t, 0, 1}};
    const uint32_t f[20][3] = {{0, 11, 5}, {0, 5, 1}, {0, 1, 7}, {0, 7, 10}, {0, 10, 11}, {1, 5, 9}, {5, 11, 4},
                               {11, 10, 2}, {10, 7, 6}, {7, 1, 8}, {3, 9, 4}, {3, 4, 2}, {3, 2, 6}, {3, 6, 8},
                               {3, 8, 9}, {4, 9, 5}, {2, 4, 11}, {6, 2, 10}, {8, 6, 7}, {9, 8, 1}};
    Mesh m;
    for (auto& v : p) {
        const float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        HyVertex x;
        std::memset(&x, 0, sizeof(x));
        for (int k = 0; k < 3; k++) { x.pos[k] = v[k] / l; x.normal[k] = v[k] / l; x.color[k] = 1.f; }
        m.vertices.push_back(x);
    }
    for (auto& tri : f) m.indices.insert(m.indices.end(), tri, tri + 3);
    return m;
}

static Mesh quad(float half) {
    Mesh m;
    const float c[4][2] = {{-half, -half}, {half, -half}, {half, half}, {-half, half}};
    for (auto& q : c) {
        HyVertex x;
        std::memset(&x, 0, sizeof(x));
        x.pos[0] = q[0]; x.pos[2] = q[1]; x.normal[1] = 1.f; x.color[0] = x.color[1] = x.color[2] = 1.f;
        m.vertices.push_back(x);
    }
    m.indices = {0, 2, 1, 0, 3, 2};
    return m;
}

static void translate_scale(float* m, float x, float y, float z, float s) {
    std::memset(m, 0, 64);
    m[0] = m[5] = m[10] = s;
    m[15] = 1.f;
    m[12] = x; m[13] = y; m[14] = z;
}

// pinhole camera at `eye` looking at the origin: inverse view (camera -> world) and
// inverse projection of a perspective with the given vertical field of view
static HyCamera camera(const float eye[3], float fovy_deg, float aspect, float frame) {
    HyCamera c;
    std::memset(&c, 0, sizeof(c));
    float f[3] = {-eye[0], -eye[1], -eye[2]};
    float fl = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (float& v : f) v /= fl;
    float r[3] = {f[1] * 0 - f[2] * 1, f[2] * 0 - f[0] * 0, f[0] * 1 - f[1] * 0};  // f x (0,1,0)
    float rl = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (float& v : r) v /= rl;
    float u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
    for (int i = 0; i < 3; i++) {
        c.inv_view[0 + i] = r[i];
        c.inv_view[4 + i] = u[i];
        c.inv_view[8 + i] = -f[i];
        c.inv_view[12 + i] = eye[i];
    }
    c.inv_view[15] = 1.f;
    const float th = std::tan(fovy_deg * 3.14159265f / 360.0f);
    c.inv_proj[0] = aspect * th;
    c.inv_proj[5] = -th;  // the reference flips y (projection[1][1] *= -1)
    c.inv_proj[11] = -10.f;
    c.inv_proj[14] = -1.f;
    c.inv_proj[15] = 10.f;
    c.frame[0] = frame;
    return c;
}

#define CK(x)                                                                   \
    do {                                                                        \
        cudaError_t e_ = (x);                                                   \
        if (e_ != cudaSuccess) {                                                \
            std::fprintf(stderr, "%s: %s\n", #x, cudaGetErrorString(e_));       \
            return 2;                                                           \
        }                                                                       \
    } while (0)

int main() {
    const uint32_t W = 96, H = 64;
    Mesh ico = icosahedron(), ground = quad(10.f);
    Scene s;
    s._materials.resize(3);
    s._materials[0].diffuseColor[0] = 0.8f; s._materials[0].roughnessFactor = 0.7f; s._materials[0].metallicFactor = 0.f;
    s._materials[1].shadingModel = 3; s._materials[1].roughnessFactor = 0.1f;  // mirror
    s._materials[2].diffuseColor[2] = 0.3f; s._materials[2].roughnessFactor = 0.5f; s._materials[2].metallicFactor = 1.f;
    Object g; g.mesh = &ground; g.materialIdx = 0;
    s._entities.push_back(g);
    for (int i = 0; i < 3; i++) {
        Object o; o.mesh = &ico; o.materialIdx = i % 3;
        translate_scale(o.m_matrix, -2.f + 2.f * i, 1.f, 0.5f * i, 0.8f);
        s._entities.push_back(o);
    }
    Light pl; pl.position[0] = 2; pl.position[1] = 6; pl.position[2] = 2; pl.intensity = 20.f; pl.radius = 0.2f;
    Light dl; dl.type = DIRECTIONAL_LIGHT; dl.position[0] = 0.3f; dl.position[1] = 1.f; dl.position[2] = 0.2f;
    dl.intensity = 1.f;
    s._lights = {pl, dl};

    const float eye[3] = {0.f, 4.f, 10.f};
    int fails = 0;
    try {
        HybridRenderer r(0);
        r._samples = 4;
        r.rng_mode = HY_RNG_DECORRELATED;
        r.max_recursion = 2;
        r.load_data_to_gpu(s);
        HyBvhStats bs = r.create_acceleration_structures();
        if (bs.num_tris != 2 + 3 * 20) { std::fprintf(stderr, "triangles %u\n", bs.num_tris); return 1; }
        // a small one-level structure fits in L2: shadow rays walk far first
        if (r.anyhit_order() != HY_ANYHIT_FAR_FIRST) { std::fprintf(stderr, "any-hit order\n"); return 1; }

        // the same inputs through the C ABI directly
        HyCtx* raw = nullptr;
        check(hy_create(&raw, nullptr), "hy_create");
        {
            std::vector<HyVertex> v(ground.vertices);
            v.insert(v.end(), ico.vertices.begin(), ico.vertices.end());
            std::vector<uint32_t> idx(ground.indices);
            idx.insert(idx.end(), ico.indices.begin(), ico.indices.end());
            std::vector<HyPrimitive> prims;
            std::vector<float> xf;
            for (size_t e = 0; e < s._entities.size(); e++) {
                HyPrimitive p;
                p.first_index = e == 0 ? 0 : 6;
                p.index_count = e == 0 ? 6 : 60;
                p.vertex_offset = e == 0 ? 0 : 4;
                p.material_id = (uint32_t)s._entities[e].materialIdx;
                p.transform_id = p.instance_id = (uint32_t)e;
                prims.push_back(p);
                xf.insert(xf.end(), s._entities[e].m_matrix, s._entities[e].m_matrix + 16);
            }
            check(hy_scene_set_geometry(raw, v.data(), (uint32_t)v.size(), idx.data(), (uint32_t)idx.size(),
                                        prims.data(), (uint32_t)prims.size(), xf.data(), (uint32_t)xf.size() / 16),
                  "geometry");
            std::vector<HyMaterial> m;
            for (size_t i = 0; i < s._materials.size(); i++) m.push_back(s._materials[i].materialToShader((int)i));
            check(hy_scene_set_materials(raw, m.data(), (uint32_t)m.size()), "materials");
            HyLight l[2] = {pl.toUbo(), dl.toUbo()};
            check(hy_scene_set_lights(raw, l, 2), "lights");
            check(hy_bvh_build(raw, nullptr), "build");
        }

        float* planes[6];
        const size_t npx = (size_t)W * H;
        for (int p = 0; p < 6; p++) CK(cudaMalloc(&planes[p], npx * 16));
        HyGBuffer gb;
        std::memset(&gb, 0, sizeof(gb));
        gb.width = W;
        gb.height = H;
        for (int p = 0; p < 6; p++) {
            gb.plane[p] = planes[p];
            gb.format[p] = p == 3 ? HY_FMT_RG32F : HY_FMT_RGBA32F;
        }
        uint8_t *hist_a, *hist_b, *out_a, *out_b;
        CK(cudaMalloc(&hist_a, npx * 2));
        CK(cudaMalloc(&hist_b, npx * 2));
        CK(cudaMemset(hist_a, 0, npx * 2));
        CK(cudaMemset(hist_b, 0, npx * 2));
        CK(cudaMalloc(&out_a, npx * 4));
        CK(cudaMalloc(&out_b, npx * 4));
        std::vector<uint8_t> ha(npx * 4), hb(npx * 4);

        float view[16] = {};
        for (int frame = 0; frame < 3; frame++) {
            const int32_t f = r.update_frame(view);  // same view every frame: 0, 1, 2
            if (f != frame) { std::fprintf(stderr, "frame counter %d != %d\n", f, frame); return 1; }
            HyCamera cam = camera(eye, 60.f, (float)W / H, (float)f);
            check(hy_gbuffer_primary(r.handle(), &cam, W, H, planes), "gbuffer");
            HyStats st = r.rasterize_hybrid(gb, cam, hist_a, nullptr, out_a);
            HyPassConfig cfg = r.pass_config();
            HyAccum acc{HY_ACCUM_U8, 2, hist_b};
            check(hy_hybrid_forward(raw, &gb, &cam, &cfg, &acc, nullptr, out_b, nullptr), "forward");
            CK(cudaDeviceSynchronize());
            CK(cudaMemcpy(ha.data(), out_a, npx * 4, cudaMemcpyDeviceToHost));
            CK(cudaMemcpy(hb.data(), out_b, npx * 4, cudaMemcpyDeviceToHost));
            if (std::memcmp(ha.data(), hb.data(), npx * 4) != 0) {
                std::fprintf(stderr, "frame %d differs from the C ABI result\n", frame);
                fails++;
            }
            if (st.shadow_rays == 0) { std::fprintf(stderr, "no shadow rays\n"); fails++; }
        }
        view[0] += 1.f;
        if (r.update_frame(view) != 0) { std::fprintf(stderr, "camera move did not restart accumulation\n"); fails++; }

        // move an entity and refit
        translate_scale(s._entities[2].m_matrix, 0.5f, 1.5f, -1.f, 1.2f);
        r.update_tlas(s);
        HyCamera cam = camera(eye, 60.f, (float)W / H, 0.f);
        check(hy_gbuffer_primary(r.handle(), &cam, W, H, planes), "gbuffer after refit");
        r.rasterize_hybrid(gb, cam, hist_a, nullptr, out_a);
        r.synchronize();

        // the two-level structure (BLAS per mesh, TLAS over the entities) renders the
        // same frame through the adapter and through the C ABI, before and after a
        // TLAS update
        {
            r.load_data_to_gpu(s);
            HyBvhStats b2 = r.create_acceleration_structures(true);
            HyBvhLayout lay;
            check(hy_bvh_layout(r.handle(), &lay), "layout");
            if (!lay.two_level || lay.num_instances != 4 || lay.num_blas != 2 || b2.num_tris != 2 + 3 * 20) {
                std::fprintf(stderr, "two-level layout %u %u %u\n", lay.two_level, lay.num_instances, lay.num_blas);
                fails++;
            }
            std::vector<float> xf;
            for (const Object& o : s._entities) xf.insert(xf.end(), o.m_matrix, o.m_matrix + 16);
            check(hy_bvh_refit(raw, xf.data(), (uint32_t)s._entities.size()), "raw refit");
            check(hy_bvh_build_instanced(raw, nullptr), "raw two-level build");
            for (int step = 0; step < 2; step++) {
                if (step == 1) {
                    translate_scale(s._entities[3].m_matrix, 1.f, 2.f, 0.f, 0.6f);
                    r.update_tlas(s);
                    xf.clear();
                    for (const Object& o : s._entities) xf.insert(xf.end(), o.m_matrix, o.m_matrix + 16);
                    check(hy_bvh_refit(raw, xf.data(), (uint32_t)s._entities.size()), "raw TLAS update");
                }
                HyCamera c2 = camera(eye, 60.f, (float)W / H, 1.f);
                check(hy_gbuffer_primary(r.handle(), &c2, W, H, planes), "gbuffer two-level");
                CK(cudaMemset(hist_a, 0, npx * 2));
                CK(cudaMemset(hist_b, 0, npx * 2));
                r.rasterize_hybrid(gb, c2, hist_a, nullptr, out_a);
                HyPassConfig cfg = r.pass_config();
                HyAccum acc{HY_ACCUM_U8, 2, hist_b};
                check(hy_hybrid_forward(raw, &gb, &c2, &cfg, &acc, nullptr, out_b, nullptr), "forward two-level");
                CK(cudaDeviceSynchronize());
                CK(cudaMemcpy(ha.data(), out_a, npx * 4, cudaMemcpyDeviceToHost));
                CK(cudaMemcpy(hb.data(), out_b, npx * 4, cudaMemcpyDeviceToHost));
                if (std::memcmp(ha.data(), hb.data(), npx * 4) != 0) {
                    std::fprintf(stderr, "two-level frame %d differs from the C ABI result\n", step);
                    fails++;
                }
            }
        }

        // errors come back as exceptions with the C code
        try {
            Scene bad = s;
            bad._entities[1].materialIdx = 7;
            r.load_data_to_gpu(bad);
            r.create_acceleration_structures();
            r.rasterize_hybrid(gb, cam, hist_a, nullptr, out_a);
            std::fprintf(stderr, "a missing material was accepted\n");
            fails++;
        } catch (const Error& e) {
            if (e.code() != HY_ERR_INVALID_ARG) { std::fprintf(stderr, "unexpected code %d\n", e.code()); fails++; }
        }
        for (int p = 0; p < 6; p++) cudaFree(planes[p]);
        cudaFree(hist_a); cudaFree(hist_b); cudaFree(out_a); cudaFree(out_b);
        hy_destroy(raw);
    } catch (const Error& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    if (fails) return 1;
    std::printf("adapter OK\n");
    return 0;
}
