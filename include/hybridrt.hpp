/* C++ host side of libhybridrt: the reference renderer's scene types and the
 * hybrid part of its Renderer, over the C ABI of hybridrt.h.
 *
 *   hybridrt::Material  <- Material (src/material.h:12-37); materialToShader()
 *                          packs it like src/material.cpp:19-26
 *   hybridrt::Light     <- Light (src/entity.h:56-73); toUbo() packs uboLight
 *                          like src/vk_engine.cpp:146-164
 *   hybridrt::Mesh      <- Mesh vertices/indices (src/vk_mesh.h)
 *   hybridrt::Object    <- Object (src/entity.h:38-54): mesh, materialIdx, m_matrix
 *   hybridrt::Scene     <- Scene (src/scene.h:7-23): _entities, _lights, plus the
 *                          material list (Material::_materials)
 *   hybridrt::HybridRenderer <- the hybrid path of Renderer (src/renderer.h):
 *       load_data_to_gpu()          Renderer::load_data_to_gpu + the per-entity
 *                                   buffers of create_hybrid_descriptors
 *                                   (src/renderer.cpp:1477-1530, 3015-3048)
 *       create_acceleration_structures()
 *                                   create_bottom/top_acceleration_structure
 *                                   (src/renderer.cpp:1643-1688)
 *       update_lights()             the uboLight refresh of VulkanEngine::update
 *                                   (src/vk_engine.cpp:146-164)
 *       update_tlas()               the per-frame TLAS rebuild
 *                                   (src/vk_engine.cpp:172-187), as a refit
 *       rasterize_hybrid()          the shadow / denoise / hybrid submissions of
 *                                   Renderer::rasterize_hybrid (src/renderer.cpp:559-580)
 * Header-only; link libhybridrt.  Errors throw hybridrt::Error. */
#ifndef HYBRIDRT_HPP
#define HYBRIDRT_HPP

#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "hybridrt.h"

namespace hybridrt {

class Error : public std::runtime_error {
public:
    Error(int code, const std::string& what)
        : std::runtime_error(what + ": " + hy_error_string(code)), code_(code) {}
    int code() const { return code_; }

private:
    int code_;
};

inline void check(int rc, const char* what) {
    if (rc != HY_OK) throw Error(rc, what);
}

enum LightType { DIRECTIONAL_LIGHT = 0, POINT_LIGHT = 1, SPOT_LIGHT = 2 };  // src/entity.h:6-10

struct Material {
    int shadingModel = 0;                     // 0 PBR, 3 mirror, 4 glass (hybridHit.rchit)
    float diffuseColor[4] = {1, 1, 1, 1};
    float metallicFactor = 1.f;
    float roughnessFactor = 1.f;
    float ior = 1.f;
    int diffuseTexture = -1, metallicRoughnessTexture = -1, emissiveTexture = -1, normalTexture = -1;

    // GPUMaterial: (diffuse.rgb, ior), texture ids, (shadingModel, metallic, roughness, index)
    HyMaterial materialToShader(int index) const {
        HyMaterial m;
        m.diffuse[0] = diffuseColor[0];
        m.diffuse[1] = diffuseColor[1];
        m.diffuse[2] = diffuseColor[2];
        m.diffuse[3] = ior;
        m.textures[0] = (float)diffuseTexture;
        m.textures[1] = (float)normalTexture;
        m.textures[2] = (float)emissiveTexture;
        m.textures[3] = (float)metallicRoughnessTexture;
        m.smr[0] = (float)shadingModel;
        m.smr[1] = metallicFactor;
        m.smr[2] = roughnessFactor;
        m.smr[3] = (float)index;
        return m;
    }
};

struct Light {
    LightType type = POINT_LIGHT;
    float color[3] = {1, 1, 1};
    float position[3] = {0, 0, 0};  // a directional light's direction
    float intensity = 1000.f;
    float maxDistance = 500.f;
    float radius = 1.f;

    HyLight toUbo() const {
        HyLight l;
        std::memset(&l, 0, sizeof(l));
        for (int i = 0; i < 3; i++) { l.pos[i] = position[i]; l.color[i] = color[i]; }
        l.pos[3] = type == DIRECTIONAL_LIGHT ? -1.f : maxDistance;
        l.color[3] = intensity;
        l.radius = radius;
        return l;
    }
};

struct Mesh {
    std::vector<HyVertex> vertices;
    std::vector<uint32_t> indices;
};

struct Object {
    const Mesh* mesh = nullptr;
    int materialIdx = 0;
    float m_matrix[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};  // column-major
};

struct Scene {
    std::vector<Object> _entities;
    std::vector<Light> _lights;
    std::vector<Material> _materials;
    std::vector<uint8_t> skybox_rgba8, irradiance_rgba8;  // equirect maps (miss.rmiss / irradiance)
    uint32_t skybox_w = 0, skybox_h = 0, irradiance_w = 0, irradiance_h = 0;
    struct Texture { std::vector<uint8_t> rgba8; uint32_t width = 0, height = 0; };
    std::vector<Texture> _textures;  // Texture::_textures in load order; Material::*Texture index it
};

class HybridRenderer {
public:
    explicit HybridRenderer(int device = 0, void* stream = nullptr, uint64_t max_device_bytes = 0) {
        HyCreateInfo ci;
        std::memset(&ci, 0, sizeof(ci));
        ci.device = device;
        ci.stream = stream;
        ci.max_device_bytes = max_device_bytes;
        check(hy_create(&ctx_, &ci), "hy_create");
    }
    ~HybridRenderer() { hy_destroy(ctx_); }
    HybridRenderer(const HybridRenderer&) = delete;
    HybridRenderer& operator=(const HybridRenderer&) = delete;

    HyCtx* handle() const { return ctx_; }

    // samplesBuffer, MAX_RECURSION, the RNG mode, frameCountBuffer
    uint32_t _samples = 1;
    uint32_t max_recursion = 8;
    uint32_t rng_mode = HY_RNG_REFERENCE;
    int32_t _denoise_frame = 0;
    uint32_t accum_format = HY_ACCUM_U8;

    void load_data_to_gpu(const Scene& s) {
        std::vector<HyVertex> verts;
        std::vector<uint32_t> idx;
        std::vector<HyPrimitive> prims;
        std::vector<float> xf;
        std::vector<const Mesh*> seen;
        std::vector<uint32_t> vofs, iofs;
        for (size_t e = 0; e < s._entities.size(); e++) {
            const Object& o = s._entities[e];
            if (!o.mesh) throw Error(HY_ERR_INVALID_ARG, "entity without a mesh");
            size_t k = 0;
            while (k < seen.size() && seen[k] != o.mesh) k++;
            if (k == seen.size()) {  // a mesh shared by several entities is uploaded once
                seen.push_back(o.mesh);
                vofs.push_back((uint32_t)verts.size());
                iofs.push_back((uint32_t)idx.size());
                verts.insert(verts.end(), o.mesh->vertices.begin(), o.mesh->vertices.end());
                idx.insert(idx.end(), o.mesh->indices.begin(), o.mesh->indices.end());
            }
            HyPrimitive p;
            p.first_index = iofs[k];
            p.index_count = (uint32_t)o.mesh->indices.size();
            p.vertex_offset = vofs[k];
            p.material_id = (uint32_t)o.materialIdx;
            p.transform_id = (uint32_t)e;
            p.instance_id = (uint32_t)e;
            prims.push_back(p);
            xf.insert(xf.end(), o.m_matrix, o.m_matrix + 16);
        }
        check(hy_scene_set_geometry(ctx_, verts.data(), (uint32_t)verts.size(), idx.data(), (uint32_t)idx.size(),
                                    prims.data(), (uint32_t)prims.size(), xf.data(), (uint32_t)s._entities.size()),
              "hy_scene_set_geometry");
        std::vector<HyMaterial> mats;
        for (size_t i = 0; i < s._materials.size(); i++) mats.push_back(s._materials[i].materialToShader((int)i));
        check(hy_scene_set_materials(ctx_, mats.data(), (uint32_t)mats.size()), "hy_scene_set_materials");
        update_lights(s);
        if (!s.skybox_rgba8.empty())
            check(hy_scene_set_env(ctx_, 0, s.skybox_rgba8.data(), s.skybox_w, s.skybox_h), "hy_scene_set_env");
        if (!s.irradiance_rgba8.empty())
            check(hy_scene_set_env(ctx_, 1, s.irradiance_rgba8.data(), s.irradiance_w, s.irradiance_h),
                  "hy_scene_set_env");
        if (!s._textures.empty()) {
            std::vector<const uint8_t*> px;
            std::vector<uint32_t> w, h;
            for (const Scene::Texture& t : s._textures) {
                px.push_back(t.rgba8.data());
                w.push_back(t.width);
                h.push_back(t.height);
            }
            check(hy_scene_set_textures(ctx_, px.data(), w.data(), h.data(), (uint32_t)px.size()),
                  "hy_scene_set_textures");
        }
        num_lights_ = (uint32_t)s._lights.size();
    }

    // two_level: one BLAS per distinct mesh under a TLAS over the entities, as
    // the reference's BLAS/TLAS pair; otherwise one BVH over the flattened scene
    HyBvhStats create_acceleration_structures(bool two_level = false) {
        HyBvhStats st;
        if (two_level) check(hy_bvh_build_instanced(ctx_, &st), "hy_bvh_build_instanced");
        else check(hy_bvh_build(ctx_, &st), "hy_bvh_build");
        return st;
    }

    // child order of the shadow rays' any-hit walk (HY_ANYHIT_*; AUTO by default)
    void set_anyhit_order(uint32_t order) { check(hy_scene_set_anyhit_order(ctx_, order), "hy_scene_set_anyhit_order"); }
    uint32_t anyhit_order() {
        uint32_t o = 0;
        check(hy_scene_anyhit_order(ctx_, &o), "hy_scene_anyhit_order");
        return o;
    }

    void update_lights(const Scene& s) {
        std::vector<HyLight> l;
        for (const Light& x : s._lights) l.push_back(x.toUbo());
        check(hy_scene_set_lights(ctx_, l.empty() ? nullptr : l.data(), (uint32_t)l.size()), "hy_scene_set_lights");
        num_lights_ = (uint32_t)l.size();
    }

    // entities moved: new transforms, same topology
    void update_tlas(const Scene& s) {
        std::vector<float> xf;
        for (const Object& o : s._entities) xf.insert(xf.end(), o.m_matrix, o.m_matrix + 16);
        check(hy_bvh_refit(ctx_, xf.data(), (uint32_t)s._entities.size()), "hy_bvh_refit");
    }

    HyPassConfig pass_config(uint32_t flags = 0) const {
        HyPassConfig c;
        std::memset(&c, 0, sizeof(c));
        c.shadow_spp = _samples;
        c.max_bounces = max_recursion;
        c.rng_mode = rng_mode;
        c.accum_frame = _denoise_frame;
        c.flags = flags;
        return c;
    }

    // The frame counter of VulkanEngine (src/vk_engine.cpp:670-686): a view matrix
    // different from the last one restarts accumulation (frame 0), else it counts up.
    int32_t update_frame(const float view[16]) {
        if (!have_view_ || std::memcmp(view, last_view_, sizeof(last_view_)) != 0) {
            _denoise_frame = -1;
            std::memcpy(last_view_, view, sizeof(last_view_));
            have_view_ = true;
        }
        return ++_denoise_frame;
    }

    // One frame: shadow rays -> denoise accumulation -> hybrid shading at
    // _denoise_frame.  gbuffer, the history (num_lights planes of width x height)
    // and the outputs are device memory; either output may be null.  cam.frame[0]
    // seeds the per-pixel RNG (the reference passes _denoise_frame there).
    HyStats rasterize_hybrid(const HyGBuffer& gbuffer, const HyCamera& cam, void* d_denoised_history,
                             float* d_out_rgba32f, uint8_t* d_rt_image_bgra8, uint32_t flags = 0) {
        HyPassConfig cfg = pass_config(flags);
        HyAccum acc;
        acc.format = accum_format;
        acc.num_lights = num_lights_;
        acc.history = d_denoised_history;
        HyStats st;
        std::memset(&st, 0, sizeof(st));
        check(hy_hybrid_forward(ctx_, &gbuffer, &cam, &cfg, &acc, d_out_rgba32f, d_rt_image_bgra8, &st),
              "hy_hybrid_forward");
        return st;
    }

    void synchronize() { check(hy_synchronize(ctx_), "hy_synchronize"); }

private:
    HyCtx* ctx_ = nullptr;
    uint32_t num_lights_ = 0;
    float last_view_[16] = {};
    bool have_view_ = false;
};

}  // namespace hybridrt

#endif  // HYBRIDRT_HPP
