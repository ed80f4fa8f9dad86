/*
 * hybridrt.h — C ABI of the GB300-native hybrid ray-tracing pass.
 *
 * The pass replaces the three GPU submissions that VkPinut's
 * Renderer::rasterize_hybrid records after its G-buffer raster pass
 * (src/renderer.cpp:559-580):
 *
 *   shadow trace   data/shaders/shadowRaygen.rgen + shadow.rmiss   -> hy_shadow_pass
 *   denoise        data/shaders/blur.comp                          -> hy_accumulate_pass
 *   hybrid trace   data/shaders/hybridRaygen.rgen + hybridHit.rchit
 *                  + miss.rmiss                                    -> hy_shade_pass
 *   all three, fused where the data flow allows                    -> hy_hybrid_forward
 *
 * and the driver-built acceleration structures (src/renderer.cpp:1696-1865)
 * with a binary tree built on the GPU (binned SAH by default, or an LBVH) and
 * collapsed to a compressed 8-wide BVH (hy_bvh_build).
 *
 * Conventions
 *   - Every entry point returns HY_OK (0) or a negative HY_ERR_* code; no C++
 *     exception crosses this boundary.
 *   - Pointers named d_* are device pointers owned by the caller; pointers
 *     named h_* (and the scene upload arrays) are host pointers.
 *   - Work is stream-ordered on the context's stream.  Entry points that
 *     return statistics or an error status read back a 4-byte status word and
 *     so synchronise that stream.
 *   - A context is used from one host thread at a time.
 *   - Struct layouts that mirror a reference type keep its std140/std430
 *     layout so a Vulkan-side buffer can be memcpy'd straight in.
 */
#ifndef HYBRIDRT_H
#define HYBRIDRT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HY_ABI_VERSION 5

/* ---- error codes (the reference aborts through VK_CHECK, src/vk_engine.h:15-24) ---- */
enum {
    HY_OK                  = 0,
    HY_ERR_INVALID_ARG     = -1,
    HY_ERR_OOM             = -2,
    HY_ERR_CUDA            = -3,
    HY_ERR_TIMEOUT         = -4,  /* a bounded device loop ran out of its iteration budget */
    HY_ERR_STACK_OVERFLOW  = -5,  /* traversal stack exceeded its depth */
    HY_ERR_QUEUE_OVERFLOW  = -6,
    HY_ERR_NAN_INPUT       = -7,
    HY_ERR_NOT_READY       = -8,  /* scene or BVH missing */
    HY_ERR_UNSUPPORTED     = -9,
    HY_ERR_TOO_LARGE       = -10, /* input exceeds the fixed scratch of an allocation-free entry point */
    HY_ERR_BAD_INDEX       = -11  /* a traversal met a node/record index outside the structure */
};

/* device status-word bits (HyStats.error_flags) */
#define HY_STATUS_STACK_OVERFLOW 0x1u
#define HY_STATUS_TIMEOUT        0x2u
#define HY_STATUS_NAN_INPUT      0x4u
#define HY_STATUS_QUEUE_OVERFLOW 0x8u
#define HY_STATUS_BAD_INDEX      0x10u  /* a node/triangle index fell outside the structure */

typedef struct HyCtx HyCtx;

typedef struct HyCreateInfo {
    int32_t  device;            /* CUDA device ordinal */
    uint32_t flags;             /* reserved, 0 */
    void*    stream;            /* cudaStream_t to run on; NULL: the context creates its own */
    uint64_t max_device_bytes;  /* cap on context-owned device memory; 0 = no cap */
} HyCreateInfo;

/* == uboLight, src/vk_engine.h:76-80 (std140, 48 B).  pos.w = maxDistance, or -1
 *    for a directional light (src/vk_engine.cpp:146-164); color.w = intensity. */
typedef struct HyLight {
    float pos[4];
    float color[4];
    float radius;
    float _pad[3];
} HyLight;

/* == GPUMaterial, src/material.h:5-10, filled by Material::materialToShader
 *    (src/material.cpp:19-26): diffuse = (rgb, ior); textures = (diffuse,
 *    normal, emissive, metallicRoughness) texture ids or -1; smr =
 *    (shadingModel, metallic, roughness, material index). */
typedef struct HyMaterial {
    float diffuse[4];
    float textures[4];
    float smr[4];
} HyMaterial;

/* == Vertex, src/vk_mesh.h:21-33 (44 B, tightly packed). */
typedef struct HyVertex {
    float pos[3];
    float normal[3];
    float color[3];
    float uv[2];
} HyVertex;

/* One Primitive of a Node (src/vk_mesh.h:72-155).  first_index/index_count
 * address the index array; index values are relative to vertex_offset (the
 * start of the owning mesh's vertices).  material_id/transform_id are the
 * .y/.z of the per-primitive id vec4 (src/vk_mesh.cpp:521-533). */
typedef struct HyPrimitive {
    uint32_t first_index;
    uint32_t index_count;
    uint32_t vertex_offset;
    uint32_t material_id;
    uint32_t transform_id;
    uint32_t instance_id;
} HyPrimitive;

/* == RTCameraData, src/vk_engine.h:56-62 (column-major glm mat4s).
 *    frame[0] seeds the per-pixel RNG: _denoise_frame with denoise on, else 0
 *    (src/vk_engine.cpp:733). */
typedef struct HyCamera {
    float inv_view[16];
    float inv_proj[16];
    float frame[4];
} HyCamera;

/* G-buffer plane formats.  The reference's own attachments are
 * RGBA16F, RGBA16F, RGBA8, RG16F, RGBA8, RGBA8 (src/renderer.cpp:255-260). */
enum {
    HY_FMT_RGBA32F = 0,
    HY_FMT_RG32F   = 1,
    HY_FMT_RGBA16F = 2,
    HY_FMT_RG16F   = 3,
    HY_FMT_RGBA8   = 4
};

/* Plane order and encoding of geometry_shader.frag:66-76:
 *   0 (worldPos, materialIdx)  1 (N*0.5+0.5, 1)  2 albedo.rgb
 *   3 motion*0.5+0.5           4 (0, roughness, metallic)  5 emissive.rgb
 * Rows are tightly packed (pitch = width * texel size). */
typedef struct HyGBuffer {
    uint32_t    width;
    uint32_t    height;
    const void* plane[6];
    uint32_t    format[6];
} HyGBuffer;

/* Per-light shadow images.  HY_ACCUM_U8 is the reference's R8_UNORM
 * (src/renderer.cpp:1538); HY_ACCUM_F32 keeps full precision.  Light l's
 * plane starts at l * width * height elements. */
enum { HY_ACCUM_U8 = 0, HY_ACCUM_F32 = 1 };

typedef struct HyAccum {
    uint32_t format;
    uint32_t num_lights;   /* the pass shades with the scene's first num_lights lights (<= its count) */
    void*    history;      /* device, caller-owned: the reference's _denoisedImages */
} HyAccum;

/* RNG modes.  REFERENCE reproduces sampleDisk's by-value seed
 * (helpers.glsl:82-93): all samples of one pixel are the same ray, which is
 * traced once.  DECORRELATED advances the TEA/LCG stream per sample. */
enum { HY_RNG_REFERENCE = 0, HY_RNG_DECORRELATED = 1 };

#define HY_FLAG_FULL_BLUR_DISPATCH 0x1u /* also accumulate the texels the W/16 x H/16 dispatch skips */
#define HY_FLAG_NO_ACCUM           0x2u /* shade from the raw shadow images, no denoise pass */
#define HY_FLAG_COUNT_TRAVERSAL    0x4u /* count BVH nodes visited / triangles tested into HyStats */
#define HY_FLAG_NO_STATUS_SYNC     0x8u /* do not read back the status word (no host sync) */
/* Schedules of DECORRELATED shadow rays with spp >= 2.  Default: tile streams — a
 * warp takes an 8x4 tile and, light by light, its lanes walk the tile's 32 x spp
 * samples (adjacent lanes on samples of the same or a neighbouring pixel), each
 * lane without waiting for the others until the light is done. */
#define HY_FLAG_PIXEL_PARALLEL     0x10u /* one lane per pixel, lights and samples in turn */
#define HY_FLAG_RAY_POOL           0x20u /* the samples of a pixel-light from a per-warp ray pool that refills
                                            each lane as soon as its ray ends */
#define HY_FLAG_LANE_GROUPS        0x40u /* the samples of a pixel-light on a fixed group of adjacent lanes,
                                            which waits for its slowest sample before the next pixel-light */
/* GGX-sampled reflection ray for mirror texels (shading model 3: the benchmark scenes give it to
 * materials with roughness < 0.3).  The reference reflects perfectly (hybridRaygen.rgen:125); with
 * this flag the first bounce direction is reflect(-V, H) around a microfacet normal H drawn with
 * density D(H) (N.H), D the reference's DistributionGGX (helpers.glsl:33-45, alpha = roughness^2
 * from G-buffer plane 4), from two draws of the texel's TEA/LCG stream (random.glsl:3-33) made
 * before the bounce loop; a direction below the surface falls back to the mirror direction.  The
 * later bounces and everything else are the reference's. */
#define HY_FLAG_GGX_REFLECTION     0x80u

typedef struct HyPassConfig {
    uint32_t shadow_spp;    /* samplesBuffer.samples (1..64, src/renderer.cpp:656) */
    uint32_t max_bounces;   /* MAX_RECURSION (helpers.glsl:8): 8 */
    uint32_t rng_mode;      /* HY_RNG_* */
    int32_t  accum_frame;   /* frameCountBuffer = _denoise_frame (src/vk_engine.cpp:722) */
    uint32_t flags;         /* HY_FLAG_* */
    uint32_t block_size;    /* threads per block: the single-view passes take 32..128 in steps of 32
                               (0 = 128); a batch's tuning 64, 128 or 256 (0 = 256) */
    uint32_t queue_chunk;   /* work items fetched per warp from the ray queue; 0 = default */
    uint32_t stack_depth;   /* short traversal stack: the first stack_depth entries of each lane's
                               stack in shared memory, deeper ones in local memory.  Single-view
                               tile-stream shadow kernel: 0 (default, all local; measured equal)
                               or 8; a batch's tuning: 0, 8, 16 or 32; other values:
                               HY_ERR_UNSUPPORTED / HY_ERR_INVALID_ARG */
    uint32_t group_lanes;   /* DECORRELATED shadow rays: lanes per pixel-light group (power of two,
                               2..32, each lane traces spp / group_lanes samples in turn);
                               0 = the next power of two >= spp */
    uint32_t min_blocks;    /* shadow-kernel variant: compiled for 5 (96 registers) or 8 (64 registers)
                               resident 128-thread blocks per SM, the lane-group kernel also for 6
                               and 7, a batch's tile-stream kernel for 6 (80) and 8 (64);
                               0 = 6 for the lane-group kernel, 8 otherwise */
    uint32_t visits_per_round; /* BVH node visits a shadow lane makes between two scheduling rounds
                                  of the persistent shadow kernels (1..16; a lane whose ray ends
                                  early waits for the round); 0 = 4 (tile streams: 8) */
} HyPassConfig;

typedef struct HyStats {
    uint64_t shadow_rays;       /* rays traced by the shadow pass */
    uint64_t reflection_rays;   /* closest-hit bounce rays of mirror/glass pixels */
    uint64_t hit_shadow_rays;   /* shadow rays cast from bounce hit points */
    uint64_t nodes_visited;     /* with HY_FLAG_COUNT_TRAVERSAL */
    uint64_t tris_tested;       /* with HY_FLAG_COUNT_TRAVERSAL */
    uint32_t error_flags;       /* HY_STATUS_* */
    uint32_t _pad;
} HyStats;

typedef struct HyBvhStats {
    uint32_t num_tris;
    uint32_t num_bvh2_nodes;    /* internal nodes of the binary LBVH */
    uint32_t num_bvh8_nodes;
    uint32_t depth;             /* BVH8 levels */
    float    build_ms;          /* device time of the whole build */
    float    scene_lo[3];
    float    scene_hi[3];
} HyBvhStats;

/* Ray / hit records of hy_trace_rays: 32 B in, 16 B out.  tri_id is the
 * triangle's global index (primitives in upload order, index_count/3 each);
 * b1/b2 are the barycentrics of vertices 1/2 (Vulkan's hit attributes). */
typedef struct HyRay { float org[3]; float tmin; float dir[3]; float tmax; } HyRay;
typedef struct HyHit { float t; uint32_t tri_id; float b1; float b2; } HyHit;
#define HY_NO_HIT 0xffffffffu

/* ---- context ---- */
int         hy_create(HyCtx** out, const HyCreateInfo* info);
void        hy_destroy(HyCtx* ctx);
const char* hy_error_string(int code);
int         hy_get_abi_version(void);
int         hy_synchronize(HyCtx* ctx);
/* Allocation hook for fault-injection tests: the next `n`-th device
 * allocation made by the context fails with HY_ERR_OOM (0 disables). */
int         hy_debug_fail_alloc_after(HyCtx* ctx, uint32_t n);
/* Per-ray limits of every BVH walk of the context's passes, lowered for
 * failure-detection tests: a ray that makes more than max_node_visits node
 * visits stops and the call returns HY_ERR_TIMEOUT; one whose traversal stack
 * would grow past max_stack_depth entries stops and the call returns
 * HY_ERR_STACK_OVERFLOW.  Both limits are counters tested before the step
 * they guard, so running out stops the ray and nothing else: the context
 * stays usable.  0 restores the built-in limit (2^22 visits, 64 entries);
 * max_stack_depth > 64 is HY_ERR_INVALID_ARG.  The reference's policy for a
 * failed GPU call is to abort the process (VK_CHECK, src/vk_engine.h:15-24). */
int         hy_debug_set_traversal_limits(HyCtx* ctx, uint32_t max_node_visits, uint32_t max_stack_depth);

/* ---- scene upload (host arrays; replaces Renderer::load_data_to_gpu,
 *      src/renderer.cpp:1477-1530, and the per-entity rtVertexAttribute /
 *      index / id buffers of create_hybrid_descriptors, :3015-3048) ---- */
int hy_scene_set_geometry(HyCtx* ctx,
                          const HyVertex* verts, uint32_t num_verts,
                          const uint32_t* indices, uint32_t num_indices,
                          const HyPrimitive* prims, uint32_t num_prims,
                          const float* transforms /* column-major mat4s */, uint32_t num_transforms);
int hy_scene_set_materials(HyCtx* ctx, const HyMaterial* mats, uint32_t num_mats);
int hy_scene_set_lights(HyCtx* ctx, const HyLight* lights, uint32_t num_lights);
/* slot 0 = sky (miss.rmiss, skybox[0]), slot 1 = irradiance (environmentTexture[1]) */
int hy_scene_set_env(HyCtx* ctx, int slot, const uint8_t* rgba8, uint32_t width, uint32_t height);
/* Material textures: Texture::_textures in load order (src/vk_textures.cpp, R8G8B8A8_UNORM,
 * sampled NEAREST / REPEAT as by the sampler of src/renderer.cpp:3059); a material's
 * textures[0] (diffuse), [2] (emissive) and [3] (metallic-roughness) index this list
 * (-1: none), as hybridHit.rchit:63-65, closesthit.rchit:76-78 and
 * geometry_shader.frag:56-59 read them.  Replaces the binding-7 texture array of
 * create_hybrid_descriptors (src/renderer.cpp:3050-3069).  A pass whose materials name a
 * texture past the list returns HY_ERR_INVALID_ARG. */
int hy_scene_set_textures(HyCtx* ctx, const uint8_t* const* rgba8, const uint32_t* widths,
                          const uint32_t* heights, uint32_t count);

/* ---- acceleration structure (replaces buildBlas/buildTlas) ---- */
/* Algorithm of the binary tree that hy_bvh_build, hy_bvh_build_instanced (each
 * BLAS and the TLAS) and the TLAS rebuild of hy_bvh_refit collapse into 8-wide
 * nodes.  Both start from the triangles sorted by the 30-bit Morton code of
 * their box centroids.
 *   HY_BUILD_SAH  (default) top down: each range of two or more triangles is
 *                 split where the surface area heuristic over 32 bins per axis
 *                 of its centroid bounds is lowest (sum over both sides of box
 *                 area x triangles), the sides stably partitioned; a range whose
 *                 centroids coincide is split at its middle.  Fewer node visits
 *                 per ray (about 30 % on a 1.5 M-triangle terrain-and-spheres
 *                 scene) for a longer build.
 * Either tree is collapsed into 8-wide nodes by a surface-area-heuristic
 * program over slot budgets (how many of a node's 8 child slots each subtree
 * gets).
 *   HY_BUILD_LBVH Karras's radix tree over the Morton keys: the fastest build.
 * The 8-wide node format, the traversal and every result but node and
 * triangle counts are the same.  The mode applies from the next build. */
enum { HY_BUILD_SAH = 0, HY_BUILD_LBVH = 1 };
int hy_scene_set_build_mode(HyCtx* ctx, uint32_t mode);
int hy_bvh_build(HyCtx* ctx, HyBvhStats* stats);
/* Re-transforms the triangles with new transforms and refits every node box
 * (topology kept): the per-frame TLAS update of src/vk_engine.cpp:172-187. */
int hy_bvh_refit(HyCtx* ctx, const float* transforms, uint32_t num_transforms);
/* Copies the built structure out for topology checks.  Any pointer may be
 * NULL.  order: num_tris triangle ids in leaf order; morton: the Morton code
 * of each (sorted for HY_BUILD_LBVH); bvh2: 10 words per internal node (left,
 * right, first, last, lo[3], hi[3]; a child with bit 31 set is the leaf at
 * that position of order; LBVH: node i is Karras's node i, the root 0; SAH:
 * the node splitting [first, last] before position m is node m - 1, the root
 * the node with first 0 and last num_tris - 1); bvh8: 20 words
 * per node; tris: 12 words per triangle.  Two-level structure: bvh8 and tris
 * only (HyBvhLayout.num_nodes / num_records entries); morton, order and bvh2
 * must be NULL. */
int hy_bvh_download(HyCtx* ctx, uint32_t* morton, uint32_t* order, uint32_t* bvh2,
                    uint32_t* bvh8, float* tris);

/* Two-level structure, the driver's BLAS/TLAS split (one BLAS per primitive,
 * src/vk_mesh.cpp:424-470 + buildBlas, src/renderer.cpp:1696-1753; one TLAS
 * instance per primitive, src/vk_mesh.cpp:472-492 + buildTlas,
 * src/renderer.cpp:1757-1865).  One BLAS per distinct mesh (primitives with
 * equal first_index, index_count and vertex_offset share it), built over the
 * mesh's object-space triangles; a TLAS over one instance per primitive with
 * triangles, whose box is its mesh box through its transform.  Rays enter an
 * instance through its world-to-object transform (t is the same in both
 * frames; hit ids stay global triangle ids).  hy_bvh_refit then rebuilds the
 * instance records and the TLAS only (the per-frame TLAS update of
 * src/vk_engine.cpp:172-187).  HY_FLAG_RAY_POOL, and HY_FLAG_LANE_GROUPS in a
 * batch's tuning, return HY_ERR_UNSUPPORTED on it. */
int hy_bvh_build_instanced(HyCtx* ctx, HyBvhStats* stats);

typedef struct HyBvhLayout {
    uint32_t two_level;      /* 0: one BVH8 over world-space triangles */
    uint32_t num_nodes;      /* 80-byte nodes (two-level: TLAS region first, then each BLAS) */
    uint32_t num_records;    /* 48-byte leaf records (two-level: TLAS instance entries first) */
    uint32_t num_instances;  /* two-level: TLAS instances */
    uint32_t num_blas;       /* two-level: distinct meshes */
    uint32_t tlas_region;    /* two-level: nodes and records reserved for the TLAS (= instances) */
    uint32_t tlas_nodes;     /* two-level: nodes the TLAS uses (the rest of its region is zero) */
    uint32_t depth;          /* BVH8 levels (two-level: TLAS + deepest BLAS) */
} HyBvhLayout;
int hy_bvh_layout(HyCtx* ctx, HyBvhLayout* out);
/* Two-level only.  records: 16 words per instance (world->object rows
 * 3 x (m0, m1, m2, t), then BLAS root node, first global triangle, primitive,
 * 0 as uint32 bits); boxes: 6 floats per instance (the TLAS box, lo then hi). */
int hy_bvh_download_instances(HyCtx* ctx, float* records, float* boxes);

/* Child order of any-hit traversal (shadow rays, hy_trace_rays with any_hit).
 * Closest-hit rays always walk a node's children front to back (rank = slot
 * ^ the ray's near octant).  Any-hit rays return the same occlusion either
 * way, but the order sets how soon they meet an occluder and which nodes
 * they touch:
 *   HY_ANYHIT_FAR_FIRST  back to front (from the ray's far end): a shadow ray
 *                        starts on a surface and meets its occluders away
 *                        from it, so fewer node visits;
 *   HY_ANYHIT_NEAR_FIRST front to back: a tile's rays to successive lights
 *                        start at the same nodes, the better order when the
 *                        structure does not fit in L2 and node fetches go to
 *                        DRAM;
 *   HY_ANYHIT_AUTO       (default) far first for a one-level structure whose
 *                        nodes and leaf records fit in the device's L2, near
 *                        first otherwise (two-level structures included).
 * The order is a property of the scene: it applies to every pass on it,
 * batched views included.  hy_scene_anyhit_order reports the order a pass
 * uses now (HY_ERR_NOT_READY without a built structure).  Which triangle an
 * any-hit query reports can differ between the orders; whether it hits
 * cannot. */
enum { HY_ANYHIT_AUTO = 0, HY_ANYHIT_FAR_FIRST = 1, HY_ANYHIT_NEAR_FIRST = 2 };
int hy_scene_set_anyhit_order(HyCtx* ctx, uint32_t order);
int hy_scene_anyhit_order(HyCtx* ctx, uint32_t* resolved);

/* ---- ray queries (any_hit: TerminateOnFirstHit semantics) ---- */
int hy_trace_rays(HyCtx* ctx, const HyRay* d_rays, uint32_t num_rays, int any_hit,
                  HyHit* d_hits, HyStats* stats);

/* ---- G-buffer producer: primary rays (raygen.rgen:29-40 camera model)
 *      writing the geometry_shader.frag encoding into RGBA32F/RG32F planes ---- */
int hy_gbuffer_primary(HyCtx* ctx, const HyCamera* cam, uint32_t width, uint32_t height,
                       float* d_planes[6]);

/* ---- the pass ---- */
/* shadowRaygen.rgen: writes one shadow image per light into d_shadow
 * (format accum_format, num_lights planes). */
int hy_shadow_pass(HyCtx* ctx, const HyGBuffer* gb, const HyCamera* cam,
                   const HyPassConfig* cfg, uint32_t accum_format, void* d_shadow, HyStats* stats);
/* blur.comp: folds the shadow images into the history (in place). */
int hy_accumulate_pass(HyCtx* ctx, const HyGBuffer* gb, const HyPassConfig* cfg,
                       const void* d_shadow, HyAccum* accum);
/* hybridRaygen.rgen + hybridHit.rchit + miss.rmiss: shades from the
 * accumulated shadow images.  d_out_rgba32f (W*H*4 floats) and
 * d_out_bgra8 (the reference's B8G8R8A8 _rtImage) may each be NULL. */
int hy_shade_pass(HyCtx* ctx, const HyGBuffer* gb, const HyCamera* cam,
                  const HyPassConfig* cfg, const HyAccum* accum,
                  float* d_out_rgba32f, uint8_t* d_out_bgra8, HyStats* stats);
/* The three passes in order, fused where the data flow allows. */
int hy_hybrid_forward(HyCtx* ctx, const HyGBuffer* gb, const HyCamera* cam,
                      const HyPassConfig* cfg, HyAccum* accum,
                      float* d_out_rgba32f, uint8_t* d_out_bgra8, HyStats* stats);
/* Same, with host G-buffer planes and host outputs: the planes are copied in
 * and the outputs copied back inside the call (pinned host memory makes the
 * copies asynchronous).  The history stays on the device (accum). */
int hy_hybrid_forward_host(HyCtx* ctx, const HyGBuffer* h_gb, const HyCamera* cam,
                           const HyPassConfig* cfg, HyAccum* accum,
                           float* h_out_rgba32f, uint8_t* h_out_bgra8, HyStats* stats);

/* ---- path-traced mode (replaces Renderer::raytrace, src/renderer.cpp:465-501:
 *      raygen.rgen + closesthit.rchit + miss.rmiss + shadow.rmiss) ----
 * A camera ray through the centre of every pixel of a width x height image,
 * followed for up to cfg->max_bounces segments (MAX_RECURSION) through mirror
 * and glass hits; at each hit every light with N.L > 0 gets cfg->shadow_spp
 * shadow rays (samplesBuffer.samples; one ray in REFERENCE mode, where
 * sampleDisk's by-value seed repeats it).  The frame's colour goes to
 * d_out_rgba32f (W*H*4 floats, may be NULL) and into d_image_bgra8, the
 * reference's B8G8R8A8 _rtImage (W*H*4 bytes, may be NULL): stored when
 * cam->frame[0] < 0, else mixed with the image's 8-bit content with weight
 * 1 / (1 + frame) (raygen.rgen:69-80).  cam->frame[0] also seeds the RNG. */
int hy_pathtrace_pass(HyCtx* ctx, const HyCamera* cam, uint32_t width, uint32_t height, const HyPassConfig* cfg,
                      uint8_t* d_image_bgra8, float* d_out_rgba32f, HyStats* stats);

/* ---- post (replaces the post pass, postFragment.frag:9-20, drawn by
 *      Renderer::build_post_command_buffers, src/renderer.cpp:2875) ----
 * rgb = pow(max(rgb, 0.001), 1/2.2) per pixel, alpha kept, into the B8G8R8A8
 * d_out_bgra8 (UNORM; a swapchain with an sRGB format would encode again on
 * write).  The input is the pass's 8-bit image d_in_bgra8 (the reference's
 * _rtImage) or, when that is NULL, the float image d_in_rgba32f. */
int hy_post_resolve(HyCtx* ctx, uint32_t width, uint32_t height, const uint8_t* d_in_bgra8,
                    const float* d_in_rgba32f, uint8_t* d_out_bgra8);

/* ---- per-kernel timing (the reference's only timer is the frame rate it
 *      prints, src/renderer.cpp:614) ----
 * While enabled, every kernel launch of the context's passes is bracketed by
 * CUDA events on the context's stream (no host synchronisation).
 * hy_profile_read waits for the stream, reports per kernel its launch count
 * and summed device time, and clears the record; at most 4096 launches are
 * kept between reads.  Enabling clears the record too. */
typedef struct HyKernelTime {
    char     kernel[40];
    uint32_t launches;
    float    total_ms;
} HyKernelTime;
int hy_profile_enable(HyCtx* ctx, int enable);
int hy_profile_read(HyCtx* ctx, HyKernelTime* out, uint32_t capacity, uint32_t* count);

/* ---- differentiation (no counterpart in the reference, whose passes are
 *      forward only) ----
 *
 * hy_hybrid_backward is the adjoint of hy_shade_pass (hybridRaygen.rgen +
 * hybridHit.rchit + miss.rmiss): given dLoss/dImage for the image that
 * hy_shade_pass / hy_hybrid_forward produced from the same G-buffer, camera,
 * configuration and shadow images (accum->history, exactly what the shading
 * read), it returns the gradient of the loss with respect to
 *   materials, HY_GRAD_MATERIAL_PARAMS floats each: diffuse[0..2] (the
 *     shaders linearise it with pow(., 2.2)), roughness (smr[2]),
 *     metallic (smr[1]);
 *   lights, HY_GRAD_LIGHT_PARAMS floats each: pos[0..2] (a directional
 *     light's direction), intensity (color[3]).
 * Visibility is held fixed: the shadow images, which triangle each bounce ray
 * hits and the bounce-hit shadow rays' outcomes are constants (edge and
 * penumbra terms are not differentiated).  Branches of the shaders that
 * switch on a light's side of the surface take the side they took in the
 * forward pass.  The G-buffer's albedo (plane 2) and roughness/metallic
 * (plane 4 .y/.z) are taken to be the material's own values at the texel's
 * material index (plane 0 .w), as hy_gbuffer_primary writes them; their
 * gradients go to that material.  Values a texture supplies (textures[0] for
 * the diffuse colour, textures[3] for roughness/metallic) are constants and
 * get no gradient.  Bounce rays and bounce-hit shadow rays are re-traced
 * (nothing is stored by the forward pass).
 *
 * d_grad_rgba32f: device, W*H*4 floats laid out like hy_shade_pass's
 * d_out_rgba32f (alpha ignored).  d_grad_materials (num_mats*5) and
 * d_grad_lights (num_lights*4, the scene's light count; lights past
 * accum->num_lights get 0) are device arrays, overwritten; either may be
 * NULL.  cfg->max_bounces <= HY_GRAD_MAX_BOUNCES and accum->num_lights <=
 * HY_GRAD_MAX_LIGHTS, else HY_ERR_UNSUPPORTED.  Sums over pixels use float
 * atomics, so the last bits may vary from run to run. */
#define HY_GRAD_MATERIAL_PARAMS 5
#define HY_GRAD_LIGHT_PARAMS 4
#define HY_GRAD_MAX_BOUNCES 8
#define HY_GRAD_MAX_LIGHTS 64
int hy_hybrid_backward(HyCtx* ctx, const HyGBuffer* gb, const HyCamera* cam, const HyPassConfig* cfg,
                       const HyAccum* accum, const float* d_grad_rgba32f, float* d_grad_materials,
                       float* d_grad_lights, HyStats* stats);

/* ---- batches: many views of several scenes in one persistent launch ----
 *
 * Each view is one hybrid pass (its own G-buffer, camera, configuration,
 * history and outputs) over one of the scene contexts in `scenes` (contexts
 * that hold a scene and a built BVH; `ctx` itself may be one of them).  The
 * shadow rays of all views run in one persistent launch over a global queue
 * of (view, 8x4 tile) units, then all views are shaded in one launch; views
 * on their reset frame (accum_frame <= 0) get blur.comp's reset branch in
 * between.  By default the sequence is captured as a CUDA graph the first
 * time a batch of this shape (view count, tile count, reset views, tuning) is
 * seen and replayed afterwards; the per-view parameters travel through a
 * pinned table copied in by the graph, so cameras, frames and buffers may
 * change between replays.  Runs on ctx's stream; all contexts must share
 * its device.  tuning (NULL: defaults) selects the launch shape of the shadow
 * kernel: queue_chunk (tiles per queue pull, 1..1024), block_size (threads per
 * block: 64, 128 or 256), min_blocks (register cap as resident 128-thread
 * blocks per SM: 6 or 8, i.e. 80 or 64 registers) and stack_depth (entries of
 * each lane's traversal stack in shared memory: 0, 8, 16 or 32); flags may
 * hold HY_FLAG_LANE_GROUPS (the lane-group kernel, 128 threads, no shared
 * stack) and HY_FLAG_COUNT_TRAVERSAL.  Counting launches and batches holding
 * a two-level scene run one shape (128 threads, no shared stack); other
 * shapes return HY_ERR_UNSUPPORTED for them.  The shape changes speed, never
 * the images. */
typedef struct HyView {
    uint32_t     scene;        /* index into scenes[] */
    uint32_t     _pad;
    HyGBuffer    gbuffer;      /* device planes */
    HyCamera     camera;
    HyPassConfig config;       /* the view's spp, bounces, RNG mode, accumulation frame, flags */
    HyAccum      accum;        /* the view's history (device) */
    float*       out_rgba32f;  /* device, may be NULL */
    uint8_t*     out_bgra8;    /* device, may be NULL */
} HyView;

#define HY_BATCH_NO_GRAPH       0x1u /* enqueue the launches directly instead of replaying a captured graph */
#define HY_BATCH_NO_STATUS_SYNC 0x2u /* return without reading back the status word (stats must be NULL) */
#define HY_BATCH_MAX_VIEWS 1024u

int hy_batch_forward(HyCtx* ctx, HyCtx* const* scenes, uint32_t num_scenes, const HyView* views,
                     uint32_t num_views, uint32_t batch_flags, const HyPassConfig* tuning, HyStats* stats);

/* Launch-shape autotuner of hy_batch_forward (the tuning space of the
 * reference's one-view-per-frame renderer has no counterpart): times the batch
 * under candidate shapes, one axis at a time (queue chunk {1..32 tiles = 32..1024
 * pixels}, block size {64, 128, 256}, register cap {6, 8}, shared stack entries
 * {0, 8, 16, 32}) with the others at their best so far, each shape as the
 * fastest of `reps` (1..64) graph replays, and writes the fastest shape to
 * *tuning (queue_chunk, block_size, min_blocks, stack_depth; the other fields
 * 0 / defaults) and its time to *best_ms (may be NULL).  It runs the batch as
 * given about 12 x (reps + 1) times (12 shapes), so the views' histories and outputs are
 * overwritten: tune on the frames' first batch or on copies.  Pass the result
 * to hy_batch_forward; a C++ application can keep it per GPU and workload. */
int hy_batch_autotune(HyCtx* ctx, HyCtx* const* scenes, uint32_t num_scenes, const HyView* views,
                      uint32_t num_views, uint32_t reps, HyPassConfig* tuning, float* best_ms);

/* ---- allocation-free accumulation (no counterpart in the reference) ----
 *
 * hy_accumulate_pass without a context and without any device allocation,
 * for callers that may not allocate device memory themselves or have it
 * allocated for them: an engine whose allocator owns and budgets every
 * device allocation (as VMA does for VkPinut), or a frame loop that cannot
 * afford the device-wide wait of cudaFree.  It computes exactly what
 * hy_accumulate_pass computes, on the calling thread's current device and on
 * `stream` (a cudaStream_t; NULL is the default stream), and returns without
 * synchronising.
 *
 * The reset-frame branch (accum_frame <= 0) snapshots the history into a
 * fixed scratch array of HY_NOALLOC_SCRATCH_BYTES that lives in the library
 * and is held by every GPU that loads it until the process exits.  Calls
 * whose history (width * height * num_lights * 1 or 4 bytes) exceeds it
 * return HY_ERR_TOO_LARGE.  The first call on a device looks up the array's
 * device address (once per device); make that first call before any stream
 * capture.  The address stays cached for the life of the process, so after a
 * cudaDeviceReset of a device the entry point must not be called on that
 * device again.  All calls on a device share the one array, so calls whose work
 * overlaps on the GPU (different streams, not ordered) race on it; order
 * them on one stream.  The array keeps the last call's contents; nothing in
 * it needs to start at zero. */
#define HY_NOALLOC_SCRATCH_BYTES (16u << 20)
int hy_accumulate_pass_noalloc(const HyGBuffer* gb, const HyPassConfig* cfg, const void* d_shadow,
                               HyAccum* accum, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* HYBRIDRT_H */
