// Host-side context of libhybridrt (not part of the C ABI).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/hybridrt.h"

struct HyCtx;

namespace hy {

// Device allocation owned by the context; grows on demand, never shrinks.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    template <class T> T* as() const { return (T*)p; }
};

int ctx_alloc(HyCtx* c, DevBuf& b, size_t bytes);  // HY_OK / HY_ERR_OOM / HY_ERR_CUDA
void ctx_free(HyCtx* c, DevBuf& b);

// Accumulated per-pass device counters (u64 each)
enum { ST_SHADOW = 0, ST_REFL, ST_HITSHADOW, ST_NODES, ST_TRIS, ST_COUNT };
// work-queue counters (u32 each)
enum { WQ_SHADOW = 0, WQ_SHADE, WQ_MISC, WQ_COUNT };

}  // namespace hy

struct HyCtx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    uint64_t max_bytes = 0, used_bytes = 0;
    uint32_t fail_after = 0, alloc_calls = 0;
    uint32_t dbg_max_iters = 0, dbg_stack_cap = 0;  // hy_debug_set_traversal_limits (0: the built-in limits)
    int num_sms = 0;
    int l2_bytes = 0;  // the device's L2 size (the automatic any-hit order compares the structure with it)

    // ---- scene ----
    hy::DevBuf verts, vattr, idx, prims, xf, nrm, prim_tri0, tri_prim, mats, lights, env[2];
    hy::DevBuf tex_px, tex_tab;  // material textures: concatenated RGBA8 texels, (first, w, h, 0) per texture
    uint32_t nverts = 0, nidx = 0, nprims = 0, nxf = 0, ntri = 0, nmats = 0, nlights = 0, ntex = 0;
    std::vector<HyMaterial> h_mats;  // host copy for texture-id validation
    uint32_t max_material_id = 0;
    uint32_t env_w[2] = {0, 0}, env_h[2] = {0, 0};
    bool geometry_ok = false;

    // ---- acceleration structure ----
    hy::DevBuf world;       // float4 x3 per triangle (world-space vertices)
    hy::DevBuf tribox;      // float lo[3], hi[3] per triangle
    hy::DevBuf centroid;    // float4 per triangle
    hy::DevBuf keys[2], vals[2];
    hy::DevBuf bvh2;        // 10 words per internal node: left,right,first,last, lo[3], hi[3]
    hy::DevBuf parent;      // n-1 internal + n leaves
    hy::DevBuf flags;       // refit arrival counters
    hy::DevBuf bounds;      // 6 orderable ints + build scratch
    hy::DevBuf lvl_ref[2], plan, ni, nt, ni_scan, nt_scan;
    hy::DevBuf scan_tmp, hist, total;
    hy::DevBuf nodes, tris;
    hy::DevBuf node_ref, node_plan;  // per BVH8 node: its BVH2 subtree, its 8 slot children (refits)
    hy::DevBuf dp_cost, dp_k;        // collapse slot budgets: 8 costs, 9 choices per binary-tree node
    uint32_t build_mode = HY_BUILD_SAH;  // hy_scene_set_build_mode
    // binned-SAH build scratch (hy_sah.cu): range queues, bins, chunk maps, counters
    hy::DevBuf sah_ranges[2], sah_small, sah_bins, sah_split, sah_chunks, sah_first, sah_ccnt, sah_coff, sah_ctr;
    uint32_t n_bvh8 = 0, depth = 0;
    bool bvh_ok = false;

    // ---- two-level structure (hy_bvh_build_instanced) ----
    // nodes / tris then hold the TLAS region (tlas_region nodes and records)
    // followed by one BLAS per distinct mesh
    bool two_level = false;
    hy::DevBuf xinv;                 // 12 floats per transform: world->object rows (always kept current)
    hy::DevBuf inst;                 // 64 B per instance: 3 rows + (BLAS root, first triangle, primitive, 0)
    hy::DevBuf inst_box;             // 6 floats per instance: its TLAS box
    hy::DevBuf inst_prim, prim_mesh, blas_node0;
    hy::DevBuf mesh_vrange;          // per mesh: smallest, largest vertex index its triangles use
    hy::DevBuf inst_chunks;          // (instance, first vertex, end vertex, 0): the box work of a TLAS update
    hy::DevBuf inst_keys;            // 6 order-preserving 64-bit keys per instance (box min / max)
    uint32_t n_chunks = 0;
    std::vector<HyPrimitive> h_prims;
    std::vector<uint32_t> h_inst_prim, h_prim_mesh, h_mesh_prim, h_blas_node0;
    uint32_t ninst = 0, nblas = 0, tlas_region = 0, tlas_nodes = 0, tlas_depth = 0, blas_depth = 0;
    uint32_t anyhit_order = 0;       // HY_ANYHIT_*: child order of any-hit traversal
    uint32_t n_records = 0;          // leaf records in tris
    HyBvhStats last_build{};

    // ---- pass scratch ----
    hy::DevBuf dstats;      // u64[ST_COUNT] + u32 status + u32 queue counters
    hy::DevBuf raw_shadow;  // per-light raw shadow images (unfused path)
    hy::DevBuf hist_prev;   // history snapshot for the reprojection read
    hy::DevBuf host_in[6], host_out_f, host_out_8;  // device staging of hy_hybrid_forward_host
    // hy_hybrid_forward_host copies G-buffer planes 2-5 on a side stream while
    // the shadow kernel runs; the passes after it wait for copy_done
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_start = nullptr, copy_done = nullptr;
    bool copy_pending = false;
    hy::DevBuf grad_partial;  // per-block partial gradient vectors of hy_hybrid_backward

    // ---- per-kernel timing (hy_profile_*) ----
    struct ProfRec { int kind; cudaEvent_t a, b; };
    bool prof_on = false;
    std::vector<cudaEvent_t> prof_pool;   // created on demand, reused after each read
    size_t prof_used = 0;
    std::vector<ProfRec> prof_recs;
    uint32_t* h_status = nullptr;   // pinned readback slot
    unsigned long long* h_stats = nullptr;

    // ---- batches ----
    hy::DevBuf batch_tab;           // PassParams[num_views] + SceneDev[num_scenes]
    void* h_batch_tab = nullptr;    // pinned mirror, copied in by the captured graph
    size_t h_batch_tab_bytes = 0;
    cudaGraphExec_t batch_exec = nullptr;
    std::vector<uint64_t> batch_key;
    cudaEvent_t batch_done = nullptr;
};

namespace hy {
int bvh_build_impl(HyCtx* c, HyBvhStats* st);
int bvh_refit_impl(HyCtx* c);
int bvh_build_instanced_impl(HyCtx* c, HyBvhStats* st);
int tlas_build_impl(HyCtx* c);   // instance records + TLAS from the current transforms
int world_tris_impl(HyCtx* c);
int scan_exclusive(HyCtx* c, const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* d_total);
// binned-SAH binary tree over the n >= 2 Morton-sorted ids in ord (hy_sah.cu)
int sah_tree_impl(HyCtx* c, uint32_t n, uint32_t* ord, uint32_t* ord2, uint32_t* bvh2, uint32_t* parent,
                  uint32_t* d_root);
}  // namespace hy

#define HY_CUDA_TRY(expr)                               \
    do {                                                \
        cudaError_t _e = (expr);                        \
        if (_e != cudaSuccess) return HY_ERR_CUDA;      \
    } while (0)
