// ORACLE — test infrastructure only (see orc_math.hpp).  Scene state, BVH and
// traversal of the CPU restatement.
#pragma once
#include <cstdint>
#include <vector>

#include "../include/hybridrt.h"
#include "orc_math.hpp"

namespace orc {

constexpr int kLeafMax = 3;           // triangles per BVH8 leaf slot
constexpr float kCostNode = 1.0f;     // collapse: cost of a node visit (per unit area)
constexpr float kCostTri = 0.5f;      // collapse: cost of a triangle test (a node visit ~2 tests)
constexpr int kStackMax = 64;         // traversal stack entries
constexpr uint32_t kMaxIters = 1u << 22;  // node visits per ray before giving up

struct Env { uint32_t w = 0, h = 0; std::vector<uint8_t> px; };

struct Bvh2Node { uint32_t left, right, first, last; float lo[3], hi[3]; };
constexpr uint32_t kLeafBit = 0x80000000u;

// 80-byte compressed BVH8 node as 20 words (the product's layout):
//  w0-2 p.xyz | w3 e.x | e.y<<8 | e.z<<16 | imask<<24 | w4 child_base | w5 tri_base
//  w6-7 meta[8] | w8-9 qlo_x[8] | w10-11 qlo_y | w12-13 qlo_z | w14-15 qhi_x | w16-17 qhi_y | w18-19 qhi_z
struct Bvh8Node { uint32_t w[20]; };

struct Bvh {
    uint32_t n = 0;
    float slo[3], shi[3];
    std::vector<uint32_t> morton, order;   // sorted morton codes and triangle ids
    std::vector<Bvh2Node> bvh2;            // n-1 internal nodes
    uint32_t root = 0;                     // root reference (kLeafBit | 0 for one triangle)
    std::vector<Bvh8Node> bvh8;            // BFS order
    std::vector<float> tris;               // 12 floats per packed triangle
    uint32_t depth = 0;
    std::vector<uint32_t> node_ref;        // BVH2 subtree of each BVH8 node (refits)
    std::vector<uint32_t> node_plan;       // its 8 slot children, 0xffffffff = empty (refits)
};

// Two-level structure (the driver's BLAS-per-primitive + TLAS split,
// src/vk_mesh.cpp:424-492, src/renderer.cpp:1696-1865): one BLAS per distinct
// mesh (primitives with equal first_index, index_count and vertex_offset share
// it) over its object-space triangles, and a TLAS over the instance boxes.
// Node array: the TLAS region (tlas_region nodes, root 0, unused tail zero),
// then each BLAS.  Record array: tlas_region instance entries (box lo, hi, hi
// and the instance index), then each BLAS's triangles (object-space vertices
// and the triangle's index within its mesh).
struct Bvh2L {
    std::vector<Bvh8Node> nodes;
    std::vector<float> tris;            // 12 floats per record
    std::vector<float> inst;            // 16 per instance: world->object rows 3 x (m0 m1 m2 t), root, tri0, prim, 0
    std::vector<float> inst_box;        // 6 per instance: TLAS item box (lo, hi)
    std::vector<uint32_t> inst_prim;    // primitive of each instance (primitives with triangles, in order)
    std::vector<uint32_t> prim_mesh;    // BLAS of each primitive, 0xffffffff when it has no triangles
    std::vector<uint32_t> mesh_prim;    // first primitive of each BLAS (its index range)
    std::vector<uint32_t> blas_node0, blas_rec0, blas_nodes;
    std::vector<uint32_t> mesh_vrange;  // 2 per BLAS: first vertex, one past the last vertex its triangles use
    std::vector<float> xinv;            // 12 per transform: world->object rows
    uint32_t ninst = 0, nblas = 0, tlas_region = 0, tlas_nodes = 0, tlas_depth = 0, blas_depth = 0;
};

struct Counters { uint64_t nodes = 0, tris = 0; uint32_t status = 0; };

struct Hit { float t; uint32_t id; float b1, b2; };

struct Scene {
    std::vector<HyVertex> verts;
    std::vector<uint32_t> idx;
    std::vector<HyPrimitive> prims;
    std::vector<float> xf;        // 16 per transform (column-major)
    std::vector<float> nrm;       // 9 per transform: mat3(transpose(inverse(M))), column-major
    std::vector<HyMaterial> mats;
    std::vector<HyLight> lights;
    Env env[2];
    std::vector<Env> tex;         // material textures (RGBA8, NEAREST / REPEAT), by texture id
    // derived geometry
    uint32_t ntri = 0;
    std::vector<float> world;        // 9 floats per triangle (v0, v1, v2) in world space
    std::vector<uint32_t> tri_prim;  // primitive of each triangle
    std::vector<uint32_t> prim_tri0; // first global triangle of each primitive
    Bvh bvh;
    bool bvh_ok = false;
    Bvh2L two;                    // valid when two_level
    bool two_level = false;
    uint32_t anyhit_order = HY_ANYHIT_AUTO;  // child order of any-hit traversal
    uint32_t build_mode = HY_BUILD_SAH;      // binary tree under the 8-wide nodes
};

// XOR applied to the near octant to rank the children of any-hit traversal:
// 7 = far first, 0 = near first.  HY_ANYHIT_AUTO as the product resolves it
// for structures that fit in L2 (every case the oracle runs): far first for
// one level, near first for two levels.
inline uint32_t anyhit_flip(const Scene& s) {
    if (s.anyhit_order == HY_ANYHIT_FAR_FIRST) return 7u;
    if (s.anyhit_order == HY_ANYHIT_NEAR_FIRST || s.two_level) return 0u;
    return 7u;
}

// geometry / BVH
void scene_derive(Scene& s);
void derive_world(Scene& s);   // normal matrices and world triangles from the current transforms
void bvh_build(Scene& s);
void bvh_build_instanced(Scene& s);   // two-level structure
void bvh_refit(Scene& s);             // two-level: instance records and TLAS rebuilt, BLASes kept
// traversal: mode 0 = brute force over all triangles, 1 = BVH8 (op-for-op the
// product's traversal, so node/triangle counts are comparable)
Hit trace(const Scene& s, const float o[3], const float d[3], float tmin, float tmax, bool any_hit,
          int mode, Counters* c);

}  // namespace orc
