// Tile streams: the warp-cooperative shadow-ray schedule shared by the hybrid
// pass (hy_pass.cu) and the path-traced mode (hy_pt.cu).  Per light, each lane
// publishes one pixel's shadow-ray inputs (position, distance, sampleDisk's
// frame, the RNG state of the pixel-light's first sample) in shared memory;
// the warp then traces the 32 x n_rays samples as items q (sample q % n_rays of
// pixel q / n_rays), claimed in order from a per-warp counter by whichever
// lanes are free, each lane walking its rays with several node visits per
// scheduling round and without waiting for the others; unoccluded samples are
// counted per pixel with shared-memory atomics.
#pragma once
#include <cuda_runtime.h>

#include "hy_device.cuh"
#include "hy_pass.h"
#include "hy_shade.cuh"

namespace hy {

// The top levels of the node array (BFS order: levels 0-2 of an 8-wide tree
// are its first 73 nodes) staged in shared memory once per block.  Measured
// neutral at 1080p (0 / 9 / 73 / 128 staged nodes: 2,551 / 2,547 / 2,560 /
// 2,553 Mrays/s): those nodes are L1-resident anyway.
constexpr uint32_t kTopNodes = 73;
__device__ __forceinline__ uint32_t stage_top(const SceneDev& S, uint4* top, uint32_t limit) {
    const uint32_t ntop = min(min(S.num_nodes, kTopNodes), limit);
    for (uint32_t i = threadIdx.x; i < ntop * 5; i += blockDim.x) top[i] = __ldg(&S.nodes[i / 5].q[i % 5]);
    __syncthreads();
    return ntop;
}

// Per-warp shared state of the tile streams, per pixel of the warp's tile and
// the current light: position and distance to the light; the disk frame of
// sampleDisk (position + L, tangent, bitangent); the RNG state of the
// pixel-light's first sample (w of PL, as bits); a not-traced mark (w of T,
// 0xffffffff); the unoccluded count.
// Items of a light are traced in the order of their disk samples (kSortItems at
// most per warp and light; more are traced in item order).
constexpr uint32_t kSortItems = 512, kSortBuckets = 64;
struct StreamSlots {
    float4 pos[128];
    float4 PL[128];
    float4 T[128];
    float4 B[128];
    uint32_t cnt[128];
    uint32_t next[4];  // per warp: the next unclaimed item of the current light
    // per warp: the traced items of the light ordered by their disk sample, the
    // sample's cell per item, and the cell counts / cursors of the counting sort
    uint16_t order[4][kSortItems];
    uint8_t key[4][kSortItems];
    uint32_t bucket[4][kSortBuckets];
};

constexpr uint32_t kNotTraced = 0xffffffffu;

// lane's slot for the current light; first_state: the RNG state of sample 0
__device__ __forceinline__ void stream_publish(StreamSlots& sm, bool traced, f3 position, f3 L, float dist,
                                               uint32_t first_state) {
    const uint32_t i = threadIdx.x;
    if (traced) {
        const DiskFrame d = disk_frame(position, L);
        sm.pos[i] = make_float4(position.x, position.y, position.z, dist);
        sm.PL[i] = make_float4(d.PL.x, d.PL.y, d.PL.z, __uint_as_float(first_state));
        sm.T[i] = make_float4(d.T.x, d.T.y, d.T.z, 0.f);
        sm.B[i] = make_float4(d.B.x, d.B.y, d.B.z, 0.f);
    } else {
        sm.T[i].w = __uint_as_float(kNotTraced);
    }
    sm.cnt[i] = 0;
    if ((i & 31) == 0) sm.next[i >> 5] = 0;
}

// The warp's items of one light (every lane calls it, after all lanes have
// published): sample k of a pixel starts from its first state advanced 2k LCG
// steps (sampleDisk's two draws per sample), its ray from position +
// offset * dir to distance + 1.  On return sm.cnt holds each pixel's
// unoccluded samples.
template <bool COUNT, bool TWO, class Stack>
__device__ __forceinline__ void stream_light(const SceneDev& S, const PassParams& P, StreamSlots& sm, uint32_t nrays,
                                             float radius, float offset, Stack stk, Trav& t, RayPre& r,
                                             LaneStats& ls, uint32_t& nn, uint32_t& nt, const uint4* top,
                                             uint32_t ntop) {
    const uint32_t lane = threadIdx.x & 31, wb = threadIdx.x & ~31u, warp = threadIdx.x >> 5;
    uint32_t total = 32u * nrays;
    uint32_t* next = &sm.next[warp];
    __syncwarp();
    // ---- the order of the light's items: a counting sort of the traced items by
    //      the cell of their disk sample on an 8x8 grid over the disk (cells in
    //      Morton order), so that the lanes' rays at any moment are nearly
    //      parallel rays from the tile's nearby pixels and walk the same nodes.
    //      The rays themselves do not change: only which lane traces which ray,
    //      and when ----
    const bool sorted = nrays > 1 && total <= kSortItems;
    if (sorted) {
        uint32_t* bk = sm.bucket[warp];
        bk[lane] = 0;
        bk[lane + 32] = 0;
        __syncwarp();
        for (uint32_t q = lane; q < total; q += 32) {
            const uint32_t pi = q / nrays, k = q - pi * nrays;
            uint32_t key = 0xffu;
            if (__float_as_uint(sm.T[wb + pi].w) != kNotTraced) {
                uint32_t st = lcg_jump(__float_as_uint(sm.PL[wb + pi].w), 2u * k);
                const float r1 = rnd(st), r2 = rnd(st);
                // the disk point in units of the radius (approximate: it only orders the items)
                float sn, cs;
                __sincosf(6.2831853f * r2, &sn, &cs);
                const float rr = sqrtf(r1);
                const uint32_t ix = min(7u, (uint32_t)fmaxf((rr * cs + 1.0f) * 4.0f, 0.0f));
                const uint32_t iy = min(7u, (uint32_t)fmaxf((rr * sn + 1.0f) * 4.0f, 0.0f));
                key = (ix & 1u) | ((iy & 1u) << 1) | ((ix & 2u) << 1) | ((iy & 2u) << 2) | ((ix & 4u) << 2) |
                      ((iy & 4u) << 3);
                atomicAdd(&bk[key], 1u);
            }
            sm.key[warp][q] = (uint8_t)key;
        }
        __syncwarp();
        // exclusive scan of the 64 counts, two per lane
        const uint32_t c0 = bk[2 * lane], c1 = bk[2 * lane + 1], c = c0 + c1;
        uint32_t incl = c;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
            if (lane >= (uint32_t)d) incl += y;
        }
        total = __shfl_sync(0xffffffffu, incl, 31);  // the traced items
        __syncwarp();
        bk[2 * lane] = incl - c;
        bk[2 * lane + 1] = incl - c + c0;
        __syncwarp();
        for (uint32_t q = lane; q < 32u * nrays; q += 32) {
            const uint32_t key = sm.key[warp][q];
            if (key != 0xffu) sm.order[warp][atomicAdd(&bk[key], 1u)] = (uint16_t)q;
        }
        __syncwarp();
    }
    bool live = false, more = true;
    uint32_t cur = 0;
    for (;;) {
        // ---- this lane's next item of a traced pixel, claimed from the warp's
        //      counter: items go to whichever lanes are free, in order, so the
        //      warp's work stays balanced until the light's last items ----
        while (!live && more) {
            // one shared atomic per group of lanes claiming together, lane order kept
            const uint32_t m = __activemask(), leader = __ffs(m) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(next, (uint32_t)__popc(m));
            base = __shfl_sync(m, base, leader);
            uint32_t q = base + (uint32_t)__popc(m & ((1u << lane) - 1u));
            if (q >= total) { more = false; break; }
            if (sorted) q = sm.order[warp][q];
            const uint32_t pi = q / nrays, k = q - pi * nrays;
            const float4 tp = sm.T[wb + pi];
            if (__float_as_uint(tp.w) == kNotTraced) continue;
            const float4 pp = sm.pos[wb + pi], pl = sm.PL[wb + pi], bp = sm.B[wb + pi];
            const f3 pos = mk(pp.x, pp.y, pp.z);
            const DiskFrame d{mk(tp.x, tp.y, tp.z), mk(bp.x, bp.y, bp.z), mk(pl.x, pl.y, pl.z)};
            uint32_t st = lcg_jump(__float_as_uint(pl.w), 2u * k);
            const f3 dir = sampleDisk(radius, pos, d, st);
            r = ray_pre(add_rn(pos, scale_rn(dir, offset)), dir);
            trav_init(t, r, __fadd_rn(pp.w, 1.0f));
            cur = pi;
            live = true;
            ls.shadow++;
        }
        // ---- up to P.inner node visits, each with its leaf triangles (testing
        //      the triangles of many lanes together instead, once enough lanes
        //      have some, measured slower: 2,190 against 2,899 Mrays/s at 1080p,
        //      the lanes waiting on triangles idle through the node visits) ----
        if (live) {
            for (uint32_t it = 0, ni = max(P.inner, 1u); it < ni; it++) {
                if (trav_step<true, COUNT, TWO>(S, r, 0.001f, t, stk, nn, nt, P.status, top, ntop)) {
                    live = false;
                    if (t.h.id == HY_NO_HIT) atomicAdd(&sm.cnt[wb + cur], 1u);
                    break;
                }
            }
        }
        if (__ballot_sync(0xffffffffu, live || more) == 0) break;
    }
    __syncwarp();
}

}  // namespace hy
