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

// Per-warp shared state of the tile streams, per pixel of the warp's tile and
// the current light: position and distance to the light; the disk frame of
// sampleDisk (position + L, tangent, bitangent); the RNG state of the
// pixel-light's first sample (w of PL, as bits); a not-traced mark (w of T,
// 0xffffffff); the unoccluded count (w of B, as bits).
// Items of a light are traced in the order of their disk samples, sorted in
// chunks of SORT items per warp and light.
// The size matters beyond occupancy: shared memory and L1 share each SM's
// 256 KB, and the driver carves shared memory in steps (..., 100, 132, 164,
// 196 KB).  At 4 warps per block and 8 blocks per SM this layout (15.4 KB, + 1
// KB the driver keeps per block) takes the 132 KB step and leaves the kernel
// 124 KB of L1 for the nodes, triangles and traversal stacks it re-reads
// (the same slots with a separate count array and 73 top nodes staged per
// block took the 196 KB step: 1080p shadow kernel 22.5 ms against 22.2 ms with
// 92 KB of L1 and no staging).
constexpr uint32_t kSortItems = 512, kSortBuckets = 64;
template <int NW, uint32_t SORT = kSortItems>  // warps per block, items sorted together
struct StreamSlotsT {
    static constexpr uint32_t kSort = SORT;
    // the sort keys of a light's items: in shared memory up to 4 warps per block,
    // in a chain of registers beyond (8-warp batch blocks: 30 KB instead of 34 KB,
    // under the 132 KB shared-memory step at 4 blocks per SM)
    static constexpr bool kKeysShared = NW <= 4;
    float4 pos[NW * 32];
    float4 PL[NW * 32];
    float4 T[NW * 32];
    float4 B[NW * 32];
    uint32_t next[NW];  // per warp: the next unclaimed item of the current light
    // per warp: the traced items of the light ordered by their disk sample, the
    // sample's cell per item (kKeysShared) and the cell counts / cursors of the
    // counting sort
    uint16_t order[NW][SORT];
    uint8_t key[kKeysShared ? NW : 1][kKeysShared ? SORT : 1];
    uint32_t bucket[NW][kSortBuckets];
};
using StreamSlots = StreamSlotsT<4>;

constexpr uint32_t kNotTraced = 0xffffffffu;

// lane's slot for the current light; first_state: the RNG state of sample 0
// the current light's unoccluded-sample count of slot i
template <class Slots>
__device__ __forceinline__ uint32_t* unocc_count(Slots& sm, uint32_t i) {
    return reinterpret_cast<uint32_t*>(&sm.B[i].w);
}

template <class Slots>
__device__ __forceinline__ void stream_publish(Slots& sm, bool traced, f3 position, f3 L, float dist,
                                               uint32_t first_state) {
    const uint32_t i = threadIdx.x;
    if (traced) {
        const DiskFrame d = disk_frame(position, L);
        sm.pos[i] = make_float4(position.x, position.y, position.z, dist);
        sm.PL[i] = make_float4(d.PL.x, d.PL.y, d.PL.z, __uint_as_float(first_state));
        sm.T[i] = make_float4(d.T.x, d.T.y, d.T.z, 0.f);
        sm.B[i] = make_float4(d.B.x, d.B.y, d.B.z, 0.f);  // w: the unoccluded count, 0
    } else {
        sm.T[i].w = __uint_as_float(kNotTraced);
        sm.B[i].w = 0.f;
    }
    if ((i & 31) == 0) sm.next[i >> 5] = 0;
}

// The warp's items of one light (every lane calls it, after all lanes have
// published): sample k of a pixel starts from its first state advanced 2k LCG
// steps (sampleDisk's two draws per sample), its ray from position +
// offset * dir to distance + 1.  On return unocc_count holds each pixel's
// unoccluded samples.
template <bool COUNT, bool TWO, class Stack, class Slots, class RW>
__device__ __forceinline__ void stream_light(const SceneDev& S, const PassParams& P, Slots& sm, uint32_t nrays,
                                             float radius, float offset, Stack stk, Trav& t, RW& r,
                                             LaneStats& ls, uint32_t& nn, uint32_t& nt, const uint4* top,
                                             uint32_t ntop) {
    const uint32_t lane = threadIdx.x & 31, wb = threadIdx.x & ~31u, warp = threadIdx.x >> 5;
    uint32_t* next = &sm.next[warp];
    const uint32_t all = 32u * nrays;
    __syncwarp();
    // the light's items in chunks of Slots::kSort (one chunk unless spp > 16)
    for (uint32_t c0 = 0; c0 < all; c0 += Slots::kSort) {
        const uint32_t cn = min(Slots::kSort, all - c0);
        uint32_t total = cn;
        // ---- the order of the chunk's items: a counting sort of the traced items by
        //      the cell of their disk sample on an 8x8 grid over the disk (cells in
        //      Morton order), so that the lanes' rays at any moment are nearly
        //      parallel rays from the tile's nearby pixels and walk the same nodes
        //      (1080p: 31.96 -> 29.90 ms per shadow launch).  The rays themselves do
        //      not change: only which lane traces which ray, and when ----
        const bool sorted = nrays > 1;
        if (sorted) {
            uint32_t* bk = sm.bucket[warp];
            bk[lane] = 0;
            bk[lane + 32] = 0;
            __syncwarp();
            // each lane's item keys (items lane + 32 i, one byte each) go to shared
            // memory or through a shift chain of registers: after the kSort / 32
            // steps item i's key is byte i
            constexpr uint32_t kSteps = Slots::kSort / 32, kWords = kSteps / 4;
            static_assert(kSteps % 4 == 0, "whole key words");
            uint32_t keys[kWords];
#pragma unroll
            for (uint32_t w = 0; w < kWords; w++) keys[w] = 0;
            for (uint32_t i = 0; i < kSteps; i++) {
                const uint32_t j = lane + 32u * i;
                uint32_t key = 0xffu;
                const uint32_t q = c0 + j, pi = j < cn ? q / nrays : 0u, k = q - pi * nrays;
                if (j < cn && __float_as_uint(sm.T[wb + pi].w) != kNotTraced) {
                    uint32_t st = lcg_jump_even(__float_as_uint(sm.PL[wb + pi].w), k);
                    const float r1 = rnd(st), r2 = rnd(st);
                    // the disk point in units of the radius (approximate: it only orders the items)
                    float sn, cs;
                    __sincosf(6.2831853f * r2, &sn, &cs);
                    const float rr = r1 > 0.f ? r1 * rsqrtf(r1) : 0.f;
                    const uint32_t ix = min(7u, (uint32_t)fmaxf((rr * cs + 1.0f) * 4.0f, 0.0f));
                    const uint32_t iy = min(7u, (uint32_t)fmaxf((rr * sn + 1.0f) * 4.0f, 0.0f));
                    key = (ix & 1u) | ((iy & 1u) << 1) | ((ix & 2u) << 1) | ((iy & 2u) << 2) | ((ix & 4u) << 2) |
                          ((iy & 4u) << 3);
                    atomicAdd(&bk[key], 1u);
                }
                if constexpr (Slots::kKeysShared) {
                    if (j < cn) sm.key[warp][j] = (uint8_t)key;
                } else {
#pragma unroll
                    for (uint32_t w = 0; w + 1 < kWords; w++) keys[w] = (keys[w] >> 8) | (keys[w + 1] << 24);
                    keys[kWords - 1] = (keys[kWords - 1] >> 8) | (key << 24);
                }
            }
            __syncwarp();
            // exclusive scan of the 64 counts, two per lane
            const uint32_t cnt0 = bk[2 * lane], cnt1 = bk[2 * lane + 1], c = cnt0 + cnt1;
            uint32_t incl = c;
    #pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= (uint32_t)d) incl += y;
            }
            total = __shfl_sync(0xffffffffu, incl, 31);  // the chunk's traced items
            __syncwarp();
            bk[2 * lane] = incl - c;
            bk[2 * lane + 1] = incl - c + cnt0;
            __syncwarp();
            for (uint32_t i = 0; i < kSteps; i++) {
                const uint32_t j = lane + 32u * i;
                uint32_t key;
                if constexpr (Slots::kKeysShared) {
                    if (j >= cn) break;
                    key = sm.key[warp][j];
                } else {
                    key = keys[0] & 0xffu;
#pragma unroll
                    for (uint32_t w = 0; w + 1 < kWords; w++) keys[w] = (keys[w] >> 8) | (keys[w + 1] << 24);
                    keys[kWords - 1] >>= 8;
                    if (j >= cn) continue;
                }
                if (key != 0xffu) sm.order[warp][atomicAdd(&bk[key], 1u)] = (uint16_t)j;
            }
        }
        if (lane == 0) *next = 0;
        __syncwarp();
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
                q = c0 + (sorted ? (uint32_t)sm.order[warp][q] : q);
                const uint32_t pi = q / nrays, k = q - pi * nrays;
                const float4 tp = sm.T[wb + pi];
                if (__float_as_uint(tp.w) == kNotTraced) continue;
                const float4 pp = sm.pos[wb + pi], pl = sm.PL[wb + pi], bp = sm.B[wb + pi];
                const f3 pos = mk(pp.x, pp.y, pp.z);
                const DiskFrame d{mk(tp.x, tp.y, tp.z), mk(bp.x, bp.y, bp.z), mk(pl.x, pl.y, pl.z)};
                uint32_t st = lcg_jump_even(__float_as_uint(pl.w), k);
                const f3 dir = sampleDisk(radius, pos, d, st);
                trav_init(t, world_set(r, add_rn(pos, scale_rn(dir, offset)), dir), __fadd_rn(pp.w, 1.0f));
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
                        if (t.h.id == HY_NO_HIT) atomicAdd(unocc_count(sm, wb + cur), 1u);
                        break;
                    }
                }
            }
            if (__ballot_sync(0xffffffffu, live || more) == 0) break;
        }
        __syncwarp();
    }
}

__device__ __forceinline__ float roundtrip(uint32_t fmt, float v) {
    return fmt == HY_ACCUM_U8 ? __fdiv_rn((float)quant8(v), 255.0f) : v;
}

// A lane's pixel in the shadow kernels (set-up, current light, sample state).
struct ShadowLane {
    f3 position, N, L;
    float dist, radius;
    uint32_t pix, seed, light, k, nrays;
    float sf;
    int smode;
    bool in_blur, setup;
};

template <bool ACCUM>
__device__ __forceinline__ void shadow_finalize(const PassParams& P, const ShadowLane& s, size_t plane, float v) {
    const size_t li = (size_t)s.light * plane + s.pix;
    if (!ACCUM) {
        accum_store(P.accum_fmt, P.shadow, li, v);
    } else if (s.in_blur) {
        const float center = roundtrip(P.accum_fmt, v);
        const float old = accum_load(P.accum_fmt, P.hist, li);
        const float a = __fdiv_rn(1.0f, __fadd_rn((float)P.accum_frame, 1.0f));
        accum_store(P.accum_fmt, P.hist, li, __fadd_rn(__fmul_rn(old, __fsub_rn(1.0f, a)), __fmul_rn(center, a)));
    }
}

// ---------------------------------------------------------------------------------
// One 8x4 tile of a view, light by light.  ACC: 0 raw shadow images, 1 the
// running mean into the history, 2 either (accum) at run time.  reference:
// REFERENCE RNG (one ray per pixel-light from the pixel's seed, by value).
template <bool COUNT, bool TWO, int ACC, class Stack, class Slots, class RW>
__device__ __forceinline__ void stream_tile(const SceneDev& S, const PassParams& P, uint32_t tile, bool reference,
                                            bool accum, Slots& sm, Stack stk, Trav& t, RW& r,
                                            ShadowLane& s, LaneStats& ls, uint32_t& nn, uint32_t& nt,
                                            const uint4* top, uint32_t ntop) {
    const uint32_t lane = threadIdx.x & 31, wb = threadIdx.x & ~31u;
    const size_t plane = (size_t)P.W * P.H;
    const uint32_t spp = P.spp, nrays = reference ? 1u : spp;
    const uint32_t x = (tile % P.tiles_x) * 8 + (lane & 7), y = (tile / P.tiles_x) * 4 + (lane >> 3);
    const bool present = x < P.W && y < P.H;
    auto finalize = [&](float v) {
        if (ACC == 0 || (ACC == 2 && !accum)) shadow_finalize<false>(P, s, plane, v);
        else shadow_finalize<true>(P, s, plane, v);
    };
    uint32_t seed0 = 0, rays_before = 0;
    if (present) {
        s.pix = y * P.W + x;
        const float4 g0 = fetch_texel(P.plane[0], P.fmt[0], s.pix);
        const float4 g1 = fetch_texel(P.plane[1], P.fmt[1], s.pix);
        s.position = mk(g0.x, g0.y, g0.z);
        s.N = normalize_rn(mk(__fsub_rn(__fmul_rn(g1.x, 2.0f), 1.0f), __fsub_rn(__fmul_rn(g1.y, 2.0f), 1.0f),
                              __fsub_rn(__fmul_rn(g1.z, 2.0f), 1.0f)));
        const int mi = mat_index(g0.w, S.num_mats);
        s.smode = mi >= 0 ? (int)S.mats[mi].smr[0] : 0;
        s.in_blur = x < P.blur_w && y < P.blur_h;
        seed0 = tea(s.pix, P.frame_u);
    }
    for (uint32_t l = 0; l < P.num_lights; l++) {
        // ---- light l for this lane's pixel ----
        bool traced = false;
        s.light = l;
        if (present) {
            const LightGeo lg = light_geo(S.lights[l], s.position, s.N);
            float v = -1.f;
            if (s.smode == 4) v = 1.0f;
            else if (!(lg.NdotL > 0.f)) v = 0.0f;
            else if (!(lg.dist < lg.maxd)) v = 1.0f;
            if (v >= 0.f) finalize(v);
            else traced = true;
            stream_publish(sm, traced, s.position, lg.L, lg.dist,
                           !traced || reference ? seed0 : lcg_jump(seed0, 2u * rays_before));
        } else {
            stream_publish(sm, false, s.position, s.position, 0.f, 0u);
        }
        if (__ballot_sync(0xffffffffu, traced) != 0) {
            // shadowRaygen.rgen:78: origin position + 0.1 dir, tmax distance + 1
            stream_light<COUNT, TWO>(S, P, sm, nrays, S.lights[l].radius, 1e-1f, stk, t, r, ls, nn, nt, top, ntop);
            if (traced) {
                const uint32_t unocc = *unocc_count(sm, wb + lane);
                finalize(reference ? (float)unocc : __fdiv_rn((float)unocc, (float)spp));
            }
        }
        if (traced) rays_before += spp;
        __syncwarp();  // the slots are rewritten by the next light's set-up
    }
}

// the view of a batch tile: s_begin holds each view's first tile (ascending)
__device__ __forceinline__ uint32_t view_of_tile(const uint32_t* s_begin, uint32_t nviews, uint32_t tile) {
    uint32_t lo = 0, hi = nviews;  // s_begin[lo] <= tile < s_begin[hi]
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (s_begin[mid] <= tile) lo = mid;
        else hi = mid;
    }
    return lo;
}

// the same from the views' own first tiles in the batch's table (global memory,
// L1-cached): the tile-stream batch kernel keeps its shared memory for the slots
__device__ __forceinline__ uint32_t view_of_tile(const PassParams* views, uint32_t nviews, uint32_t tile) {
    uint32_t lo = 0, hi = nviews;  // views[lo].tile_begin <= tile < views[hi].tile_begin
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&views[mid].tile_begin) <= tile) lo = mid;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ void finalize_rt(const PassParams& P, bool accum, const ShadowLane& s, size_t plane,
                                            float v) {
    if (accum) shadow_finalize<true>(P, s, plane, v);
    else shadow_finalize<false>(P, s, plane, v);
}

}  // namespace hy
