// The batched shadow pass over tile streams with its launch shape as template
// parameters: threads per block, resident blocks per SM (the register cap) and
// how many entries of each lane's traversal stack sit in shared memory (the
// rest in the lane's local array).  The batch's autotuner sweeps these
// (hy_batch_autotune).  hy_batch_64.cu, hy_batch_128.cu and hy_batch_256.cu
// instantiate one block size each, so the variants compile in parallel.
#pragma once
#include <cuda_runtime.h>

#include "hy_device.cuh"
#include "hy_pass.h"
#include "hy_shade.cuh"
#include "hy_stream.cuh"

namespace hy {

// A warp pulls (view, tile) units from the batch's queue and walks each tile
// light by light (stream_tile) with that view's parameters; REFERENCE-RNG views
// trace one ray per pixel-light.  ANY_TWO: the batch holds a two-level scene
// (compiled separately: the second traversal raises the register pressure of
// the one-level case).  SHORT > 0: the first SHORT stack entries of each lane in
// dynamic shared memory (SHORT x BLOCK x 8 bytes), entry i of thread t at
// s_stack[i * BLOCK + t] (conflict-free).
static_assert(sizeof(PassParams) % 4 == 0 && sizeof(SceneDev) % 4 == 0, "copied to shared memory as words");
template <bool COUNT, int BLOCK, int MINB, int SHORT, bool ANY_TWO>
__global__ void __launch_bounds__(BLOCK, MINB) k_shadow_batch_stream(const BatchParams B) {
    constexpr int NW = BLOCK / 32;
    __shared__ StreamSlotsT<NW> sm;
    // per warp: its current view's parameters and scene, copied from the
    // global tables when the warp moves to another view
    __shared__ PassParams s_view[NW];
    __shared__ SceneDev s_scene[NW];
    extern __shared__ uint2 s_stack[];
    LaneStats ls;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint2 stk[kStackMax - SHORT];
    ShadowLane s;
    Trav t;
    RayPre r;
    uint32_t chunk_cur = 0, chunk_end = 0, nn = 0, nt = 0, cur_view = 0xffffffffu;
    for (;;) {
        if (chunk_cur == chunk_end) {
            uint32_t t0 = 0;
            if (lane == 0) t0 = atomicAdd(B.queue, B.chunk);
            t0 = __shfl_sync(0xffffffffu, t0, 0);
            if (t0 >= B.total_tiles) break;
            chunk_cur = t0;
            chunk_end = min(t0 + B.chunk, B.total_tiles);
        }
        const uint32_t unit = chunk_cur++;
        const uint32_t v = view_of_tile(B.views, B.nviews, unit);
        if (v != cur_view) {
            __syncwarp();
            const uint32_t* vs = reinterpret_cast<const uint32_t*>(&B.views[v]);
            uint32_t* vd = reinterpret_cast<uint32_t*>(&s_view[warp]);
            for (uint32_t i = lane; i < sizeof(PassParams) / 4; i += 32) vd[i] = vs[i];
            const uint32_t* ss = reinterpret_cast<const uint32_t*>(&B.scenes[B.views[v].scene]);
            uint32_t* sd = reinterpret_cast<uint32_t*>(&s_scene[warp]);
            for (uint32_t i = lane; i < sizeof(SceneDev) / 4; i += 32) sd[i] = ss[i];
            __syncwarp();
            cur_view = v;
        }
        const PassParams& P = s_view[warp];
        const SceneDev& S = s_scene[warp];
        const bool accum = !(P.flags & HY_FLAG_NO_ACCUM) && P.accum_frame > 0;
        const bool reference = P.rng_mode == HY_RNG_REFERENCE;
        if constexpr (SHORT > 0) {
            const SplitStackT<SHORT, BLOCK> sst{s_stack + threadIdx.x, stk};
            if (ANY_TWO && S.two_level)
                stream_tile<COUNT, true, 2>(S, P, unit - P.tile_begin, reference, accum, sm, sst, t, r, s, ls, nn, nt,
                                            nullptr, 0);
            else
                stream_tile<COUNT, false, 2>(S, P, unit - P.tile_begin, reference, accum, sm, sst, t, r, s, ls, nn,
                                             nt, nullptr, 0);
        } else {
            if (ANY_TWO && S.two_level)  // a two-level scene: the same tile with the instance walk
                stream_tile<COUNT, true, 2>(S, P, unit - P.tile_begin, reference, accum, sm, stk, t, r, s, ls, nn, nt,
                                            nullptr, 0);
            else
                stream_tile<COUNT, false, 2>(S, P, unit - P.tile_begin, reference, accum, sm, stk, t, r, s, ls, nn,
                                             nt, nullptr, 0);
        }
    }
    if (COUNT) { ls.nodes += nn; ls.tris += nt; }
    flush_stats(ls, B.stats);
}

// MB: the register cap as resident 128-thread blocks per SM (8: 64 registers,
// 6: 80); the kernel's own MINB scales it to BLOCK threads
template <int BLOCK, int MB>
static void* batch_stream_short(int shortd) {
    constexpr int MINB = MB * 128 / BLOCK;
    switch (shortd) {
        case 0: return (void*)k_shadow_batch_stream<false, BLOCK, MINB, 0, false>;
        case 8: return (void*)k_shadow_batch_stream<false, BLOCK, MINB, 8, false>;
        case 16: return (void*)k_shadow_batch_stream<false, BLOCK, MINB, 16, false>;
        case 32: return (void*)k_shadow_batch_stream<false, BLOCK, MINB, 32, false>;
        default: return nullptr;
    }
}

// The kernel of a launch shape, nullptr where none is compiled.  Counting
// launches and batches holding a two-level scene have one shape each (128
// threads, no shared stack; 64 / 96 registers).
template <int BLOCK>
static void* batch_stream_kernel_b(bool count, int minb, int shortd, bool two) {
    if (count || two) {
        if constexpr (BLOCK == 128) {
            if (shortd != 0) return nullptr;
            if (two)
                return count ? (void*)k_shadow_batch_stream<true, 128, 5, 0, true>
                             : (void*)k_shadow_batch_stream<false, 128, 5, 0, true>;
            return (void*)k_shadow_batch_stream<true, 128, 8, 0, false>;
        }
        return nullptr;
    }
    if (minb == 8) return batch_stream_short<BLOCK, 8>(shortd);
    if (minb == 6) return batch_stream_short<BLOCK, 6>(shortd);
    return nullptr;
}

}  // namespace hy
