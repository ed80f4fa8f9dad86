// The tile-stream shadow kernel (the default shadow schedule), instantiated in
// hy_stream_raw.cu (raw per-light images), hy_stream_accum.cu (folded into the
// history) and hy_stream_two.cu (two-level structures), so the variants
// compile in parallel.
#pragma once
#include <cuda_runtime.h>

#include <type_traits>

#include "hy_device.cuh"
#include "hy_pass.h"
#include "hy_shade.cuh"
#include "hy_stream.cuh"

namespace hy {

// ---------------------------------------------------------------------------------
// Shadow rays, light-major over a tile: a warp takes an 8x4 tile and, light
// by light, traces all 32 x n_rays samples of its pixels (n_rays = spp for
// DECORRELATED; 1 for REFERENCE, whose samples are one ray), item q being
// sample q % n_rays of pixel q / n_rays; free lanes claim the items in order
// from a per-warp shared counter.  Lane i sets
// up light l for pixel i (its G-buffer texel, the skip tests of
// shadowRaygen.rgen:43-63) and publishes position, distance, sampleDisk's frame
// (tangent, bitangent, position + L: the same for every sample of the
// pixel-light) and the RNG state of its first sample in shared memory; every
// lane then traces items without waiting for the others (a lane whose rays
// are short takes more of them), counting unoccluded samples per pixel with shared-memory
// atomics; once the warp's items for light l are all traced, lane i folds
// pixel i's count into its factor.  A lane waits only at the end of a light
// (for the slowest sum of spp rays) instead of after every pixel-light (for
// the slowest single ray), and the samples in flight stay within a few
// adjacent pixels of one light.  Seeds as in k_shadow_group (LCG jump-ahead),
// so the rays equal those of k_shadow.
// ---------------------------------------------------------------------------------
template <bool COUNT, bool ACCUM, int MINB, bool TWO = false, bool SHORT = false>
__global__ void __launch_bounds__(128, MINB) k_shadow_stream(const SceneDev S, const PassParams P) {
    __shared__ StreamSlots sm;
    __shared__ uint2 s_stack[SHORT ? kShortStack * 128 : 1];
    // two-level: each lane's world ray set-up (WorldRaySlot, 64 B a lane): 8
    // blocks at 23.6 KB stay on the 196 KB shared-memory step (the 68-byte
    // padded layout of the same data took 24.1 KB and the 228 KB step)
    __shared__ float s_world[TWO ? 16 * 128 : 1];
    LaneStats ls;
    const uint32_t lane = threadIdx.x & 31;
    uint2 stk[kStackMax];
    ShadowLane s;
    Trav t;
    std::conditional_t<TWO, WorldRaySlot, RayPre> r{};
    if constexpr (TWO) r.p = s_world + threadIdx.x;
    uint32_t chunk_cur = 0, chunk_end = 0, nn = 0, nt = 0;
    for (;;) {
        if (chunk_cur == chunk_end) {
            uint32_t t0 = 0;
            if (lane == 0) t0 = atomicAdd(P.queue, P.chunk);
            t0 = __shfl_sync(0xffffffffu, t0, 0);
            if (t0 >= P.ntiles) break;
            chunk_cur = t0;
            chunk_end = min(t0 + P.chunk, P.ntiles);
        }
        if (SHORT)
            stream_tile<COUNT, TWO, ACCUM ? 1 : 0>(S, P, chunk_cur++, P.rng_mode == HY_RNG_REFERENCE, ACCUM, sm,
                                                   SplitStack{s_stack + threadIdx.x, stk}, t, r, s, ls, nn, nt, nullptr,
                                                   0u);
        else
            stream_tile<COUNT, TWO, ACCUM ? 1 : 0>(S, P, chunk_cur++, P.rng_mode == HY_RNG_REFERENCE, ACCUM, sm, stk, t,
                                                   r, s, ls, nn, nt, nullptr, 0u);
    }
    if (COUNT) { ls.nodes += nn; ls.tris += nt; }
    flush_stats(ls, P.stats);
}

// one-level kernels: the register cap as resident 128-thread blocks per SM
// (5-8), or 8 with the first stack entries in shared memory
template <bool ACCUM>
static void* stream_kernel_one(bool count, int minb, bool short_stack) {
    if (short_stack)
        return count ? (void*)k_shadow_stream<true, ACCUM, 8, false, true>
                     : (void*)k_shadow_stream<false, ACCUM, 8, false, true>;
    if (minb >= 8) return count ? (void*)k_shadow_stream<true, ACCUM, 8> : (void*)k_shadow_stream<false, ACCUM, 8>;
    if (minb == 7) return count ? (void*)k_shadow_stream<true, ACCUM, 7> : (void*)k_shadow_stream<false, ACCUM, 7>;
    if (minb >= 6) return count ? (void*)k_shadow_stream<true, ACCUM, 6> : (void*)k_shadow_stream<false, ACCUM, 6>;
    return count ? (void*)k_shadow_stream<true, ACCUM, 5> : (void*)k_shadow_stream<false, ACCUM, 5>;
}

}  // namespace hy
