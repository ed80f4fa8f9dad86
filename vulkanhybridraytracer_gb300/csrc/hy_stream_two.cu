// Tile-stream shadow kernels over two-level structures (hy_stream_kernel.cuh):
// 8 resident blocks (64 registers; the 4K instanced frame 290 ms against 309 at
// 5 blocks and 296 at 6).
#include "hy_stream_kernel.cuh"

namespace hy {
void* stream_kernel_two(bool accum, bool count) {
    if (accum) return count ? (void*)k_shadow_stream<true, true, 8, true> : (void*)k_shadow_stream<false, true, 8, true>;
    return count ? (void*)k_shadow_stream<true, false, 8, true> : (void*)k_shadow_stream<false, false, 8, true>;
}
}  // namespace hy
