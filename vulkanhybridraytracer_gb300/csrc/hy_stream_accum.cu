// Tile-stream shadow kernels folding the shadow factors into the history
// (hy_stream_kernel.cuh).
#include "hy_stream_kernel.cuh"

namespace hy {
void* stream_kernel_accum(bool count, int minb, bool short_stack) {
    return stream_kernel_one<true>(count, minb, short_stack);
}
}  // namespace hy
