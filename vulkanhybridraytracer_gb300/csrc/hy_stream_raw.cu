// Tile-stream shadow kernels writing raw per-light images (hy_stream_kernel.cuh).
#include "hy_stream_kernel.cuh"

namespace hy {
void* stream_kernel_raw(bool count, int minb, bool short_stack) { return stream_kernel_one<false>(count, minb, short_stack); }
}  // namespace hy
