// The batched tile-stream shadow kernels of 64 threads per block (hy_batch.cuh).
#include "hy_batch.cuh"

namespace hy {
void* batch_stream_kernel_64(bool count, int minb, int shortd, bool two) {
    return batch_stream_kernel_b<64>(count, minb, shortd, two);
}
}  // namespace hy
