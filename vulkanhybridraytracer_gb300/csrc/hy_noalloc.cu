// hy_accumulate_pass_noalloc: the accumulation pass (blur.comp) for callers
// that must not allocate device memory.
//
// Engines built like VkPinut route every device allocation through their own
// allocator (the reference creates all buffers and images through VMA,
// src/vk_engine.cpp:307-312) and budget it per frame; a pass that called
// cudaMalloc/cudaFree behind that allocator's back would break the budget,
// and cudaFree also waits for the whole device, stalling the frame loop.
// hy_accumulate_pass needs a context, whose creation and scratch buffers
// allocate.  This entry point takes no context: the history snapshot that the
// reset-frame branch needs lives in the fixed array below, which every GPU
// that loads the library holds until the process exits.
#include <cuda_runtime.h>

#include <mutex>

#include "hy_pass.h"

namespace {

static __device__ __align__(256) unsigned char g_noalloc_scratch[HY_NOALLOC_SCRATCH_BYTES];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device.  In host code
// the array's name is only a host-side stand-in, so the address is looked up
// once per device (with that device current) and cached.  cudaDeviceReset
// unloads the module that holds the array, so a process that resets a device
// must not call the entry point on that device again: the cached address
// would point at freed memory.
int scratch_address(void** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return HY_ERR_CUDA; }
    if (dev < 0 || dev >= kMaxDevices) return HY_ERR_UNSUPPORTED;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_scratch_addr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) { cudaGetLastError(); return HY_ERR_CUDA; }
        g_scratch_addr[dev] = p;
    }
    *out = g_scratch_addr[dev];
    return HY_OK;
}

uint32_t plane_bytes(uint32_t f) {
    switch (f) {
        case HY_FMT_RGBA32F: return 16;
        case HY_FMT_RG32F: return 8;
        case HY_FMT_RGBA16F: return 8;
        case HY_FMT_RG16F: return 4;
        case HY_FMT_RGBA8: return 4;
        default: return 0;
    }
}

}  // namespace

extern "C" int hy_accumulate_pass_noalloc(const HyGBuffer* gb, const HyPassConfig* cfg, const void* d_shadow,
                                          HyAccum* acc, void* stream) {
    if (!gb || !cfg || !d_shadow || !acc || !acc->history || acc->format > HY_ACCUM_F32 || acc->num_lights == 0)
        return HY_ERR_INVALID_ARG;
    if (gb->width == 0 || gb->height == 0 || !gb->plane[3] || plane_bytes(gb->format[3]) == 0)
        return HY_ERR_INVALID_ARG;
    // the same bound as every other pass: pixel indices are 32-bit
    if ((unsigned long long)gb->width * gb->height >= (1ull << 31)) return HY_ERR_INVALID_ARG;
    if ((uintptr_t)gb->plane[3] % plane_bytes(gb->format[3]) != 0) return HY_ERR_INVALID_ARG;
    hy::AccumParams A;
    A.W = gb->width;
    A.H = gb->height;
    A.num_lights = acc->num_lights;
    A.fmt = acc->format;
    A.frame = cfg->accum_frame;
    if (cfg->flags & HY_FLAG_FULL_BLUR_DISPATCH) { A.blur_w = A.W; A.blur_h = A.H; }
    else { A.blur_w = (A.W / 16) * 16; A.blur_h = (A.H / 16) * 16; }
    A.motion = gb->plane[3];
    A.motion_fmt = gb->format[3];
    A.shadow = d_shadow;
    A.hist = acc->history;
    A.hist_prev = acc->history;
    cudaStream_t s = (cudaStream_t)stream;
    if (A.frame <= 0) {
        // the reprojected read must see the history as it was before this call
        const unsigned long long bytes =
            (unsigned long long)A.W * A.H * A.num_lights * (acc->format == HY_ACCUM_U8 ? 1u : 4u);
        if (bytes > HY_NOALLOC_SCRATCH_BYTES) return HY_ERR_TOO_LARGE;
        void* scratch = nullptr;
        int rc = scratch_address(&scratch);
        if (rc) return rc;
        if (cudaMemcpyAsync(scratch, acc->history, (size_t)bytes, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
            cudaGetLastError();
            return HY_ERR_CUDA;
        }
        A.hist_prev = scratch;
    }
    if (hy::launch_accumulate(A, s) != cudaSuccess) { cudaGetLastError(); return HY_ERR_CUDA; }
    return HY_OK;
}
