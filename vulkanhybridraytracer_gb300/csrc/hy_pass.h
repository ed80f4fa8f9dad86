// Launch parameters shared by hy_pass.cu (device) and hy_api.cu (host).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "hy_device.cuh"

namespace hy {

// *_G: the sample-parallel shadow kernel (DECORRELATED rays, spp >= 2) with lane
// groups per pixel-light; *_P: the same rays from a per-warp ray pool
enum {
    MODE_SHADOW = 0, MODE_SHADE = 1, MODE_SHADOW_ACCUM = 2, MODE_SHADOW_G = 3, MODE_SHADOW_ACCUM_G = 4,
    MODE_SHADOW_P = 5, MODE_SHADOW_ACCUM_P = 6, MODE_SHADOW_S = 7, MODE_SHADOW_ACCUM_S = 8
};

struct PassParams {
    uint32_t W, H;
    const void* plane[6];
    uint32_t fmt[6];
    f3 cam_pos;              // viewInverse * (0,0,0,1)
    uint32_t frame_u;        // uint(int(cam.frame.x)): the per-pixel RNG frame
    uint32_t spp, max_bounces, rng_mode, flags;
    int32_t accum_frame;     // blur.comp frame
    uint32_t accum_fmt;
    void* shadow;            // raw shadow images
    void* hist;              // accumulated history
    float* out_f;
    uint8_t* out_8;
    uint32_t tiles_x, ntiles, chunk;
    uint32_t blur_w, blur_h; // texels the blur dispatch covers
    uint32_t group;          // lanes per pixel-light in the sample-parallel shadow kernel
    uint32_t inner;          // node visits per scheduling round of that kernel (>= 1)
    uint32_t short_stack;    // tile streams: the first stack entries in shared memory
    uint32_t shade_minb;     // shade kernel: resident blocks it is compiled for
    unsigned long long* stats;
    uint32_t* status;
    uint32_t* queue;
    // batches: the view's scene and its first tile in the batch's global tile range
    uint32_t scene, tile_begin;
    uint32_t num_lights;     // the pass uses the scene's first num_lights lights
};

// A batch: a device table of per-view PassParams over a device table of
// scenes; persistent warps pull (view, tile) units from one global queue.
constexpr uint32_t kMaxBatchViews = 1024;
struct BatchParams {
    const PassParams* views;
    const SceneDev* scenes;
    uint32_t nviews, total_tiles, chunk;
    unsigned long long* stats;
    uint32_t* status;
    uint32_t* queue;
};

struct AccumParams {
    uint32_t W, H, num_lights, fmt;
    int32_t frame;
    uint32_t blur_w, blur_h;
    const void* motion;
    uint32_t motion_fmt;
    const void* shadow;
    void* hist;
    const void* hist_prev;
};

struct GbufParams {
    uint32_t W, H;
    float inv_view[16], inv_proj[16];
    float* planes[6];
    uint32_t* status;
};

// The adjoint of the shading pass: dLoss/dImage in, per-material (diffuse
// rgb, roughness, metallic) and per-light (position xyz, intensity) gradients
// out.  `out` holds one partial gradient vector per block (grid rows) when
// the vector fits shared memory, else one vector the blocks add into.
constexpr int kGradMaxBounces = HY_GRAD_MAX_BOUNCES;
struct GradParams {
    PassParams P;
    const float4* grad;   // dLoss/dImage, RGBA32F (alpha ignored)
    float* out;
    uint32_t nparam;      // num_mats * 5 + num_lights * 4
    uint32_t light_off;   // num_mats * 5
};
cudaError_t grad_launch_shape(uint32_t nparam, int num_sms, uint32_t ntiles, int* grid, bool* smem,
                              size_t* smem_bytes);
cudaError_t launch_shade_grad(const SceneDev& S, const GradParams& G, int grid, bool smem, size_t smem_bytes,
                              float* out_mat, float* out_light, cudaStream_t s);

// Path-traced mode: P.out_8 is the accumulated B8G8R8A8 image, P.out_f the
// frame's colour; the camera matrices give the primary rays.
struct PtParams {
    PassParams P;
    float inv_view[16], inv_proj[16];
    int32_t frame;           // int(cam.frame.x): RNG frame and accumulation weight
};
cudaError_t pathtrace_occupancy(bool count, bool stream, bool two, int minb, int* blocks_per_sm);
cudaError_t launch_pathtrace(bool count, bool stream, int minb, const SceneDev& S, const PtParams& T, int grid,
                             cudaStream_t s);

cudaError_t launch_pixels(int mode, bool count, int minb, const SceneDev& S, const PassParams& P, int grid, int block,
                          cudaStream_t s);
cudaError_t pixel_occupancy(int mode, bool count, int minb, bool two, bool short_stack, int shade_minb, int block,
                            int* blocks_per_sm);
cudaError_t launch_accumulate(const AccumParams& A, cudaStream_t s);
cudaError_t launch_post(const uint8_t* in_bgra8, const float* in_rgba32f, uint32_t n, uint8_t* out_bgra8,
                        cudaStream_t s);
cudaError_t launch_trace(const SceneDev& S, const HyRay* rays, uint32_t n, bool any, bool count, HyHit* hits,
                         unsigned long long* stats, uint32_t* status, int grid, cudaStream_t s);
cudaError_t launch_gbuffer(const SceneDev& S, const GbufParams& G, cudaStream_t s);
// batches: block / shortd are the tile-stream kernel's threads per block and
// shared stack entries (the shade and lane-group kernels: 128 / 0)
cudaError_t launch_batch(bool shade, bool count, int minb, bool stream, bool two, int block, int shortd,
                         const BatchParams& B, int grid, cudaStream_t s);
cudaError_t batch_occupancy(bool shade, bool count, int minb, bool stream, bool two, int block, int shortd,
                            int* blocks_per_sm);
// tile-stream shadow kernels (hy_stream_raw.cu, hy_stream_accum.cu, hy_stream_two.cu)
void* stream_kernel_raw(bool count, int minb, bool short_stack);
void* stream_kernel_accum(bool count, int minb, bool short_stack);
void* stream_kernel_two(bool accum, bool count);
void* batch_stream_kernel_64(bool count, int minb, int shortd, bool two);
void* batch_stream_kernel_128(bool count, int minb, int shortd, bool two);
void* batch_stream_kernel_256(bool count, int minb, int shortd, bool two);

}  // namespace hy
