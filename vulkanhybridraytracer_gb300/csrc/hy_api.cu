// C ABI of libhybridrt: context, scene upload, acceleration structure, passes.
//
// The three submissions of Renderer::rasterize_hybrid (src/renderer.cpp:559-580)
// become stream-ordered kernel launches on the context's stream; there is no
// host round trip between them (the reference waits for the queue to idle
// after each).  Scene upload mirrors Renderer::load_data_to_gpu
// (src/renderer.cpp:1477-1530) and the per-entity buffers of
// create_hybrid_descriptors (src/renderer.cpp:3015-3048).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "hy_internal.h"
#include "hy_pass.h"

using namespace hy;

namespace hy {

int ctx_alloc(HyCtx* c, DevBuf& b, size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (b.p && b.bytes >= bytes) return HY_OK;
    c->alloc_calls++;
    if (c->fail_after && c->alloc_calls >= c->fail_after) { c->fail_after = 0; return HY_ERR_OOM; }
    size_t old = b.bytes;
    if (c->max_bytes && c->used_bytes - old + bytes > c->max_bytes) return HY_ERR_OOM;
    if (b.p) { cudaFree(b.p); b.p = nullptr; b.bytes = 0; c->used_bytes -= old; }
    cudaError_t e = cudaMalloc(&b.p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        b.p = nullptr;
        return e == cudaErrorMemoryAllocation ? HY_ERR_OOM : HY_ERR_CUDA;
    }
    b.bytes = bytes;
    c->used_bytes += bytes;
    return HY_OK;
}

void ctx_free(HyCtx* c, DevBuf& b) {
    if (b.p) { cudaFree(b.p); c->used_bytes -= b.bytes; }
    b.p = nullptr;
    b.bytes = 0;
}

}  // namespace hy

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

template <class T> int upload(HyCtx* c, DevBuf& b, const T* src, size_t count) {
    int rc = ctx_alloc(c, b, count * sizeof(T));
    if (rc) return rc;
    if (count) HY_CUDA_TRY(cudaMemcpyAsync(b.p, src, count * sizeof(T), cudaMemcpyHostToDevice, c->stream));
    HY_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return HY_OK;
}

inline bool finite_all(const float* p, size_t n) {
    for (size_t i = 0; i < n; i++)
        if (!std::isfinite(p[i])) return false;
    return true;
}

void inverse4(const double* a, double* inv) {
    inv[0] = a[5] * a[10] * a[15] - a[5] * a[11] * a[14] - a[9] * a[6] * a[15] + a[9] * a[7] * a[14] + a[13] * a[6] * a[11] - a[13] * a[7] * a[10];
    inv[4] = -a[4] * a[10] * a[15] + a[4] * a[11] * a[14] + a[8] * a[6] * a[15] - a[8] * a[7] * a[14] - a[12] * a[6] * a[11] + a[12] * a[7] * a[10];
    inv[8] = a[4] * a[9] * a[15] - a[4] * a[11] * a[13] - a[8] * a[5] * a[15] + a[8] * a[7] * a[13] + a[12] * a[5] * a[11] - a[12] * a[7] * a[9];
    inv[12] = -a[4] * a[9] * a[14] + a[4] * a[10] * a[13] + a[8] * a[5] * a[14] - a[8] * a[6] * a[13] - a[12] * a[5] * a[10] + a[12] * a[6] * a[9];
    inv[1] = -a[1] * a[10] * a[15] + a[1] * a[11] * a[14] + a[9] * a[2] * a[15] - a[9] * a[3] * a[14] - a[13] * a[2] * a[11] + a[13] * a[3] * a[10];
    inv[5] = a[0] * a[10] * a[15] - a[0] * a[11] * a[14] - a[8] * a[2] * a[15] + a[8] * a[3] * a[14] + a[12] * a[2] * a[11] - a[12] * a[3] * a[10];
    inv[9] = -a[0] * a[9] * a[15] + a[0] * a[11] * a[13] + a[8] * a[1] * a[15] - a[8] * a[3] * a[13] - a[12] * a[1] * a[11] + a[12] * a[3] * a[9];
    inv[13] = a[0] * a[9] * a[14] - a[0] * a[10] * a[13] - a[8] * a[1] * a[14] + a[8] * a[2] * a[13] + a[12] * a[1] * a[10] - a[12] * a[2] * a[9];
    inv[2] = a[1] * a[6] * a[15] - a[1] * a[7] * a[14] - a[5] * a[2] * a[15] + a[5] * a[3] * a[14] + a[13] * a[2] * a[7] - a[13] * a[3] * a[6];
    inv[6] = -a[0] * a[6] * a[15] + a[0] * a[7] * a[14] + a[4] * a[2] * a[15] - a[4] * a[3] * a[14] - a[12] * a[2] * a[7] + a[12] * a[3] * a[6];
    inv[10] = a[0] * a[5] * a[15] - a[0] * a[7] * a[13] - a[4] * a[1] * a[15] + a[4] * a[3] * a[13] + a[12] * a[1] * a[7] - a[12] * a[3] * a[5];
    inv[14] = -a[0] * a[5] * a[14] + a[0] * a[6] * a[13] + a[4] * a[1] * a[14] - a[4] * a[2] * a[13] - a[12] * a[1] * a[6] + a[12] * a[2] * a[5];
    inv[3] = -a[1] * a[6] * a[11] + a[1] * a[7] * a[10] + a[5] * a[2] * a[11] - a[5] * a[3] * a[10] - a[9] * a[2] * a[7] + a[9] * a[3] * a[6];
    inv[7] = a[0] * a[6] * a[11] - a[0] * a[7] * a[10] - a[4] * a[2] * a[11] + a[4] * a[3] * a[10] + a[8] * a[2] * a[7] - a[8] * a[3] * a[6];
    inv[11] = -a[0] * a[5] * a[11] + a[0] * a[7] * a[9] + a[4] * a[1] * a[11] - a[4] * a[3] * a[9] - a[8] * a[1] * a[7] + a[8] * a[3] * a[5];
    inv[15] = a[0] * a[5] * a[10] - a[0] * a[6] * a[9] - a[4] * a[1] * a[10] + a[4] * a[2] * a[9] + a[8] * a[1] * a[6] - a[8] * a[2] * a[5];
    double det = a[0] * inv[0] + a[1] * inv[4] + a[2] * inv[8] + a[3] * inv[12];
    double r = 1.0 / det;
    for (int i = 0; i < 16; i++) inv[i] *= r;
}

// rows of inverse(M) (world -> object) of each transform, 3 x (m0 m1 m2 t)
std::vector<float> world_to_object(const float* xf, uint32_t n) {
    std::vector<float> out((size_t)n * 12);
    for (uint32_t t = 0; t < n; t++) {
        double m[16], inv[16];
        for (int i = 0; i < 16; i++) m[i] = xf[(size_t)t * 16 + i];
        inverse4(m, inv);
        for (int r = 0; r < 3; r++)
            for (int k = 0; k < 4; k++) out[(size_t)t * 12 + r * 4 + k] = (float)inv[k * 4 + r];
    }
    return out;
}

// mat3(transpose(inverse(M))) of each transform, column-major 3x3
std::vector<float> normal_matrices(const float* xf, uint32_t n) {
    std::vector<float> out((size_t)n * 9);
    for (uint32_t t = 0; t < n; t++) {
        double m[16], inv[16];
        for (int i = 0; i < 16; i++) m[i] = xf[(size_t)t * 16 + i];
        inverse4(m, inv);
        for (int c = 0; c < 3; c++)
            for (int r = 0; r < 3; r++) out[(size_t)t * 9 + c * 3 + r] = (float)inv[r * 4 + c];
    }
    return out;
}

// HY_ANYHIT_AUTO: far first while the nodes (80 B) and leaf records (48 B)
// fit in L2 — measured on a 1.5M-triangle scene (90 MB): 8.7 % fewer node
// visits, 9.6 % faster; on a 7.35M-triangle one (440 MB): 26 % fewer visits
// but 2 % slower, each visit's fetches going to DRAM — and near first for
// two-level structures
static uint32_t anyhit_flip(const HyCtx* c) {
    if (c->anyhit_order == HY_ANYHIT_FAR_FIRST) return 7u;
    if (c->anyhit_order == HY_ANYHIT_NEAR_FIRST || c->two_level) return 0u;
    const uint64_t bytes = (uint64_t)c->n_bvh8 * 80u + (uint64_t)c->n_records * 48u;
    return c->l2_bytes > 0 && bytes <= (uint64_t)c->l2_bytes ? 7u : 0u;
}

SceneDev scene_dev(HyCtx* c) {
    SceneDev S;
    S.nodes = c->nodes.as<Node8>();
    S.tris = c->tris.as<float4>();
    S.vattr = c->vattr.as<float4>();
    S.idx = c->idx.as<uint32_t>();
    S.prims = c->prims.as<HyPrimitive>();
    S.tri_prim = c->tri_prim.as<uint32_t>();
    S.prim_tri0 = c->prim_tri0.as<uint32_t>();
    S.nrm = c->nrm.as<float>();
    S.mats = c->mats.as<HyMaterial>();
    S.lights = c->lights.as<HyLight>();
    S.env0 = c->env[0].as<uchar4>();
    S.env1 = c->env[1].as<uchar4>();
    S.num_mats = c->nmats;
    S.num_lights = c->nlights;
    S.tex_px = c->tex_px.as<uchar4>();
    S.tex_tab = c->tex_tab.as<uint4>();
    S.num_tex = c->ntex;
    S.num_nodes = c->bvh_ok ? c->n_bvh8 : 0;
    S.num_tris = c->bvh_ok ? c->n_records : 0;
    S.inst = c->inst.as<float4>();
    S.num_inst = c->bvh_ok && c->two_level ? c->ninst : 0;
    S.two_level = c->bvh_ok && c->two_level ? 1u : 0u;
    S.anyhit_flip = anyhit_flip(c);
    S.max_iters = c->dbg_max_iters ? c->dbg_max_iters : kMaxIters;
    S.stack_cap = c->dbg_stack_cap ? (int)std::min<uint32_t>(c->dbg_stack_cap, kStackMax) : kStackMax;
    for (int i = 0; i < 2; i++) { S.env_w[i] = c->env_w[i]; S.env_h[i] = c->env_h[i]; }
    return S;
}

// zero the counters, status word and queue slots of a call
int reset_counters(HyCtx* c) {
    HY_CUDA_TRY(cudaMemsetAsync(c->dstats.p, 0, c->dstats.bytes, c->stream));
    return HY_OK;
}
unsigned long long* dev_stats(HyCtx* c) { return c->dstats.as<unsigned long long>(); }
uint32_t* dev_status(HyCtx* c) { return (uint32_t*)(c->dstats.as<unsigned long long>() + ST_COUNT); }
uint32_t* dev_queue(HyCtx* c, int k) { return dev_status(c) + 1 + k; }

int status_to_code(uint32_t s) {
    if (s & HY_STATUS_STACK_OVERFLOW) return HY_ERR_STACK_OVERFLOW;
    if (s & HY_STATUS_TIMEOUT) return HY_ERR_TIMEOUT;
    if (s & HY_STATUS_QUEUE_OVERFLOW) return HY_ERR_QUEUE_OVERFLOW;
    if (s & HY_STATUS_NAN_INPUT) return HY_ERR_NAN_INPUT;
    if (s & HY_STATUS_BAD_INDEX) return HY_ERR_BAD_INDEX;
    return HY_OK;
}

// read back counters + status (synchronises the stream)
int finish_call(HyCtx* c, HyStats* st, bool sync) {
    HY_CUDA_TRY(cudaGetLastError());
    if (!sync && !st) return HY_OK;
    HY_CUDA_TRY(cudaMemcpyAsync(c->h_stats, c->dstats.p, ST_COUNT * 8 + 4, cudaMemcpyDeviceToHost, c->stream));
    HY_CUDA_TRY(cudaStreamSynchronize(c->stream));
    uint32_t status;
    std::memcpy(&status, c->h_stats + ST_COUNT, 4);
    if (st) {
        st->shadow_rays = c->h_stats[ST_SHADOW];
        st->reflection_rays = c->h_stats[ST_REFL];
        st->hit_shadow_rays = c->h_stats[ST_HITSHADOW];
        st->nodes_visited = c->h_stats[ST_NODES];
        st->tris_tested = c->h_stats[ST_TRIS];
        st->error_flags = status;
        st->_pad = 0;
    }
    return status_to_code(status);
}

uint32_t fmt_bytes(uint32_t f) {
    switch (f) {
        case HY_FMT_RGBA32F: return 16;
        case HY_FMT_RG32F: return 8;
        case HY_FMT_RGBA16F: return 8;
        case HY_FMT_RG16F: return 4;
        case HY_FMT_RGBA8: return 4;
        default: return 0;
    }
}

int check_gbuffer(const HyGBuffer* gb, bool need_all) {
    if (!gb || gb->width == 0 || gb->height == 0) return HY_ERR_INVALID_ARG;
    if ((uint64_t)gb->width * gb->height >= (1ull << 31)) return HY_ERR_INVALID_ARG;
    for (int p = 0; p < 6; p++) {
        bool needed = need_all || p == 0 || p == 1 || p == 3;
        if (!needed) continue;
        if (!gb->plane[p] || fmt_bytes(gb->format[p]) == 0) return HY_ERR_INVALID_ARG;
        if (((uintptr_t)gb->plane[p]) % fmt_bytes(gb->format[p]) != 0) return HY_ERR_INVALID_ARG;
    }
    return HY_OK;
}

int check_cfg(const HyPassConfig* cfg) {
    if (!cfg) return HY_ERR_INVALID_ARG;
    if (cfg->shadow_spp == 0 || cfg->shadow_spp > 4096) return HY_ERR_INVALID_ARG;
    if (cfg->max_bounces > 64) return HY_ERR_INVALID_ARG;
    if (cfg->rng_mode > HY_RNG_DECORRELATED) return HY_ERR_INVALID_ARG;
    return HY_OK;
}

int check_scene_ready(HyCtx* c) {
    if (!c->geometry_ok || !c->bvh_ok) return HY_ERR_NOT_READY;
    if (c->nmats == 0) return HY_ERR_NOT_READY;
    if (c->max_material_id >= c->nmats) return HY_ERR_INVALID_ARG;  // a primitive names a missing material
    // the shaders sample textures x (diffuse), z (emissive), w (metallic-roughness) when > -1
    for (const HyMaterial& m : c->h_mats)
        for (int k : {0, 2, 3})
            if (m.textures[k] > -1.f && !(m.textures[k] < (float)c->ntex)) return HY_ERR_INVALID_ARG;
    return HY_OK;
}

int grid_for(HyCtx* c, int mode, bool count, int minb, bool short_stack, int shade_minb, int block) {
    int per = 0;
    if (pixel_occupancy(mode, count, minb, c->two_level, short_stack, shade_minb, block, &per) != cudaSuccess ||
        per <= 0)
        per = 1;
    return per * c->num_sms;
}

// tile streams: node visits per scheduling round (1080p shadow kernel at 8
// resident blocks over the SAH structure: 8 / 12 / 16 visits 22.8 / 22.5 / 23.2 ms)
constexpr uint32_t kStreamSteps = 12;

PassParams make_params(HyCtx* c, const HyGBuffer* gb, const HyCamera* cam, const HyPassConfig* cfg,
                       uint32_t accum_fmt, void* shadow, void* hist, float* out_f, uint8_t* out_8) {
    PassParams P;
    std::memset(&P, 0, sizeof(P));
    P.W = gb->width;
    P.H = gb->height;
    for (int i = 0; i < 6; i++) { P.plane[i] = gb->plane[i]; P.fmt[i] = gb->format[i]; }
    // viewInverse * vec4(0,0,0,1), same op order as the device mat-vec
    float cp[3];
    for (int i = 0; i < 3; i++) {
        float a = cam->inv_view[0 * 4 + i] * 0.f;
        a = a + cam->inv_view[1 * 4 + i] * 0.f;
        a = a + cam->inv_view[2 * 4 + i] * 0.f;
        a = a + cam->inv_view[3 * 4 + i] * 1.f;
        cp[i] = a;
    }
    P.cam_pos = f3{cp[0], cp[1], cp[2]};
    P.frame_u = (uint32_t)(int32_t)cam->frame[0];
    P.spp = cfg->shadow_spp;
    P.max_bounces = cfg->max_bounces;
    P.rng_mode = cfg->rng_mode;
    P.flags = cfg->flags;
    P.accum_frame = cfg->accum_frame;
    P.accum_fmt = accum_fmt;
    P.shadow = shadow;
    P.hist = hist;
    P.out_f = out_f;
    P.out_8 = out_8;
    P.tiles_x = (P.W + 7) / 8;
    P.ntiles = P.tiles_x * ((P.H + 3) / 4);
    P.chunk = cfg->queue_chunk ? cfg->queue_chunk : 1;
    // node visits per scheduling round of the persistent shadow kernels: 4
    // measured 9.5 % ahead of 1 for the lane groups on the 1080p workload
    // (2: 6.8 %, 3: 8.8 %, 8: 8.9 %); the tile streams default to 8 (at 8
    // resident blocks: 4: -3.9 %, 6: -1.7 %, 12: -3.6 %, 16: -2.7 %)
    P.inner = cfg->visits_per_round ? std::min(cfg->visits_per_round, 16u) : 4u;
    if (cfg->flags & HY_FLAG_FULL_BLUR_DISPATCH) { P.blur_w = P.W; P.blur_h = P.H; }
    else { P.blur_w = (P.W / 16) * 16; P.blur_h = (P.H / 16) * 16; }
    P.stats = dev_stats(c);
    P.num_lights = c->nlights;
    P.status = dev_status(c);
    return P;
}

// ---- per-kernel timing ----
// the first seven are the MODE_* values of hy_pass.h
enum { PK_ACCUM = MODE_SHADOW_ACCUM_S + 1, PK_GRAD, PK_PATHTRACE, PK_COUNT };
const char* const kProfNames[PK_COUNT] = {"k_shadow",       "k_pixels<shade>",       "k_shadow<accum>",
                                          "k_shadow_group", "k_shadow_group<accum>", "k_shadow_pool",
                                          "k_shadow_pool<accum>", "k_shadow_stream", "k_shadow_stream<accum>",
                                          "k_accumulate", "k_shade_grad", "k_pathtrace"};
static_assert(MODE_SHADOW == 0 && MODE_SHADE == 1 && MODE_SHADOW_ACCUM == 2 && MODE_SHADOW_G == 3 &&
                  MODE_SHADOW_ACCUM_G == 4 && MODE_SHADOW_P == 5 && MODE_SHADOW_ACCUM_P == 6 &&
                  MODE_SHADOW_S == 7 && MODE_SHADOW_ACCUM_S == 8,
              "profile names follow the pass modes");

cudaEvent_t prof_event(HyCtx* c) {
    if (c->prof_used == c->prof_pool.size()) {
        cudaEvent_t e = nullptr;
        if (cudaEventCreate(&e) != cudaSuccess) { cudaGetLastError(); return nullptr; }
        c->prof_pool.push_back(e);
    }
    return c->prof_pool[c->prof_used++];
}

// brackets the launches in its scope with events when profiling is on
struct ProfScope {
    HyCtx* c;
    int kind;
    cudaEvent_t a = nullptr;
    ProfScope(HyCtx* ctx, int k) : c(ctx), kind(k) {
        if (c->prof_on && c->prof_recs.size() < 4096 && (a = prof_event(c))) cudaEventRecord(a, c->stream);
    }
    ~ProfScope() {
        if (!a) return;
        cudaEvent_t b = prof_event(c);
        if (!b) return;
        cudaEventRecord(b, c->stream);
        c->prof_recs.push_back(HyCtx::ProfRec{kind, a, b});
    }
};

int run_pixels(HyCtx* c, int mode, const PassParams& P0, const HyPassConfig* cfg, int queue_slot) {
    bool count = (cfg->flags & HY_FLAG_COUNT_TRAVERSAL) != 0;
    int block = cfg->block_size ? (int)cfg->block_size : 128;
    if (block % 32 || block > 128) return HY_ERR_INVALID_ARG;  // kernels are built for <= 128 threads
    if (c->two_level && (cfg->flags & HY_FLAG_RAY_POOL)) return HY_ERR_UNSUPPORTED;
    PassParams P = P0;
    P.queue = dev_queue(c, queue_slot);
    // shadow schedules: tile streams (the default, any RNG mode and spp), or for
    // DECORRELATED spp >= 2 the lane groups / the per-warp ray pool on request,
    // or one lane per pixel (HY_FLAG_PIXEL_PARALLEL)
    const bool sampled = P.rng_mode == HY_RNG_DECORRELATED && P.spp >= 2;
    if ((mode == MODE_SHADOW || mode == MODE_SHADOW_ACCUM) && !(cfg->flags & HY_FLAG_PIXEL_PARALLEL)) {
        if (sampled && (cfg->flags & HY_FLAG_RAY_POOL)) {
            mode = mode == MODE_SHADOW ? MODE_SHADOW_P : MODE_SHADOW_ACCUM_P;
        } else if (!sampled || !(cfg->flags & HY_FLAG_LANE_GROUPS)) {
            mode = mode == MODE_SHADOW ? MODE_SHADOW_S : MODE_SHADOW_ACCUM_S;
        } else {
            mode = mode == MODE_SHADOW ? MODE_SHADOW_G : MODE_SHADOW_ACCUM_G;
            uint32_t G = 2;
            while (G < P.spp && G < 32) G <<= 1;
            if (cfg->group_lanes) {
                G = cfg->group_lanes;
                if (G < 2 || G > 32 || (G & (G - 1))) return HY_ERR_INVALID_ARG;
            }
            P.group = G;
        }
    }
    // measured fastest on the 1080p workload: 6 resident blocks (80 registers)
    // for the lane-group kernel (1.4 % ahead of 8), 8 (64 registers) otherwise;
    // 12 node visits per round for the tile streams (4 for the others)
    const bool grouped = mode == MODE_SHADOW_G || mode == MODE_SHADOW_ACCUM_G;
    const bool streams = mode == MODE_SHADOW_S || mode == MODE_SHADOW_ACCUM_S;
    int minb = cfg->min_blocks ? (int)cfg->min_blocks : (grouped ? 6 : 8);
    if (streams && !cfg->visits_per_round) P.inner = kStreamSteps;
    if (cfg->stack_depth && cfg->stack_depth != 8) return HY_ERR_UNSUPPORTED;
    P.short_stack = streams && !c->two_level && cfg->stack_depth == 8;
    // the shade kernel at 8 resident blocks (64 registers): 1.69 ms per 1080p frame
    // against 2.28 uncapped (167 registers), 2.03 / 1.91 / 1.86 at 4 / 5 / 6
    P.shade_minb = 8;
    int grid = grid_for(c, mode, count, minb, P.short_stack != 0, (int)P.shade_minb, block);
    grid = std::max(1, std::min<int>(grid, (int)((P.ntiles * 32ull + block - 1) / block)));
    ProfScope prof(c, mode);
    HY_CUDA_TRY(launch_pixels(mode, count, minb, scene_dev(c), P, grid, block, c->stream));
    return HY_OK;
}

int ensure_size(HyCtx* c, DevBuf& b, size_t bytes) { return ctx_alloc(c, b, bytes); }

}  // namespace

extern "C" {

const char* hy_error_string(int code) {
    switch (code) {
        case HY_OK: return "ok";
        case HY_ERR_INVALID_ARG: return "invalid argument";
        case HY_ERR_OOM: return "out of device memory";
        case HY_ERR_CUDA: return "CUDA error";
        case HY_ERR_TIMEOUT: return "device loop exceeded its iteration budget";
        case HY_ERR_STACK_OVERFLOW: return "traversal stack overflow";
        case HY_ERR_QUEUE_OVERFLOW: return "ray queue overflow";
        case HY_ERR_NAN_INPUT: return "non-finite input";
        case HY_ERR_NOT_READY: return "scene or acceleration structure not ready";
        case HY_ERR_UNSUPPORTED: return "unsupported";
        case HY_ERR_TOO_LARGE: return "input exceeds the fixed scratch of the allocation-free entry point";
        case HY_ERR_BAD_INDEX: return "acceleration structure index out of range (corrupt structure)";
        default: return "unknown error";
    }
}

int hy_get_abi_version(void) { return HY_ABI_VERSION; }

int hy_create(HyCtx** out, const HyCreateInfo* info) {
    if (!out) return HY_ERR_INVALID_ARG;
    *out = nullptr;
    int dev = info ? info->device : 0;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || dev < 0 || dev >= ndev) {
        cudaGetLastError();
        return HY_ERR_CUDA;
    }
    HyCtx* c = new (std::nothrow) HyCtx();
    if (!c) return HY_ERR_OOM;
    c->device = dev;
    DeviceGuard g(dev);
    if (info) c->max_bytes = info->max_device_bytes;
    if (info && info->stream) {
        c->stream = (cudaStream_t)info->stream;
    } else {
        if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { delete c; return HY_ERR_CUDA; }
        c->own_stream = true;
    }
    cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, dev);
    if (c->num_sms <= 0) c->num_sms = 1;
    cudaDeviceGetAttribute(&c->l2_bytes, cudaDevAttrL2CacheSize, dev);
    int rc = ctx_alloc(c, c->dstats, ST_COUNT * 8 + 4 + WQ_COUNT * 4);
    if (rc == HY_OK && cudaMallocHost((void**)&c->h_stats, 64) != cudaSuccess) rc = HY_ERR_CUDA;
    if (rc) { hy_destroy(c); return rc; }
    *out = c;
    return HY_OK;
}

void hy_destroy(HyCtx* c) {
    if (!c) return;
    DeviceGuard g(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    DevBuf* bufs[] = {&c->verts, &c->vattr, &c->idx, &c->prims, &c->xf, &c->nrm, &c->prim_tri0, &c->tri_prim,
                      &c->mats, &c->lights, &c->env[0], &c->env[1], &c->world, &c->tribox, &c->centroid,
                      &c->keys[0], &c->keys[1], &c->vals[0], &c->vals[1], &c->bvh2, &c->parent, &c->flags,
                      &c->bounds, &c->lvl_ref[0], &c->lvl_ref[1], &c->plan, &c->ni, &c->nt, &c->ni_scan,
                      &c->nt_scan, &c->scan_tmp, &c->hist, &c->total, &c->nodes, &c->tris, &c->node_ref,
                      &c->node_plan, &c->dstats,
                      &c->raw_shadow, &c->hist_prev, &c->host_in[0], &c->host_in[1], &c->host_in[2],
                      &c->host_in[3], &c->host_in[4], &c->host_in[5], &c->host_out_f, &c->host_out_8,
                      &c->grad_partial, &c->tex_px, &c->tex_tab, &c->xinv, &c->inst, &c->inst_box,
                      &c->inst_prim, &c->prim_mesh, &c->blas_node0, &c->mesh_vrange, &c->inst_chunks,
                      &c->inst_keys, &c->sah_ranges[0], &c->sah_ranges[1], &c->sah_small, &c->sah_bins,
                      &c->sah_split, &c->sah_chunks, &c->sah_first, &c->sah_ccnt, &c->sah_coff, &c->sah_ctr,
                      &c->dp_cost, &c->dp_k};
    for (DevBuf* b : bufs) ctx_free(c, *b);
    if (c->h_stats) cudaFreeHost(c->h_stats);
    for (cudaEvent_t e : c->prof_pool) cudaEventDestroy(e);
    if (c->batch_exec) cudaGraphExecDestroy(c->batch_exec);
    if (c->batch_done) cudaEventDestroy(c->batch_done);
    if (c->copy_start) cudaEventDestroy(c->copy_start);
    if (c->copy_done) cudaEventDestroy(c->copy_done);
    if (c->copy_stream) { cudaStreamSynchronize(c->copy_stream); cudaStreamDestroy(c->copy_stream); }
    if (c->h_batch_tab) cudaFreeHost(c->h_batch_tab);
    ctx_free(c, c->batch_tab);
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

int hy_synchronize(HyCtx* c) {
    if (!c) return HY_ERR_INVALID_ARG;
    DeviceGuard g(c->device);
    HY_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return HY_OK;
}

int hy_debug_fail_alloc_after(HyCtx* c, uint32_t n) {
    if (!c) return HY_ERR_INVALID_ARG;
    c->fail_after = n ? c->alloc_calls + n : 0;
    return HY_OK;
}

int hy_debug_set_traversal_limits(HyCtx* c, uint32_t max_node_visits, uint32_t max_stack_depth) {
    if (!c || max_stack_depth > (uint32_t)kStackMax) return HY_ERR_INVALID_ARG;
    c->dbg_max_iters = max_node_visits;
    c->dbg_stack_cap = max_stack_depth;
    return HY_OK;
}

int hy_scene_set_geometry(HyCtx* c, const HyVertex* verts, uint32_t nv, const uint32_t* indices, uint32_t ni,
                          const HyPrimitive* prims, uint32_t np, const float* xf, uint32_t nx) {
    if (!c || (nv && !verts) || (ni && !indices) || (np && !prims) || (nx && !xf)) return HY_ERR_INVALID_ARG;
    if (np == 0 || nx == 0) return HY_ERR_INVALID_ARG;
    DeviceGuard g(c->device);
    // validation: index ranges, transform ids, finiteness
    std::vector<uint32_t> prim_tri0(np);
    uint64_t nt = 0;
    uint32_t max_mat = 0;
    for (uint32_t p = 0; p < np; p++) {
        const HyPrimitive& pr = prims[p];
        if (pr.index_count % 3 != 0) return HY_ERR_INVALID_ARG;
        if ((uint64_t)pr.first_index + pr.index_count > ni) return HY_ERR_INVALID_ARG;
        if (pr.transform_id >= nx) return HY_ERR_INVALID_ARG;
        max_mat = std::max(max_mat, pr.material_id);
        for (uint32_t k = 0; k < pr.index_count; k++)
            if ((uint64_t)indices[pr.first_index + k] + pr.vertex_offset >= nv) return HY_ERR_INVALID_ARG;
        prim_tri0[p] = (uint32_t)nt;
        nt += pr.index_count / 3;
    }
    if (nt == 0 || nt >= (1ull << 31)) return HY_ERR_INVALID_ARG;
    for (uint32_t v = 0; v < nv; v++)
        if (!finite_all(verts[v].pos, 3)) return HY_ERR_NAN_INPUT;
    if (!finite_all(xf, (size_t)nx * 16)) return HY_ERR_NAN_INPUT;
    std::vector<uint32_t> tri_prim((size_t)nt);
    for (uint32_t p = 0; p < np; p++)
        for (uint32_t k = 0; k < prims[p].index_count / 3; k++) tri_prim[prim_tri0[p] + k] = p;
    std::vector<float> vattr((size_t)nv * 8, 0.f);
    for (uint32_t v = 0; v < nv; v++) {
        vattr[(size_t)v * 8 + 0] = verts[v].normal[0];
        vattr[(size_t)v * 8 + 1] = verts[v].normal[1];
        vattr[(size_t)v * 8 + 2] = verts[v].normal[2];
        vattr[(size_t)v * 8 + 3] = verts[v].color[0];
        vattr[(size_t)v * 8 + 4] = verts[v].uv[0];
        vattr[(size_t)v * 8 + 5] = verts[v].uv[1];
        vattr[(size_t)v * 8 + 6] = verts[v].color[1];
        vattr[(size_t)v * 8 + 7] = verts[v].color[2];
    }
    std::vector<float> nrm = normal_matrices(xf, nx);
    std::vector<float> xinv = world_to_object(xf, nx);
    int rc;
    c->geometry_ok = false;
    c->bvh_ok = false;
    c->two_level = false;
    if ((rc = upload(c, c->xinv, xinv.data(), xinv.size())) ||
        (rc = upload(c, c->verts, verts, nv)) || (rc = upload(c, c->vattr, vattr.data(), vattr.size())) ||
        (rc = upload(c, c->idx, indices, ni)) || (rc = upload(c, c->prims, prims, np)) ||
        (rc = upload(c, c->xf, xf, (size_t)nx * 16)) || (rc = upload(c, c->nrm, nrm.data(), nrm.size())) ||
        (rc = upload(c, c->prim_tri0, prim_tri0.data(), np)) ||
        (rc = upload(c, c->tri_prim, tri_prim.data(), tri_prim.size())))
        return rc;
    c->h_prims.assign(prims, prims + np);
    c->nverts = nv;
    c->nidx = ni;
    c->nprims = np;
    c->nxf = nx;
    c->ntri = (uint32_t)nt;
    c->max_material_id = max_mat;
    c->geometry_ok = true;
    return HY_OK;
}

int hy_scene_set_materials(HyCtx* c, const HyMaterial* m, uint32_t n) {
    if (!c || !m || n == 0) return HY_ERR_INVALID_ARG;
    DeviceGuard g(c->device);
    int rc = upload(c, c->mats, m, n);
    if (rc) return rc;
    c->h_mats.assign(m, m + n);
    c->nmats = n;
    return HY_OK;
}

int hy_scene_set_textures(HyCtx* c, const uint8_t* const* rgba8, const uint32_t* widths, const uint32_t* heights,
                          uint32_t n) {
    if (!c || (n && (!rgba8 || !widths || !heights))) return HY_ERR_INVALID_ARG;
    uint64_t total = 0;
    std::vector<uint32_t> tab((size_t)std::max<uint32_t>(n, 1) * 4, 0u);
    for (uint32_t i = 0; i < n; i++) {
        if (!rgba8[i] || widths[i] == 0 || heights[i] == 0) return HY_ERR_INVALID_ARG;
        tab[(size_t)i * 4 + 0] = (uint32_t)total;
        tab[(size_t)i * 4 + 1] = widths[i];
        tab[(size_t)i * 4 + 2] = heights[i];
        total += (uint64_t)widths[i] * heights[i];
        if (total >= (1ull << 32)) return HY_ERR_INVALID_ARG;
    }
    DeviceGuard g(c->device);
    int rc;
    if ((rc = ctx_alloc(c, c->tex_px, (size_t)std::max<uint64_t>(total, 1) * 4))) return rc;
    for (uint32_t i = 0; i < n; i++)
        HY_CUDA_TRY(cudaMemcpyAsync((uint8_t*)c->tex_px.p + (size_t)tab[(size_t)i * 4] * 4, rgba8[i],
                                    (size_t)widths[i] * heights[i] * 4, cudaMemcpyHostToDevice, c->stream));
    if ((rc = upload(c, c->tex_tab, tab.data(), tab.size()))) return rc;  // synchronises the stream
    c->ntex = n;
    return HY_OK;
}

int hy_scene_set_lights(HyCtx* c, const HyLight* l, uint32_t n) {
    if (!c || (n && !l)) return HY_ERR_INVALID_ARG;
    DeviceGuard g(c->device);
    for (uint32_t i = 0; i < n; i++)
        if (!finite_all(l[i].pos, 4) || !finite_all(l[i].color, 4)) return HY_ERR_NAN_INPUT;
    int rc = upload(c, c->lights, l, n);
    if (rc) return rc;
    c->nlights = n;
    return HY_OK;
}

int hy_scene_set_env(HyCtx* c, int slot, const uint8_t* px, uint32_t w, uint32_t h) {
    if (!c || slot < 0 || slot > 1 || !px || w == 0 || h == 0) return HY_ERR_INVALID_ARG;
    DeviceGuard g(c->device);
    int rc = upload(c, c->env[slot], px, (size_t)w * h * 4);
    if (rc) return rc;
    c->env_w[slot] = w;
    c->env_h[slot] = h;
    return HY_OK;
}

int hy_bvh_build(HyCtx* c, HyBvhStats* st) {
    if (!c) return HY_ERR_INVALID_ARG;
    if (!c->geometry_ok) return HY_ERR_NOT_READY;
    DeviceGuard g(c->device);
    c->bvh_ok = false;
    return bvh_build_impl(c, st);
}

int hy_bvh_build_instanced(HyCtx* c, HyBvhStats* st) {
    if (!c) return HY_ERR_INVALID_ARG;
    if (!c->geometry_ok) return HY_ERR_NOT_READY;
    DeviceGuard g(c->device);
    c->bvh_ok = false;
    return bvh_build_instanced_impl(c, st);
}

int hy_bvh_layout(HyCtx* c, HyBvhLayout* out) {
    if (!c || !out) return HY_ERR_INVALID_ARG;
    if (!c->bvh_ok) return HY_ERR_NOT_READY;
    HyBvhLayout L{};
    L.two_level = c->two_level ? 1u : 0u;
    L.num_nodes = c->n_bvh8;
    L.num_records = c->n_records;
    L.num_instances = c->two_level ? c->ninst : 0;
    L.num_blas = c->two_level ? c->nblas : 0;
    L.tlas_region = c->two_level ? c->tlas_region : 0;
    L.tlas_nodes = c->two_level ? c->tlas_nodes : 0;
    L.depth = c->depth;
    *out = L;
    return HY_OK;
}

int hy_scene_set_build_mode(HyCtx* c, uint32_t mode) {
    if (!c || mode > HY_BUILD_LBVH) return HY_ERR_INVALID_ARG;
    c->build_mode = mode;
    return HY_OK;
}

int hy_scene_set_anyhit_order(HyCtx* c, uint32_t order) {
    if (!c || order > HY_ANYHIT_NEAR_FIRST) return HY_ERR_INVALID_ARG;
    c->anyhit_order = order;  // read by scene_dev at each call (a batch replay copies the scene table anew)
    return HY_OK;
}

int hy_scene_anyhit_order(HyCtx* c, uint32_t* resolved) {
    if (!c || !resolved) return HY_ERR_INVALID_ARG;
    if (!c->bvh_ok) return HY_ERR_NOT_READY;
    *resolved = anyhit_flip(c) ? HY_ANYHIT_FAR_FIRST : HY_ANYHIT_NEAR_FIRST;
    return HY_OK;
}

int hy_bvh_download_instances(HyCtx* c, float* records, float* boxes) {
    if (!c) return HY_ERR_INVALID_ARG;
    if (!c->bvh_ok || !c->two_level) return HY_ERR_NOT_READY;
    DeviceGuard g(c->device);
    HY_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (records) HY_CUDA_TRY(cudaMemcpy(records, c->inst.p, (size_t)c->ninst * 64, cudaMemcpyDeviceToHost));
    if (boxes) HY_CUDA_TRY(cudaMemcpy(boxes, c->inst_box.p, (size_t)c->ninst * 24, cudaMemcpyDeviceToHost));
    return HY_OK;
}

int hy_bvh_refit(HyCtx* c, const float* xf, uint32_t nx) {
    if (!c || !xf || nx != c->nxf) return HY_ERR_INVALID_ARG;
    if (!c->bvh_ok) return HY_ERR_NOT_READY;
    if (!finite_all(xf, (size_t)nx * 16)) return HY_ERR_NAN_INPUT;
    DeviceGuard g(c->device);
    std::vector<float> nrm = normal_matrices(xf, nx);
    std::vector<float> xinv = world_to_object(xf, nx);
    int rc;
    if ((rc = upload(c, c->xf, xf, (size_t)nx * 16)) || (rc = upload(c, c->nrm, nrm.data(), nrm.size())) ||
        (rc = upload(c, c->xinv, xinv.data(), xinv.size())))
        return rc;
    // two-level: the BLASes stay, the instance records and the TLAS follow the transforms
    if (c->two_level) return tlas_build_impl(c);
    return bvh_refit_impl(c);
}

int hy_bvh_download(HyCtx* c, uint32_t* morton, uint32_t* order, uint32_t* bvh2, uint32_t* bvh8, float* tris) {
    if (!c) return HY_ERR_INVALID_ARG;
    if (!c->bvh_ok) return HY_ERR_NOT_READY;
    DeviceGuard g(c->device);
    const size_t n = c->ntri;
    if (c->two_level && (morton || order || bvh2)) return HY_ERR_INVALID_ARG;  // nodes and records only
    HY_CUDA_TRY(cudaStreamSynchronize(c->stream));
    if (c->two_level) {
        if (bvh8) HY_CUDA_TRY(cudaMemcpy(bvh8, c->nodes.p, (size_t)c->n_bvh8 * 80, cudaMemcpyDeviceToHost));
        if (tris) HY_CUDA_TRY(cudaMemcpy(tris, c->tris.p, (size_t)c->n_records * 48, cudaMemcpyDeviceToHost));
        return HY_OK;
    }
    if (morton) HY_CUDA_TRY(cudaMemcpy(morton, c->keys[0].p, n * 4, cudaMemcpyDeviceToHost));
    if (order) HY_CUDA_TRY(cudaMemcpy(order, c->vals[0].p, n * 4, cudaMemcpyDeviceToHost));
    if (bvh2 && n > 1) HY_CUDA_TRY(cudaMemcpy(bvh2, c->bvh2.p, (n - 1) * 40, cudaMemcpyDeviceToHost));
    if (bvh8) HY_CUDA_TRY(cudaMemcpy(bvh8, c->nodes.p, (size_t)c->n_bvh8 * 80, cudaMemcpyDeviceToHost));
    if (tris) HY_CUDA_TRY(cudaMemcpy(tris, c->tris.p, n * 48, cudaMemcpyDeviceToHost));
    return HY_OK;
}

int hy_trace_rays(HyCtx* c, const HyRay* rays, uint32_t n, int any_hit, HyHit* hits, HyStats* st) {
    if (!c || (n && (!rays || !hits))) return HY_ERR_INVALID_ARG;
    if (!c->bvh_ok) return HY_ERR_NOT_READY;
    DeviceGuard g(c->device);
    int rc = reset_counters(c);
    if (rc) return rc;
    bool count = st != nullptr;
    int grid = std::max(1, std::min<int>(c->num_sms * 16, (int)((n + 127) / 128)));
    HY_CUDA_TRY(launch_trace(scene_dev(c), rays, n, any_hit != 0, count, hits, dev_stats(c), dev_status(c), grid,
                             c->stream));
    return finish_call(c, st, true);
}

int hy_gbuffer_primary(HyCtx* c, const HyCamera* cam, uint32_t W, uint32_t H, float* planes[6]) {
    if (!c || !cam || !planes || W == 0 || H == 0) return HY_ERR_INVALID_ARG;
    for (int i = 0; i < 6; i++)
        if (!planes[i]) return HY_ERR_INVALID_ARG;
    int rc = check_scene_ready(c);
    if (rc) return rc;
    DeviceGuard g(c->device);
    if ((rc = reset_counters(c))) return rc;
    GbufParams G;
    G.W = W;
    G.H = H;
    std::memcpy(G.inv_view, cam->inv_view, 64);
    std::memcpy(G.inv_proj, cam->inv_proj, 64);
    for (int i = 0; i < 6; i++) G.planes[i] = planes[i];
    G.status = dev_status(c);
    HY_CUDA_TRY(launch_gbuffer(scene_dev(c), G, c->stream));
    return finish_call(c, nullptr, true);
}

int hy_shadow_pass(HyCtx* c, const HyGBuffer* gb, const HyCamera* cam, const HyPassConfig* cfg,
                   uint32_t accum_format, void* d_shadow, HyStats* st) {
    if (!c || !cam || !d_shadow || accum_format > HY_ACCUM_F32) return HY_ERR_INVALID_ARG;
    int rc;
    if ((rc = check_gbuffer(gb, false)) || (rc = check_cfg(cfg)) || (rc = check_scene_ready(c))) return rc;
    DeviceGuard g(c->device);
    if ((rc = reset_counters(c))) return rc;
    PassParams P = make_params(c, gb, cam, cfg, accum_format, d_shadow, nullptr, nullptr, nullptr);
    if ((rc = run_pixels(c, MODE_SHADOW, P, cfg, WQ_SHADOW))) return rc;
    return finish_call(c, st, !(cfg->flags & HY_FLAG_NO_STATUS_SYNC));
}

static int accumulate_impl(HyCtx* c, const HyGBuffer* gb, const HyPassConfig* cfg, const void* shadow,
                           HyAccum* acc) {
    AccumParams A;
    A.W = gb->width;
    A.H = gb->height;
    A.num_lights = acc->num_lights;
    A.fmt = acc->format;
    A.frame = cfg->accum_frame;
    if (cfg->flags & HY_FLAG_FULL_BLUR_DISPATCH) { A.blur_w = A.W; A.blur_h = A.H; }
    else { A.blur_w = (A.W / 16) * 16; A.blur_h = (A.H / 16) * 16; }
    A.motion = gb->plane[3];
    A.motion_fmt = gb->format[3];
    A.shadow = shadow;
    A.hist = acc->history;
    A.hist_prev = acc->history;
    if (A.frame <= 0) {
        // the reprojected read sees the history as it was before this pass
        size_t bytes = (size_t)A.W * A.H * acc->num_lights * (acc->format == HY_ACCUM_U8 ? 1 : 4);
        int rc = ensure_size(c, c->hist_prev, bytes);
        if (rc) return rc;
        HY_CUDA_TRY(cudaMemcpyAsync(c->hist_prev.p, acc->history, bytes, cudaMemcpyDeviceToDevice, c->stream));
        A.hist_prev = c->hist_prev.p;
    }
    ProfScope prof(c, PK_ACCUM);
    HY_CUDA_TRY(launch_accumulate(A, c->stream));
    return HY_OK;
}

int hy_accumulate_pass(HyCtx* c, const HyGBuffer* gb, const HyPassConfig* cfg, const void* d_shadow, HyAccum* acc) {
    if (!c || !d_shadow || !acc || !acc->history || acc->format > HY_ACCUM_F32) return HY_ERR_INVALID_ARG;
    int rc;
    if ((rc = check_gbuffer(gb, false)) || (rc = check_cfg(cfg))) return rc;
    DeviceGuard g(c->device);
    if ((rc = accumulate_impl(c, gb, cfg, d_shadow, acc))) return rc;
    HY_CUDA_TRY(cudaGetLastError());
    if (!(cfg->flags & HY_FLAG_NO_STATUS_SYNC)) HY_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return HY_OK;
}

int hy_shade_pass(HyCtx* c, const HyGBuffer* gb, const HyCamera* cam, const HyPassConfig* cfg, const HyAccum* acc,
                  float* out_f, uint8_t* out_8, HyStats* st) {
    if (!c || !cam || !acc || !acc->history || acc->format > HY_ACCUM_F32) return HY_ERR_INVALID_ARG;
    int rc;
    if ((rc = check_gbuffer(gb, true)) || (rc = check_cfg(cfg)) || (rc = check_scene_ready(c))) return rc;
    if (acc->num_lights > c->nlights) return HY_ERR_INVALID_ARG;  // the pass uses the first num_lights lights
    DeviceGuard g(c->device);
    if ((rc = reset_counters(c))) return rc;
    // with HY_FLAG_NO_ACCUM the history argument holds the raw shadow images
    PassParams P = make_params(c, gb, cam, cfg, acc->format, acc->history, acc->history, out_f, out_8);
    P.num_lights = acc->num_lights;
    if ((rc = run_pixels(c, MODE_SHADE, P, cfg, WQ_SHADE))) return rc;
    return finish_call(c, st, !(cfg->flags & HY_FLAG_NO_STATUS_SYNC));
}

// the shadow kernel reads G-buffer planes 0 and 1 only; what runs after it
// waits here for planes 2-5 when hy_hybrid_forward_host copies them on its side stream
static int wait_planes(HyCtx* c) {
    if (!c->copy_pending) return HY_OK;
    c->copy_pending = false;
    HY_CUDA_TRY(cudaStreamWaitEvent(c->stream, c->copy_done, 0));
    return HY_OK;
}

static int forward_impl(HyCtx* c, const HyGBuffer* gb, const HyCamera* cam, const HyPassConfig* cfg, HyAccum* acc,
                        float* out_f, uint8_t* out_8) {
    int rc;
    if (!(cfg->flags & HY_FLAG_NO_ACCUM) && cfg->accum_frame > 0) {
        // steady state: the running mean is pointwise, so the shadow kernel folds
        // each light's factor straight into the history (no raw images)
        PassParams P = make_params(c, gb, cam, cfg, acc->format, nullptr, acc->history, out_f, out_8);
        P.num_lights = acc->num_lights;
        if ((rc = run_pixels(c, MODE_SHADOW_ACCUM, P, cfg, WQ_SHADOW))) return rc;
        if ((rc = wait_planes(c))) return rc;
        return run_pixels(c, MODE_SHADE, P, cfg, WQ_SHADE);
    }
    size_t bytes = (size_t)gb->width * gb->height * acc->num_lights * (acc->format == HY_ACCUM_U8 ? 1 : 4);
    if ((rc = ensure_size(c, c->raw_shadow, bytes ? bytes : 16))) return rc;
    PassParams P = make_params(c, gb, cam, cfg, acc->format, c->raw_shadow.p, acc->history, out_f, out_8);
    P.num_lights = acc->num_lights;
    if ((rc = run_pixels(c, MODE_SHADOW, P, cfg, WQ_SHADOW))) return rc;
    if ((rc = wait_planes(c))) return rc;
    if (!(cfg->flags & HY_FLAG_NO_ACCUM) && (rc = accumulate_impl(c, gb, cfg, c->raw_shadow.p, acc))) return rc;
    return run_pixels(c, MODE_SHADE, P, cfg, WQ_SHADE);
}

int hy_hybrid_forward(HyCtx* c, const HyGBuffer* gb, const HyCamera* cam, const HyPassConfig* cfg, HyAccum* acc,
                      float* out_f, uint8_t* out_8, HyStats* st) {
    if (!c || !cam || !acc || !acc->history || acc->format > HY_ACCUM_F32) return HY_ERR_INVALID_ARG;
    int rc;
    if ((rc = check_gbuffer(gb, true)) || (rc = check_cfg(cfg)) || (rc = check_scene_ready(c))) return rc;
    if (acc->num_lights > c->nlights) return HY_ERR_INVALID_ARG;  // the pass uses the first num_lights lights
    DeviceGuard g(c->device);
    if ((rc = reset_counters(c))) return rc;
    if ((rc = forward_impl(c, gb, cam, cfg, acc, out_f, out_8))) return rc;
    return finish_call(c, st, !(cfg->flags & HY_FLAG_NO_STATUS_SYNC));
}

int hy_hybrid_backward(HyCtx* c, const HyGBuffer* gb, const HyCamera* cam, const HyPassConfig* cfg,
                       const HyAccum* acc, const float* d_grad, float* d_grad_mats, float* d_grad_lights,
                       HyStats* st) {
    if (!c || !cam || !acc || !acc->history || acc->format > HY_ACCUM_F32 || !d_grad) return HY_ERR_INVALID_ARG;
    if (((uintptr_t)d_grad) % 16 != 0) return HY_ERR_INVALID_ARG;
    int rc;
    if ((rc = check_gbuffer(gb, true)) || (rc = check_cfg(cfg)) || (rc = check_scene_ready(c))) return rc;
    if (acc->num_lights > c->nlights) return HY_ERR_INVALID_ARG;
    if (cfg->max_bounces > HY_GRAD_MAX_BOUNCES || acc->num_lights > HY_GRAD_MAX_LIGHTS) return HY_ERR_UNSUPPORTED;
    DeviceGuard g(c->device);
    if ((rc = reset_counters(c))) return rc;
    GradParams G;
    G.P = make_params(c, gb, cam, cfg, acc->format, acc->history, acc->history, nullptr, nullptr);
    G.P.num_lights = acc->num_lights;
    G.P.queue = dev_queue(c, WQ_SHADE);
    G.grad = reinterpret_cast<const float4*>(d_grad);
    G.light_off = c->nmats * HY_GRAD_MATERIAL_PARAMS;
    G.nparam = G.light_off + c->nlights * HY_GRAD_LIGHT_PARAMS;
    int grid = 1;
    bool smem = false;
    size_t smem_bytes = 0;
    HY_CUDA_TRY(grad_launch_shape(G.nparam, c->num_sms, G.P.ntiles, &grid, &smem, &smem_bytes));
    const size_t rows = smem ? (size_t)grid : 1;
    if ((rc = ensure_size(c, c->grad_partial, rows * G.nparam * 4))) return rc;
    G.out = c->grad_partial.as<float>();
    {
        ProfScope prof(c, PK_GRAD);
        HY_CUDA_TRY(launch_shade_grad(scene_dev(c), G, grid, smem, smem_bytes, d_grad_mats, d_grad_lights,
                                      c->stream));
    }
    return finish_call(c, st, !(cfg->flags & HY_FLAG_NO_STATUS_SYNC));
}

int hy_pathtrace_pass(HyCtx* c, const HyCamera* cam, uint32_t W, uint32_t H, const HyPassConfig* cfg,
                      uint8_t* d_image, float* d_out_f, HyStats* st) {
    if (!c || !cam || W == 0 || H == 0 || (uint64_t)W * H >= (1ull << 31)) return HY_ERR_INVALID_ARG;
    if (((uintptr_t)d_image) % 4 || ((uintptr_t)d_out_f) % 16) return HY_ERR_INVALID_ARG;
    int rc;
    if ((rc = check_cfg(cfg)) || (rc = check_scene_ready(c))) return rc;
    DeviceGuard g(c->device);
    if ((rc = reset_counters(c))) return rc;
    PtParams T;
    std::memset(&T, 0, sizeof(T));
    PassParams& P = T.P;
    P.W = W;
    P.H = H;
    P.spp = cfg->shadow_spp;
    P.max_bounces = cfg->max_bounces;
    P.rng_mode = cfg->rng_mode;
    P.flags = cfg->flags;
    P.out_f = d_out_f;
    P.out_8 = d_image;
    P.tiles_x = (W + 7) / 8;
    P.ntiles = P.tiles_x * ((H + 3) / 4);
    P.chunk = cfg->queue_chunk ? cfg->queue_chunk : 1;
    P.stats = dev_stats(c);
    P.status = dev_status(c);
    P.queue = dev_queue(c, WQ_MISC);
    P.num_lights = c->nlights;  // closesthit.rchit loops over every light of the scene
    std::memcpy(T.inv_view, cam->inv_view, 64);
    std::memcpy(T.inv_proj, cam->inv_proj, 64);
    T.frame = (int32_t)cam->frame[0];
    const bool count = (cfg->flags & HY_FLAG_COUNT_TRAVERSAL) != 0;
    // shadow rays of each hit as tile streams (default), or on the hit's own lane
    const bool stream = !(cfg->flags & HY_FLAG_PIXEL_PARALLEL);
    P.inner = cfg->visits_per_round ? std::min(cfg->visits_per_round, 16u) : kStreamSteps;
    // resident blocks the tile-stream kernel is compiled for: 6 (80 registers)
    // measured fastest at 1080p (uncapped 195 registers: 1,015; 3: 1,351; 4: 1,536;
    // 5: 1,697; 6: 1,769; 8: 1,774 Mrays/s) — occupancy beats the spills
    const int minb = cfg->min_blocks ? (int)cfg->min_blocks : 6;
    int per = 0;
    if (pathtrace_occupancy(count, stream, c->two_level, minb, &per) != cudaSuccess || per <= 0) per = 1;
    int grid = std::max(1, std::min<int>(per * c->num_sms, (int)((P.ntiles * 32ull + 127) / 128)));
    {
        ProfScope prof(c, PK_PATHTRACE);
        HY_CUDA_TRY(launch_pathtrace(count, stream, minb, scene_dev(c), T, grid, c->stream));
    }
    return finish_call(c, st, !(cfg->flags & HY_FLAG_NO_STATUS_SYNC));
}

int hy_post_resolve(HyCtx* c, uint32_t W, uint32_t H, const uint8_t* in8, const float* inf, uint8_t* out) {
    if (!c || !out || (!in8 && !inf) || (uint64_t)W * H >= (1ull << 31)) return HY_ERR_INVALID_ARG;
    if (((uintptr_t)out) % 4 || ((uintptr_t)in8) % 4 || ((uintptr_t)inf) % 16) return HY_ERR_INVALID_ARG;
    DeviceGuard g(c->device);
    HY_CUDA_TRY(launch_post(in8, inf, W * H, out, c->stream));
    HY_CUDA_TRY(cudaStreamSynchronize(c->stream));
    return HY_OK;
}

int hy_profile_enable(HyCtx* c, int enable) {
    if (!c) return HY_ERR_INVALID_ARG;
    DeviceGuard g(c->device);
    HY_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->prof_on = enable != 0;
    c->prof_recs.clear();
    c->prof_used = 0;
    return HY_OK;
}

int hy_profile_read(HyCtx* c, HyKernelTime* out, uint32_t cap, uint32_t* count) {
    if (!c || !count || (cap && !out)) return HY_ERR_INVALID_ARG;
    DeviceGuard g(c->device);
    HY_CUDA_TRY(cudaStreamSynchronize(c->stream));
    uint32_t launches[PK_COUNT] = {};
    double ms[PK_COUNT] = {};
    for (const HyCtx::ProfRec& r : c->prof_recs) {
        float t = 0.f;
        HY_CUDA_TRY(cudaEventElapsedTime(&t, r.a, r.b));
        launches[r.kind]++;
        ms[r.kind] += t;
    }
    c->prof_recs.clear();
    c->prof_used = 0;
    uint32_t n = 0;
    for (int k = 0; k < PK_COUNT; k++) {
        if (!launches[k]) continue;
        if (n < cap) {
            std::memset(&out[n], 0, sizeof(HyKernelTime));
            std::strncpy(out[n].kernel, kProfNames[k], sizeof(out[n].kernel) - 1);
            out[n].launches = launches[k];
            out[n].total_ms = (float)ms[k];
        }
        n++;
    }
    *count = n;
    return HY_OK;
}

int hy_hybrid_forward_host(HyCtx* c, const HyGBuffer* hgb, const HyCamera* cam, const HyPassConfig* cfg,
                           HyAccum* acc, float* h_out_f, uint8_t* h_out_8, HyStats* st) {
    if (!c || !cam || !acc || !acc->history || acc->format > HY_ACCUM_F32) return HY_ERR_INVALID_ARG;
    int rc;
    if ((rc = check_gbuffer(hgb, true)) || (rc = check_cfg(cfg)) || (rc = check_scene_ready(c))) return rc;
    if (acc->num_lights > c->nlights) return HY_ERR_INVALID_ARG;  // the pass uses the first num_lights lights
    DeviceGuard g(c->device);
    const size_t npx = (size_t)hgb->width * hgb->height;
    HyGBuffer dgb = *hgb;
    for (int p = 0; p < 6; p++) {
        if ((rc = ensure_size(c, c->host_in[p], npx * fmt_bytes(hgb->format[p])))) return rc;
        dgb.plane[p] = c->host_in[p].p;
    }
    float* d_f = nullptr;
    uint8_t* d_8 = nullptr;
    if (h_out_f) { if ((rc = ensure_size(c, c->host_out_f, npx * 16))) return rc; d_f = c->host_out_f.as<float>(); }
    if (h_out_8) { if ((rc = ensure_size(c, c->host_out_8, npx * 4))) return rc; d_8 = c->host_out_8.as<uint8_t>(); }
    if (!c->copy_stream) HY_CUDA_TRY(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    if (!c->copy_start) HY_CUDA_TRY(cudaEventCreateWithFlags(&c->copy_start, cudaEventDisableTiming));
    if (!c->copy_done) HY_CUDA_TRY(cudaEventCreateWithFlags(&c->copy_done, cudaEventDisableTiming));
    // planes 0 and 1 on the context's stream (the shadow kernel reads them);
    // planes 2-5 on a side stream that starts once earlier work on the staging
    // buffers is done and overlaps the shadow kernel
    c->copy_pending = false;
    rc = [&]() -> int {
        HY_CUDA_TRY(cudaEventRecord(c->copy_start, c->stream));
        HY_CUDA_TRY(cudaStreamWaitEvent(c->copy_stream, c->copy_start, 0));
        c->copy_pending = true;
        for (int p = 0; p < 6; p++)
            HY_CUDA_TRY(cudaMemcpyAsync(c->host_in[p].p, hgb->plane[p], npx * fmt_bytes(hgb->format[p]),
                                        cudaMemcpyHostToDevice, p < 2 ? c->stream : c->copy_stream));
        HY_CUDA_TRY(cudaEventRecord(c->copy_done, c->copy_stream));
        int r;
        if ((r = reset_counters(c))) return r;
        return forward_impl(c, &dgb, cam, cfg, acc, d_f, d_8);
    }();
    if (rc) {
        // an error after the uploads were queued: the caller's buffers may still be
        // read by the side stream, so wait for it before returning
        if (c->copy_pending) {
            c->copy_pending = false;
            cudaStreamSynchronize(c->copy_stream);
            cudaStreamSynchronize(c->stream);
            cudaGetLastError();
        }
        return rc;
    }
    if (h_out_f) HY_CUDA_TRY(cudaMemcpyAsync(h_out_f, d_f, npx * 16, cudaMemcpyDeviceToHost, c->stream));
    if (h_out_8) HY_CUDA_TRY(cudaMemcpyAsync(h_out_8, d_8, npx * 4, cudaMemcpyDeviceToHost, c->stream));
    return finish_call(c, st, true);
}

// ---- batches -------------------------------------------------------------------
// launch shape of a batch's tile-stream shadow kernel
struct BatchShape {
    int minb;    // register cap as resident 128-thread blocks per SM
    int block;   // threads per block
    int shortd;  // shared-memory stack entries per lane
};

static int batch_enqueue(HyCtx* c, const std::vector<PassParams>& pv, const std::vector<SceneDev>& sd,
                         const HyView* views, const std::vector<uint32_t>& reset_views, const BatchParams& B,
                         bool count, const BatchShape& sh, bool stream, bool two, size_t tab_bytes) {
    cudaStream_t s = c->stream;
    HY_CUDA_TRY(cudaMemcpyAsync(c->batch_tab.p, c->h_batch_tab, tab_bytes, cudaMemcpyHostToDevice, s));
    HY_CUDA_TRY(cudaMemsetAsync(c->dstats.p, 0, c->dstats.bytes, s));
    int per = 0;
    if (batch_occupancy(false, count, sh.minb, stream, two, sh.block, sh.shortd, &per) != cudaSuccess || per <= 0)
        per = 1;
    int grid = std::max(1, std::min<int>(per * c->num_sms, (int)((B.total_tiles * 32ull + sh.block - 1) / sh.block)));
    BatchParams Bs = B;
    Bs.queue = dev_queue(c, WQ_SHADOW);
    HY_CUDA_TRY(launch_batch(false, count, sh.minb, stream, two, sh.block, sh.shortd, Bs, grid, s));
    for (uint32_t v : reset_views) {
        const HyView& vw = views[v];
        HyAccum acc = vw.accum;
        int rc = accumulate_impl(c, &vw.gbuffer, &vw.config, pv[v].shadow, &acc);
        if (rc) return rc;
    }
    if (batch_occupancy(true, count, sh.minb, false, false, 128, 0, &per) != cudaSuccess || per <= 0) per = 1;
    grid = std::max(1, std::min<int>(per * c->num_sms, (int)((B.total_tiles * 32ull + 127) / 128)));
    BatchParams Bh = B;
    Bh.queue = dev_queue(c, WQ_SHADE);
    HY_CUDA_TRY(launch_batch(true, count, sh.minb, false, false, 128, 0, Bh, grid, s));
    (void)sd;
    return HY_OK;
}

int hy_batch_forward(HyCtx* c, HyCtx* const* scenes, uint32_t ns, const HyView* views, uint32_t nv,
                     uint32_t bflags, const HyPassConfig* tuning, HyStats* st) {
    if (!c || !scenes || ns == 0 || !views || nv == 0 || nv > kMaxBatchViews) return HY_ERR_INVALID_ARG;
    int rc;
    for (uint32_t i = 0; i < ns; i++) {
        if (!scenes[i]) return HY_ERR_INVALID_ARG;
        if (scenes[i]->device != c->device) return HY_ERR_INVALID_ARG;
        if ((rc = check_scene_ready(scenes[i]))) return rc;
        // the lane-group batch kernel walks one-level structures only
        if (scenes[i]->two_level && tuning && (tuning->flags & HY_FLAG_LANE_GROUPS)) return HY_ERR_UNSUPPORTED;
    }
    DeviceGuard g(c->device);
    const bool count = tuning && (tuning->flags & HY_FLAG_COUNT_TRAVERSAL);
    const uint32_t chunk = tuning && tuning->queue_chunk ? tuning->queue_chunk : 1;
    const bool stream = !(tuning && (tuning->flags & HY_FLAG_LANE_GROUPS));
    bool any_two = false;
    for (uint32_t i = 0; i < ns; i++) any_two = any_two || scenes[i]->two_level;
    // the tile-stream kernel's launch shape: threads per block {64, 128, 256}, register
    // cap {6, 8} resident 128-thread blocks (80 / 64 registers), shared stack entries
    // {0, 8, 16, 32}; counting launches and two-level batches run the 128 / 8 (5) / 0 shape
    // default: 256 threads, 64 registers, no shared stack, one tile per pull, the shape
    // hy_batch_autotune picked for the 64-view mixed batch on a GB300
    BatchShape sh{tuning && tuning->min_blocks ? (int)tuning->min_blocks : 8,
                  tuning && tuning->block_size ? (int)tuning->block_size : (stream && !count && !any_two ? 256 : 128),
                  tuning ? (int)tuning->stack_depth : 0};
    if (chunk > 1024) return HY_ERR_INVALID_ARG;
    if (sh.block != 64 && sh.block != 128 && sh.block != 256) return HY_ERR_INVALID_ARG;
    if (sh.shortd != 0 && sh.shortd != 8 && sh.shortd != 16 && sh.shortd != 32) return HY_ERR_INVALID_ARG;
    if (stream && !count && !any_two) {
        if (sh.minb != 6 && sh.minb != 8) return HY_ERR_INVALID_ARG;
    } else {
        if ((sh.block != 128 || sh.shortd != 0) && stream) return HY_ERR_UNSUPPORTED;
        if (!stream && (sh.block != 128 || sh.shortd != 0)) return HY_ERR_UNSUPPORTED;
        if (stream) sh.minb = 8;
    }
    const int minb = sh.minb;
    // per-view parameters
    std::vector<PassParams> pv(nv);
    std::vector<uint32_t> reset_views;
    size_t raw_bytes = 0, snap_bytes = 0;
    std::vector<size_t> raw_off(nv, (size_t)-1);
    uint32_t total = 0;
    for (uint32_t i = 0; i < nv; i++) {
        const HyView& v = views[i];
        if (v.scene >= ns) return HY_ERR_INVALID_ARG;
        if ((rc = check_gbuffer(&v.gbuffer, true)) || (rc = check_cfg(&v.config))) return rc;
        const HyCtx* sc = scenes[v.scene];
        if (!v.accum.history || v.accum.format > HY_ACCUM_F32 || v.accum.num_lights > sc->nlights)
            return HY_ERR_INVALID_ARG;
        const size_t hbytes = (size_t)v.gbuffer.width * v.gbuffer.height * v.accum.num_lights *
                              (v.accum.format == HY_ACCUM_U8 ? 1 : 4);
        const bool accum = !(v.config.flags & HY_FLAG_NO_ACCUM) && v.config.accum_frame > 0;
        if (!accum) {
            raw_off[i] = raw_bytes;
            raw_bytes += (hbytes + 255) & ~(size_t)255;
            if (!(v.config.flags & HY_FLAG_NO_ACCUM)) {
                reset_views.push_back(i);
                snap_bytes = std::max(snap_bytes, hbytes);
            }
        }
        pv[i] = make_params(c, &v.gbuffer, &v.camera, &v.config, v.accum.format, nullptr, v.accum.history,
                            v.out_rgba32f, v.out_bgra8);
        pv[i].scene = v.scene;
        pv[i].num_lights = v.accum.num_lights;
        if (stream && !v.config.visits_per_round) pv[i].inner = kStreamSteps;
        uint32_t G = 1;
        if (v.config.rng_mode == HY_RNG_DECORRELATED)
            while (G < v.config.shadow_spp && G < 32) G <<= 1;
        pv[i].group = G;
    }
    // the queue hands out the costliest views' tiles first (shadow rays per tile:
    // lights x samples), so the launch ends on cheap tiles instead of waiting
    // for the last warps of an expensive one
    std::vector<uint32_t> order(nv);
    for (uint32_t i = 0; i < nv; i++) order[i] = i;
    auto tile_cost = [&](uint32_t i) {
        const uint64_t spp = views[i].config.rng_mode == HY_RNG_DECORRELATED ? views[i].config.shadow_spp : 1;
        return (uint64_t)pv[i].num_lights * spp + 1;
    };
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return tile_cost(a) > tile_cost(b); });
    for (uint32_t i : order) {
        pv[i].tile_begin = total;
        total += pv[i].ntiles;
    }
    if ((rc = ensure_size(c, c->raw_shadow, raw_bytes ? raw_bytes : 16))) return rc;
    if (snap_bytes && (rc = ensure_size(c, c->hist_prev, snap_bytes))) return rc;
    for (uint32_t i = 0; i < nv; i++) {
        if (raw_off[i] == (size_t)-1) continue;
        pv[i].shadow = (uint8_t*)c->raw_shadow.p + raw_off[i];
    }
    std::vector<SceneDev> sd(ns);
    for (uint32_t i = 0; i < ns; i++) sd[i] = scene_dev(scenes[i]);
    // the tables: device copy + pinned host mirror
    const size_t tab_bytes = nv * sizeof(PassParams) + ns * sizeof(SceneDev);
    if ((rc = ensure_size(c, c->batch_tab, tab_bytes))) return rc;
    if (c->batch_done) HY_CUDA_TRY(cudaEventSynchronize(c->batch_done));  // the last replay has read the mirror
    if (c->h_batch_tab_bytes < tab_bytes) {
        if (c->h_batch_tab) cudaFreeHost(c->h_batch_tab);
        c->h_batch_tab = nullptr;
        c->h_batch_tab_bytes = 0;
        HY_CUDA_TRY(cudaMallocHost(&c->h_batch_tab, tab_bytes));
        c->h_batch_tab_bytes = tab_bytes;
        if (c->batch_exec) { cudaGraphExecDestroy(c->batch_exec); c->batch_exec = nullptr; c->batch_key.clear(); }
    }
    // the device table lists the views in queue order (increasing tile_begin, which
    // the kernels' view lookup searches)
    for (uint32_t k = 0; k < nv; k++)
        std::memcpy((uint8_t*)c->h_batch_tab + k * sizeof(PassParams), &pv[order[k]], sizeof(PassParams));
    std::memcpy((uint8_t*)c->h_batch_tab + nv * sizeof(PassParams), sd.data(), ns * sizeof(SceneDev));
    BatchParams B;
    B.views = c->batch_tab.as<PassParams>();
    B.scenes = (const SceneDev*)((uint8_t*)c->batch_tab.p + nv * sizeof(PassParams));
    B.nviews = nv;
    B.total_tiles = total;
    B.chunk = chunk;
    B.stats = dev_stats(c);
    B.status = dev_status(c);
    B.queue = nullptr;
    if (bflags & HY_BATCH_NO_GRAPH) {
        if ((rc = batch_enqueue(c, pv, sd, views, reset_views, B, count, sh, stream, any_two, tab_bytes))) return rc;
    } else {
        // the graph bakes pointers of the tables, scratch and reset-view launches
        std::vector<uint64_t> key = {nv, ns, total, chunk, (uint64_t)minb, (uint64_t)count, (uint64_t)stream,
                                     (uint64_t)any_two, (uint64_t)sh.block, (uint64_t)sh.shortd,
                                     (uint64_t)(uintptr_t)c->batch_tab.p,
                                     (uint64_t)(uintptr_t)c->h_batch_tab, (uint64_t)(uintptr_t)c->raw_shadow.p,
                                     (uint64_t)(uintptr_t)c->hist_prev.p, (uint64_t)(uintptr_t)c->stream};
        for (uint32_t v : reset_views) {
            const HyView& vw = views[v];
            key.push_back(v);
            key.push_back((uint64_t)(uintptr_t)vw.accum.history);
            key.push_back((uint64_t)(uintptr_t)vw.gbuffer.plane[3]);
            key.push_back(((uint64_t)vw.gbuffer.width << 32) | vw.gbuffer.height);
            key.push_back(((uint64_t)(uint32_t)vw.config.accum_frame << 32) | vw.config.flags);
            key.push_back(((uint64_t)vw.accum.format << 32) | vw.gbuffer.format[3]);
        }
        if (!c->batch_exec || key != c->batch_key) {
            if (c->batch_exec) { cudaGraphExecDestroy(c->batch_exec); c->batch_exec = nullptr; }
            c->batch_key.clear();
            cudaGraph_t graph = nullptr;
            HY_CUDA_TRY(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
            rc = batch_enqueue(c, pv, sd, views, reset_views, B, count, sh, stream, any_two, tab_bytes);
            cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
            if (rc) { if (graph) cudaGraphDestroy(graph); return rc; }
            if (e != cudaSuccess) { cudaGetLastError(); return HY_ERR_CUDA; }
            e = cudaGraphInstantiate(&c->batch_exec, graph, 0);
            cudaGraphDestroy(graph);
            if (e != cudaSuccess) { cudaGetLastError(); c->batch_exec = nullptr; return HY_ERR_CUDA; }
            c->batch_key = key;
        }
        HY_CUDA_TRY(cudaGraphLaunch(c->batch_exec, c->stream));
    }
    if (!c->batch_done) HY_CUDA_TRY(cudaEventCreateWithFlags(&c->batch_done, cudaEventDisableTiming));
    HY_CUDA_TRY(cudaEventRecord(c->batch_done, c->stream));
    return finish_call(c, st, !(bflags & HY_BATCH_NO_STATUS_SYNC));
}

// Coordinate descent over the tile-stream batch kernel's launch shape: each axis in
// turn (queue chunk, threads per block, register cap, shared stack entries) is
// swept with the others at their best so far; a shape is timed by CUDA events on
// the context's stream around `reps` graph replays after one untimed call (which
// captures the shape's graph), and its time is the fastest replay.
int hy_batch_autotune(HyCtx* c, HyCtx* const* scenes, uint32_t ns, const HyView* views, uint32_t nv,
                      uint32_t reps, HyPassConfig* tuning, float* best_ms) {
    if (!c || !tuning || reps == 0 || reps > 64) return HY_ERR_INVALID_ARG;
    DeviceGuard g(c->device);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
        cudaGetLastError();
        if (e0) cudaEventDestroy(e0);
        return HY_ERR_CUDA;
    }
    HyPassConfig best;
    std::memset(&best, 0, sizeof(best));
    best.shadow_spp = 1;
    best.queue_chunk = 1;
    best.block_size = 128;
    best.min_blocks = 8;
    best.stack_depth = 0;
    float best_t = 0.f;
    auto time_shape = [&](const HyPassConfig& cand, float* ms) -> int {
        int rc = hy_batch_forward(c, scenes, ns, views, nv, HY_BATCH_NO_STATUS_SYNC, &cand, nullptr);
        if (rc) return rc;
        float t_min = 0.f;
        for (uint32_t k = 0; k < reps; k++) {
            HY_CUDA_TRY(cudaEventRecord(e0, c->stream));
            if ((rc = hy_batch_forward(c, scenes, ns, views, nv, HY_BATCH_NO_STATUS_SYNC, &cand, nullptr))) return rc;
            HY_CUDA_TRY(cudaEventRecord(e1, c->stream));
            HY_CUDA_TRY(cudaEventSynchronize(e1));
            float t = 0.f;
            HY_CUDA_TRY(cudaEventElapsedTime(&t, e0, e1));
            if (k == 0 || t < t_min) t_min = t;
        }
        // a device-side error of the shape (timeout, overflow) disqualifies nothing silently
        if ((rc = finish_call(c, nullptr, true))) return rc;
        *ms = t_min;
        return HY_OK;
    };
    int rc = time_shape(best, &best_t);
    static const uint32_t chunks[] = {1, 2, 4, 8, 16, 32}, blocks[] = {64, 128, 256}, minbs[] = {6, 8},
                          stacks[] = {0, 8, 16, 32};
    struct Axis { const uint32_t* v; int n; uint32_t HyPassConfig::*field; };
    const Axis axes[] = {{chunks, 6, &HyPassConfig::queue_chunk}, {blocks, 3, &HyPassConfig::block_size},
                         {minbs, 2, &HyPassConfig::min_blocks}, {stacks, 4, &HyPassConfig::stack_depth}};
    for (const Axis& a : axes) {
        if (rc) break;
        HyPassConfig cur = best;
        for (int i = 0; i < a.n && !rc; i++) {
            if (a.v[i] == best.*(a.field)) continue;
            HyPassConfig cand = cur;
            cand.*(a.field) = a.v[i];
            float t = 0.f;
            rc = time_shape(cand, &t);
            if (rc == HY_ERR_UNSUPPORTED) { rc = HY_OK; continue; }  // a shape the batch cannot take
            if (!rc && t < best_t) { best = cand; best_t = t; }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    *tuning = best;
    if (best_ms) *best_ms = best_t;
    return HY_OK;
}

}  // extern "C"
