// Top-down binned-SAH binary tree on the GPU (HY_BUILD_SAH): the tree that the
// BVH8 collapse of hy_bvh.cu turns into 8-wide nodes, in place of the LBVH's
// radix tree.  It stands in for the driver's trace-quality builds
// (src/renderer.cpp:1696-1865; BLASes and the TLAS are built with
// PREFER_FAST_TRACE, src/renderer.h:246 and src/renderer.cpp:1687).
//
// Each range [f, l] of c >= 2 triangles of the Morton-sorted order:
//   * centroid bounds as order-preserving integer keys (exact min/max, -0 below
//     +0); an axis takes part when hi - lo > 0, its scale 32 / (hi - lo);
//   * per axis and bin (floor((c - lo) * scale) clamped to 0..31): the count
//     and the box of the triangles (keys);
//   * for each axis and q = 0..30, left = bins 0..q, right = bins q+1..31, both
//     non-empty: cost = area(left) n(left) + area(right) n(right); the first
//     strictly lowest finite cost in (axis, q) order wins; the triangles with
//     bin <= q move to the front of the range, order kept on both sides (a
//     stable partition), the split m = f + n(left).  No candidate (coincident
//     centroids): m = f + c / 2, order unchanged.
//   * the range's node is node m - 1 (split positions are distinct, so the
//     n - 1 internal nodes use every index once); a one-triangle side is the
//     leaf at its position.
// Every float op is an IEEE-rounded intrinsic, so the order, the tree and the
// 8-wide nodes collapsed from it equal the CPU oracle's bit for bit.
//
// Schedule: ranges above small_max triangles are split level by level, each
// level by four launches over chunks of kChunk triangles (bin: shared-memory
// bins flushed with global atomics; eval: a block per range picks the split
// and the chunks' output offsets; scatter: the stable partition into scratch
// with a block scan; copy back).  Ranges of up to small_max triangles are
// whole subtrees for one warp each (k_sah_small), which walks them with a
// short explicit stack (the larger side pushed, the smaller taken first, so at
// most log2(small_max) entries).  small_max (64..4096) is picked per build so
// that about 16 warps per SM get a subtree; it changes the schedule only, not
// the tree.
#include <cuda_runtime.h>

#include <algorithm>
#include <climits>
#include <vector>

#include "hy_internal.h"

namespace hy {

namespace {

constexpr uint32_t kLeafRef = 0x80000000u;
constexpr uint32_t kNone = 0xffffffffu;
constexpr int kBins = 32;
constexpr int kBinWords = 7;                       // count, lo xyz keys, hi xyz keys
constexpr int kAxisWords = kBins * kBinWords;      // 224
constexpr int kNodeBinWords = 3 * kAxisWords;      // 672
constexpr uint32_t kSmallMaxCap = 4096;            // a warp builds ranges up to small_max <= this
constexpr uint32_t kChunk = 2048;                  // triangles per block in the level passes
constexpr int kStackMax = 16;                      // > log2(kSmallMaxCap) + 1
constexpr unsigned kFull = 0xffffffffu;

struct SahRange {
    uint32_t f, l;          // first and last position in the order
    uint32_t parent, side;  // parent node (kNone: the root) and side (0 left, 1 right)
    int ck[6];              // centroid bounds as keys: lo xyz, hi xyz
};
static_assert(sizeof(SahRange) == 40, "SahRange layout");

struct SahChunk { uint32_t node, start, end, first; };  // range slot, [start, end), the range's first chunk
struct SahSplit { int axis, q; uint32_t m, child[2]; };  // child: 0 none, 1 << 30 | next-level slot, 2 << 30 | small slot

enum { CTR_NEXT = 0, CTR_SMALL = 1, CTR_ROOT = 2, CTR_ERR = 3 };

__device__ __forceinline__ int okey(float x) {
    const int b = __float_as_int(x);
    return b >= 0 ? b : b ^ 0x7fffffff;
}
__device__ __forceinline__ float unkey(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7fffffff); }

__device__ __forceinline__ int sah_bin(float c, float lo, float scale) {
    const float v = __fmul_rn(__fsub_rn(c, lo), scale);
    return v >= 0.f ? (v < (float)kBins ? (int)v : kBins - 1) : 0;
}

__device__ __forceinline__ float area_keys(const int lo[3], const int hi[3]) {
    const float dx = __fsub_rn(unkey(hi[0]), unkey(lo[0]));
    const float dy = __fsub_rn(unkey(hi[1]), unkey(lo[1]));
    const float dz = __fsub_rn(unkey(hi[2]), unkey(lo[2]));
    float a = __fmul_rn(dx, dy);
    a = __fadd_rn(a, __fmul_rn(dy, dz));
    a = __fadd_rn(a, __fmul_rn(dz, dx));
    return a;
}

struct Axes {
    float lo[3], scale[3];
    bool ok[3];
};
__device__ __forceinline__ Axes axes_of(const int ck[6]) {
    Axes x;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        x.lo[a] = unkey(ck[a]);
        const float ext = __fsub_rn(unkey(ck[3 + a]), x.lo[a]);
        x.ok[a] = ext > 0.f;
        x.scale[a] = x.ok[a] ? __fdiv_rn((float)kBins, ext) : 0.f;
    }
    return x;
}

__device__ __forceinline__ void bins_clear(int* b, uint32_t tid, uint32_t nthreads) {
    for (uint32_t i = tid; i < (uint32_t)kNodeBinWords; i += nthreads) {
        const uint32_t k = i % kBinWords;
        b[i] = k == 0 ? 0 : (k < 4 ? INT_MAX : INT_MIN);
    }
}

// one triangle into the bins of every axis that takes part
__device__ __forceinline__ void bin_one(int* b, const Axes& x, float4 ce, const float* bx) {
    int kl[3], kh[3];
#pragma unroll
    for (int k = 0; k < 3; k++) { kl[k] = okey(bx[k]); kh[k] = okey(bx[3 + k]); }
    const float cc[3] = {ce.x, ce.y, ce.z};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        if (!x.ok[a]) continue;
        int* e = b + a * kAxisWords + sah_bin(cc[a], x.lo[a], x.scale[a]) * kBinWords;
        atomicAdd(e, 1);
#pragma unroll
        for (int k = 0; k < 3; k++) { atomicMin(e + 1 + k, kl[k]); atomicMax(e + 4 + k, kh[k]); }
    }
}

// Lane q holds bin q of one axis (ab: that axis's 32 x 7 words).  Returns the
// candidate of the split after bin q as (cost bits << 32 | axis * 32 + q), all
// ones when there is none (an empty side, lane 31, or a cost that is not finite).
__device__ __forceinline__ unsigned long long sweep_axis(const int* ab, int a, uint32_t lane) {
    const int* e = ab + lane * kBinWords;
    uint32_t pc = (uint32_t)e[0], sc = pc;
    int plo[3], phi[3], slo[3], shi[3];
#pragma unroll
    for (int k = 0; k < 3; k++) { plo[k] = slo[k] = e[1 + k]; phi[k] = shi[k] = e[4 + k]; }
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t oc = __shfl_up_sync(kFull, pc, d);
        const uint32_t os = __shfl_down_sync(kFull, sc, d);
        int ol[3], oh[3], ul[3], uh[3];
#pragma unroll
        for (int k = 0; k < 3; k++) {
            ol[k] = __shfl_up_sync(kFull, plo[k], d);
            oh[k] = __shfl_up_sync(kFull, phi[k], d);
            ul[k] = __shfl_down_sync(kFull, slo[k], d);
            uh[k] = __shfl_down_sync(kFull, shi[k], d);
        }
        if (lane >= (uint32_t)d) {
            pc += oc;
#pragma unroll
            for (int k = 0; k < 3; k++) { plo[k] = min(plo[k], ol[k]); phi[k] = max(phi[k], oh[k]); }
        }
        if (lane + d < 32) {
            sc += os;
#pragma unroll
            for (int k = 0; k < 3; k++) { slo[k] = min(slo[k], ul[k]); shi[k] = max(shi[k], uh[k]); }
        }
    }
    const uint32_t rc = __shfl_down_sync(kFull, sc, 1);
    int rlo[3], rhi[3];
#pragma unroll
    for (int k = 0; k < 3; k++) { rlo[k] = __shfl_down_sync(kFull, slo[k], 1); rhi[k] = __shfl_down_sync(kFull, shi[k], 1); }
    unsigned long long key = ~0ull;
    if (lane < 31 && pc > 0 && rc > 0) {
        const float t1 = __fmul_rn(area_keys(plo, phi), __uint2float_rn(pc));
        const float t2 = __fmul_rn(area_keys(rlo, rhi), __uint2float_rn(rc));
        const float cost = __fadd_rn(__fadd_rn(t1, t2), 0.f);
        if (cost < INFINITY) key = ((unsigned long long)__float_as_uint(cost) << 32) | (uint32_t)(a * kBins + lane);
    }
    return key;
}

__device__ __forceinline__ unsigned long long warp_min_u64(unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long w = __shfl_xor_sync(kFull, v, o);
        v = w < v ? w : v;
    }
    return v;
}

__device__ __forceinline__ void keys_init(int k[6]) {
    k[0] = k[1] = k[2] = INT_MAX;
    k[3] = k[4] = k[5] = INT_MIN;
}
__device__ __forceinline__ void keys_add(int k[6], float4 c) {
    const int x = okey(c.x), y = okey(c.y), z = okey(c.z);
    k[0] = min(k[0], x); k[1] = min(k[1], y); k[2] = min(k[2], z);
    k[3] = max(k[3], x); k[4] = max(k[4], y); k[5] = max(k[5], z);
}
__device__ __forceinline__ void keys_warp(int k[6]) {
#pragma unroll
    for (int j = 0; j < 3; j++) {
        k[j] = __reduce_min_sync(kFull, k[j]);
        k[3 + j] = __reduce_max_sync(kFull, k[3 + j]);
    }
}

// the node of a range split at m: its range, its link from the parent (or the
// root slot) and its one-triangle sides
__device__ __forceinline__ void write_node(uint32_t id, uint32_t f, uint32_t l, uint32_t m, uint32_t par,
                                           uint32_t side, uint32_t n, uint32_t* bvh2, uint32_t* parent,
                                           uint32_t* ctr) {
    uint32_t* nd = bvh2 + (size_t)id * 10;
    nd[2] = f;
    nd[3] = l;
    if (par == kNone) {
        ctr[CTR_ROOT] = id;
        parent[id] = kNone;
    } else {
        bvh2[(size_t)par * 10 + side] = id;
        parent[id] = par;
    }
    if (m - f == 1) { nd[0] = kLeafRef | f; parent[n - 1 + f] = id; }
    if (l - m + 1 == 1) { nd[1] = kLeafRef | m; parent[n - 1 + m] = id; }
}

// ---- root ----------------------------------------------------------------------
__global__ void k_sah_root_init(SahRange* r, uint32_t n) {
    if (threadIdx.x == 0) {
        r->f = 0;
        r->l = n - 1;
        r->parent = kNone;
        r->side = 0;
        keys_init(r->ck);
    }
}

__global__ void k_sah_root_bounds(const float4* __restrict__ cen, uint32_t n, SahRange* r) {
    int k[6];
    keys_init(k);
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) keys_add(k, cen[t]);
    keys_warp(k);
    if ((threadIdx.x & 31) == 0)
        for (int j = 0; j < 3; j++) { atomicMin(&r->ck[j], k[j]); atomicMax(&r->ck[3 + j], k[3 + j]); }
}

// ---- level passes over ranges above small_max ------------------------------------
__global__ void k_sah_bins_init(int* __restrict__ gbins, uint32_t nwords) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nwords; i += gridDim.x * blockDim.x) {
        const uint32_t k = i % kBinWords;
        gbins[i] = k == 0 ? 0 : (k < 4 ? INT_MAX : INT_MIN);
    }
}

__global__ void __launch_bounds__(256) k_sah_bin(const SahChunk* __restrict__ chunks,
                                                 const SahRange* __restrict__ ranges,
                                                 const uint32_t* __restrict__ ord, const float4* __restrict__ cen,
                                                 const float* __restrict__ box, int* __restrict__ gbins,
                                                 uint32_t* __restrict__ ccnt) {
    __shared__ int sb[kNodeBinWords];
    const SahChunk ch = chunks[blockIdx.x];
    const Axes x = axes_of(ranges[ch.node].ck);
    bins_clear(sb, threadIdx.x, blockDim.x);
    __syncthreads();
    for (uint32_t i = ch.start + threadIdx.x; i < ch.end; i += blockDim.x) {
        const uint32_t t = ord[i];
        bin_one(sb, x, cen[t], box + (size_t)t * 6);
    }
    __syncthreads();
    int* gb = gbins + (size_t)ch.node * kNodeBinWords;
    for (uint32_t j = threadIdx.x; j < (uint32_t)kNodeBinWords; j += blockDim.x) {
        const int v = sb[j];
        const uint32_t k = j % kBinWords;
        if (k == 0) {
            ccnt[(size_t)blockIdx.x * (3 * kBins) + j / kBinWords] = (uint32_t)v;
            if (v) atomicAdd(gb + j, v);
        } else if (k < 4) {
            if (v != INT_MAX) atomicMin(gb + j, v);
        } else if (v != INT_MIN) {
            atomicMax(gb + j, v);
        }
    }
}

// A block of 256 threads per range: warps 0-2 sweep one axis each; then the
// chunks' left counts and their exclusive prefix (the chunk's offset among the
// range's left triangles), the node, and the children queued.
__global__ void __launch_bounds__(256) k_sah_eval(const SahRange* __restrict__ ranges, const int* __restrict__ gbins,
                                                  const uint32_t* __restrict__ first_chunk,
                                                  const uint32_t* __restrict__ ccnt, uint32_t* __restrict__ coff,
                                                  SahSplit* __restrict__ split, SahRange* __restrict__ next,
                                                  SahRange* __restrict__ small, uint32_t n, uint32_t small_max,
                                                  uint32_t* __restrict__ bvh2, uint32_t* __restrict__ parent,
                                                  uint32_t* __restrict__ ctr) {
    __shared__ unsigned long long s_key[3];
    __shared__ uint32_t s_part[256];
    const SahRange R = ranges[blockIdx.x];
    const int* gb = gbins + (size_t)blockIdx.x * kNodeBinWords;
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const Axes x = axes_of(R.ck);
    if (w < 3) {
        unsigned long long key = ~0ull;
        if (x.ok[w]) key = warp_min_u64(sweep_axis(gb + w * kAxisWords, (int)w, lane));
        if (lane == 0) s_key[w] = key;
    }
    __syncthreads();
    const uint32_t c = R.l - R.f + 1;
    const uint32_t nch = (c + kChunk - 1) / kChunk, ch0 = first_chunk[blockIdx.x];
    unsigned long long best = s_key[0];
    best = s_key[1] < best ? s_key[1] : best;
    best = s_key[2] < best ? s_key[2] : best;
    const int ba = best == ~0ull ? -1 : (int)((uint32_t)best / kBins);
    const int bq = best == ~0ull ? 0 : (int)((uint32_t)best % kBins);
    // left count of each chunk (bins <= q of the axis), thread-serial over a
    // contiguous run of chunks, then a block scan of the runs
    const uint32_t per = (nch + 255) / 256, k0 = min(threadIdx.x * per, nch), k1 = min(k0 + per, nch);
    uint32_t run = 0;
    if (ba >= 0)
        for (uint32_t k = k0; k < k1; k++) {
            const uint32_t* cc = ccnt + (size_t)(ch0 + k) * (3 * kBins) + ba * kBins;
            uint32_t s = 0;
            for (int b = 0; b <= bq; b++) s += cc[b];
            coff[ch0 + k] = s;
            run += s;
        }
    s_part[threadIdx.x] = run;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t acc = 0;
        for (int i = 0; i < 256; i++) { const uint32_t v = s_part[i]; s_part[i] = acc; acc += v; }
        SahSplit sp;
        sp.axis = ba;
        sp.q = bq;
        sp.m = ba >= 0 ? R.f + acc : R.f + c / 2;
        const uint32_t id = sp.m - 1;
        write_node(id, R.f, R.l, sp.m, R.parent, R.side, n, bvh2, parent, ctr);
        const uint32_t cf[2] = {R.f, sp.m}, cl[2] = {sp.m - 1, R.l};
        for (int s = 0; s < 2; s++) {
            const uint32_t cs = cl[s] - cf[s] + 1;
            sp.child[s] = 0;
            if (cs < 2) continue;
            SahRange ch;
            ch.f = cf[s];
            ch.l = cl[s];
            ch.parent = id;
            ch.side = (uint32_t)s;
            keys_init(ch.ck);
            if (cs > small_max) {
                const uint32_t slot = atomicAdd(ctr + CTR_NEXT, 1u);
                next[slot] = ch;
                sp.child[s] = (1u << 30) | slot;
            } else {
                const uint32_t slot = atomicAdd(ctr + CTR_SMALL, 1u);
                small[slot] = ch;
                sp.child[s] = (2u << 30) | slot;
            }
        }
        split[blockIdx.x] = sp;
    }
    __syncthreads();
    if (ba >= 0) {
        uint32_t acc = s_part[threadIdx.x];
        for (uint32_t k = k0; k < k1; k++) {
            const uint32_t v = coff[ch0 + k];
            coff[ch0 + k] = acc;
            acc += v;
        }
    }
}

// Stable partition of one chunk into ord2: each thread takes 8 consecutive
// triangles; left ranks come from a block scan plus the chunk's offset, right
// ranks from the position.  The children's centroid bounds accumulate with
// global atomics on their queue entries.
__global__ void __launch_bounds__(256) k_sah_scatter(const SahChunk* __restrict__ chunks,
                                                     const SahRange* __restrict__ ranges,
                                                     const SahSplit* __restrict__ split,
                                                     const uint32_t* __restrict__ coff,
                                                     const uint32_t* __restrict__ ord, uint32_t* __restrict__ ord2,
                                                     const float4* __restrict__ cen, SahRange* __restrict__ next,
                                                     SahRange* __restrict__ small) {
    __shared__ uint32_t s_warp[8];
    __shared__ int s_keys[8][12];
    const SahChunk ch = chunks[blockIdx.x];
    const SahRange R = ranges[ch.node];
    const SahSplit sp = split[ch.node];
    const Axes x = axes_of(R.ck);
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t i0 = ch.start + threadIdx.x * 8;
    uint32_t t[8];
    float4 ce[8];
    uint32_t flags = 0, nl = 0;
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const uint32_t i = i0 + j;
        t[j] = 0;
        ce[j] = make_float4(0.f, 0.f, 0.f, 0.f);
        if (i < ch.end) {
            t[j] = ord[i];
            ce[j] = cen[t[j]];
            bool left;
            if (sp.axis >= 0) {
                const float cc = sp.axis == 0 ? ce[j].x : (sp.axis == 1 ? ce[j].y : ce[j].z);
                left = sah_bin(cc, x.lo[sp.axis], x.scale[sp.axis]) <= sp.q;
            } else {
                left = i < sp.m;
            }
            if (left) { flags |= 1u << j; nl++; }
        }
    }
    // block exclusive scan of nl
    uint32_t incl = nl;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t o = __shfl_up_sync(kFull, incl, d);
        if (lane >= (uint32_t)d) incl += o;
    }
    if (lane == 31) s_warp[w] = incl;
    __syncthreads();
    uint32_t wbase = 0;
    for (uint32_t k = 0; k < w; k++) wbase += s_warp[k];
    uint32_t lrank = wbase + incl - nl;  // left triangles of this chunk before this thread's
    const uint32_t off_l = sp.axis >= 0 ? coff[blockIdx.x] : 0;
    int kl[6], kr[6];
    keys_init(kl);
    keys_init(kr);
#pragma unroll
    for (int j = 0; j < 8; j++) {
        const uint32_t i = i0 + j;
        if (i >= ch.end) break;
        const bool left = (flags >> j) & 1u;
        uint32_t dst;
        if (sp.axis < 0) {
            dst = i;
        } else if (left) {
            dst = R.f + off_l + lrank;
        } else {
            const uint32_t li = i - ch.start;  // position in the chunk
            dst = sp.m + (ch.start - R.f - off_l) + (li - lrank);
        }
        if (left) lrank++;
        ord2[dst] = t[j];
        if (left) keys_add(kl, ce[j]);
        else keys_add(kr, ce[j]);
    }
    keys_warp(kl);
    keys_warp(kr);
    if (lane == 0)
        for (int k = 0; k < 6; k++) { s_keys[w][k] = kl[k]; s_keys[w][6 + k] = kr[k]; }
    __syncthreads();
    if (threadIdx.x < 12) {
        const uint32_t k = threadIdx.x, s = k / 6, kk = k % 6;
        const uint32_t ref = sp.child[s];
        if (ref) {
            int v = s_keys[0][k];
            for (int ww = 1; ww < 8; ww++) v = kk < 3 ? min(v, s_keys[ww][k]) : max(v, s_keys[ww][k]);
            SahRange* dstr = ((ref >> 30) == 1u ? next : small) + (ref & 0x3fffffffu);
            if (kk < 3) atomicMin(&dstr->ck[kk], v);
            else atomicMax(&dstr->ck[kk], v);
        }
    }
}

__global__ void k_sah_copy(const SahChunk* __restrict__ chunks, const uint32_t* __restrict__ ord2,
                           uint32_t* __restrict__ ord) {
    const SahChunk ch = chunks[blockIdx.x];
    for (uint32_t i = ch.start + threadIdx.x; i < ch.end; i += blockDim.x) ord[i] = ord2[i];
}

// ---- one warp per range of up to small_max triangles --------------------------
constexpr int kSmallWarps = 4;

__global__ void __launch_bounds__(32 * kSmallWarps) k_sah_small(const SahRange* __restrict__ tasks, uint32_t ntask,
                                                                uint32_t n, const float4* __restrict__ cen,
                                                                const float* __restrict__ box, uint32_t* ord,
                                                                uint32_t* ord2, uint32_t* __restrict__ bvh2,
                                                                uint32_t* __restrict__ parent,
                                                                uint32_t* __restrict__ ctr) {
    __shared__ int s_bins[kSmallWarps][kNodeBinWords];
    __shared__ SahRange s_stack[kSmallWarps][kStackMax];
    const uint32_t lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const uint32_t task = blockIdx.x * kSmallWarps + w;
    if (task >= ntask) return;
    int* bins = s_bins[w];
    SahRange cur = tasks[task];
    int sp = 0;
    for (;;) {
        const uint32_t f = cur.f, l = cur.l, c = l - f + 1;
        const Axes x = axes_of(cur.ck);
        unsigned long long best = ~0ull;
        if (x.ok[0] || x.ok[1] || x.ok[2]) {
            bins_clear(bins, lane, 32);
            __syncwarp();
            for (uint32_t i = f + lane; i <= l; i += 32) {
                const uint32_t t = ord[i];
                bin_one(bins, x, cen[t], box + (size_t)t * 6);
            }
            __syncwarp();
#pragma unroll
            for (int a = 0; a < 3; a++) {
                if (!x.ok[a]) continue;
                const unsigned long long k = sweep_axis(bins + a * kAxisWords, a, lane);
                best = k < best ? k : best;
            }
            best = warp_min_u64(best);
        }
        int kl[6], kr[6];
        keys_init(kl);
        keys_init(kr);
        uint32_t m;
        if (best != ~0ull) {
            const int ba = (int)((uint32_t)best / kBins), bq = (int)((uint32_t)best % kBins);
            const uint32_t cnt = lane <= (uint32_t)bq ? (uint32_t)bins[ba * kAxisWords + lane * kBinWords] : 0u;
            m = f + __reduce_add_sync(kFull, cnt);
            uint32_t nl = 0, nr = 0;
            const uint32_t lt = (1u << lane) - 1u;
            for (uint32_t i0 = f; i0 <= l; i0 += 32) {
                const uint32_t i = i0 + lane;
                const bool valid = i <= l;
                uint32_t t = 0;
                float4 ce = make_float4(0.f, 0.f, 0.f, 0.f);
                bool left = false;
                if (valid) {
                    t = ord[i];
                    ce = cen[t];
                    const float cc = ba == 0 ? ce.x : (ba == 1 ? ce.y : ce.z);
                    left = sah_bin(cc, x.lo[ba], x.scale[ba]) <= bq;
                }
                const uint32_t L = __ballot_sync(kFull, left), V = __ballot_sync(kFull, valid);
                if (valid) {
                    ord2[left ? f + nl + __popc(L & lt) : m + nr + __popc(~L & V & lt)] = t;
                    if (left) keys_add(kl, ce);
                    else keys_add(kr, ce);
                }
                nl += __popc(L);
                nr += __popc(~L & V);
            }
            __syncwarp();
            for (uint32_t i = f + lane; i <= l; i += 32) ord[i] = ord2[i];
            __syncwarp();
        } else {
            m = f + c / 2;
            for (uint32_t i = f + lane; i <= l; i += 32) {
                const float4 ce = cen[ord[i]];
                if (i < m) keys_add(kl, ce);
                else keys_add(kr, ce);
            }
        }
        keys_warp(kl);
        keys_warp(kr);
        const uint32_t id = m - 1;
        if (lane == 0) write_node(id, f, l, m, cur.parent, cur.side, n, bvh2, parent, ctr);
        const bool li = m - f >= 2, ri = l - m + 1 >= 2;
        SahRange L, R;
        L.f = f; L.l = m - 1; L.parent = id; L.side = 0;
        R.f = m; R.l = l; R.parent = id; R.side = 1;
#pragma unroll
        for (int k = 0; k < 6; k++) { L.ck[k] = kl[k]; R.ck[k] = kr[k]; }
        if (li && ri) {
            const bool lsmall = (m - f) <= (l - m + 1);
            if (sp >= kStackMax) {  // cannot happen (the stack holds at most log2(kSmallMaxCap) ranges)
                if (lane == 0) atomicExch(ctr + CTR_ERR, 1u);
                return;
            }
            if (lane == 0) s_stack[w][sp] = lsmall ? R : L;
            sp++;
            cur = lsmall ? L : R;
        } else if (li) {
            cur = L;
        } else if (ri) {
            cur = R;
        } else {
            if (sp == 0) break;
            __syncwarp();
            cur = s_stack[w][--sp];
        }
        __syncwarp();
    }
}

inline uint32_t cdiv_u(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

}  // namespace

// Binary tree over the n >= 2 ids in ord (Morton sorted; permuted in place),
// ord2 n words of scratch.  Writes words 0-3 of every internal node of bvh2,
// parent (internal nodes at [0, n-1), leaf positions at n-1+i) and the root
// id to *d_root (device).
int sah_tree_impl(HyCtx* c, uint32_t n, uint32_t* ord, uint32_t* ord2, uint32_t* bvh2, uint32_t* parent,
                  uint32_t* d_root) {
    if (n < 2) return HY_ERR_INVALID_ARG;
    cudaStream_t s = c->stream;
    // subtrees for about 16 warps per SM, each of 64..4096 triangles
    uint32_t small_max = 64;
    while (small_max < kSmallMaxCap && (uint64_t)small_max * 16u * (uint32_t)c->num_sms < n) small_max <<= 1;
    const uint32_t bigcap = n / (small_max + 1) + 2;
    const uint32_t smallcap = n / 2 + 2;
    const uint32_t chunkcap = n / kChunk + bigcap + 2;
    int rc;
    if ((rc = ctx_alloc(c, c->sah_ranges[0], (size_t)bigcap * sizeof(SahRange))) ||
        (rc = ctx_alloc(c, c->sah_ranges[1], (size_t)bigcap * sizeof(SahRange))) ||
        (rc = ctx_alloc(c, c->sah_small, (size_t)smallcap * sizeof(SahRange))) ||
        (rc = ctx_alloc(c, c->sah_bins, (size_t)bigcap * kNodeBinWords * 4)) ||
        (rc = ctx_alloc(c, c->sah_split, (size_t)bigcap * sizeof(SahSplit))) ||
        (rc = ctx_alloc(c, c->sah_chunks, (size_t)chunkcap * sizeof(SahChunk))) ||
        (rc = ctx_alloc(c, c->sah_first, (size_t)bigcap * 4)) ||
        (rc = ctx_alloc(c, c->sah_ccnt, (size_t)chunkcap * 3 * kBins * 4)) ||
        (rc = ctx_alloc(c, c->sah_coff, (size_t)chunkcap * 4)) || (rc = ctx_alloc(c, c->sah_ctr, 16)))
        return rc;
    uint32_t* ctr = c->sah_ctr.as<uint32_t>();
    HY_CUDA_TRY(cudaMemsetAsync(ctr, 0, 16, s));
    const bool root_small = n <= small_max;
    SahRange* root = root_small ? c->sah_small.as<SahRange>() : c->sah_ranges[0].as<SahRange>();
    k_sah_root_init<<<1, 32, 0, s>>>(root, n);
    k_sah_root_bounds<<<std::min<uint32_t>(cdiv_u(n, 256), 4 * (uint32_t)c->num_sms), 256, 0, s>>>(
        c->centroid.as<float4>(), n, root);
    HY_CUDA_TRY(cudaGetLastError());
    uint32_t nbig = root_small ? 0 : 1, nsmall = root_small ? 1 : 0;
    if (root_small) {
        const uint32_t one = 1;
        HY_CUDA_TRY(cudaMemcpyAsync(ctr + CTR_SMALL, &one, 4, cudaMemcpyHostToDevice, s));
    }
    std::vector<SahRange> h_ranges;
    std::vector<SahChunk> h_chunks;
    std::vector<uint32_t> h_first;
    int cur = 0;
    for (uint32_t level = 0; nbig > 0; level++) {
        if (level > n) return HY_ERR_TIMEOUT;  // every level splits off at least one triangle
        SahRange* ranges = c->sah_ranges[cur].as<SahRange>();
        SahRange* next = c->sah_ranges[cur ^ 1].as<SahRange>();
        h_ranges.resize(nbig);
        HY_CUDA_TRY(cudaMemcpyAsync(h_ranges.data(), ranges, (size_t)nbig * sizeof(SahRange), cudaMemcpyDeviceToHost,
                                    s));
        HY_CUDA_TRY(cudaStreamSynchronize(s));
        h_chunks.clear();
        h_first.resize(nbig);
        for (uint32_t j = 0; j < nbig; j++) {
            h_first[j] = (uint32_t)h_chunks.size();
            for (uint64_t st = h_ranges[j].f; st <= h_ranges[j].l; st += kChunk)
                h_chunks.push_back({j, (uint32_t)st, (uint32_t)std::min<uint64_t>(st + kChunk, (uint64_t)h_ranges[j].l + 1),
                                    h_first[j]});
        }
        const uint32_t nch = (uint32_t)h_chunks.size();
        if (nch > chunkcap) return HY_ERR_CUDA;
        HY_CUDA_TRY(cudaMemcpyAsync(c->sah_chunks.p, h_chunks.data(), (size_t)nch * sizeof(SahChunk),
                                    cudaMemcpyHostToDevice, s));
        HY_CUDA_TRY(cudaMemcpyAsync(c->sah_first.p, h_first.data(), (size_t)nbig * 4, cudaMemcpyHostToDevice, s));
        HY_CUDA_TRY(cudaMemsetAsync(ctr + CTR_NEXT, 0, 4, s));
        const SahChunk* chunks = c->sah_chunks.as<SahChunk>();
        k_sah_bins_init<<<std::min<uint32_t>(cdiv_u(nbig * kNodeBinWords, 256), 1024), 256, 0, s>>>(
            c->sah_bins.as<int>(), nbig * kNodeBinWords);
        k_sah_bin<<<nch, 256, 0, s>>>(chunks, ranges, ord, c->centroid.as<float4>(), c->tribox.as<float>(),
                                      c->sah_bins.as<int>(), c->sah_ccnt.as<uint32_t>());
        k_sah_eval<<<nbig, 256, 0, s>>>(ranges, c->sah_bins.as<int>(), c->sah_first.as<uint32_t>(),
                                        c->sah_ccnt.as<uint32_t>(), c->sah_coff.as<uint32_t>(),
                                        c->sah_split.as<SahSplit>(), next, c->sah_small.as<SahRange>(), n,
                                        small_max, bvh2, parent, ctr);
        k_sah_scatter<<<nch, 256, 0, s>>>(chunks, ranges, c->sah_split.as<SahSplit>(), c->sah_coff.as<uint32_t>(),
                                          ord, ord2, c->centroid.as<float4>(), next, c->sah_small.as<SahRange>());
        k_sah_copy<<<nch, 256, 0, s>>>(chunks, ord2, ord);
        HY_CUDA_TRY(cudaGetLastError());
        uint32_t h_ctr[2];
        HY_CUDA_TRY(cudaMemcpyAsync(h_ctr, ctr, 8, cudaMemcpyDeviceToHost, s));
        HY_CUDA_TRY(cudaStreamSynchronize(s));
        nbig = h_ctr[CTR_NEXT];
        nsmall = h_ctr[CTR_SMALL];
        if (nbig > bigcap || nsmall > smallcap) return HY_ERR_CUDA;
        cur ^= 1;
    }
    if (nsmall > 0) {
        k_sah_small<<<cdiv_u(nsmall, kSmallWarps), 32 * kSmallWarps, 0, s>>>(
            c->sah_small.as<SahRange>(), nsmall, n, c->centroid.as<float4>(), c->tribox.as<float>(), ord, ord2, bvh2,
            parent, ctr);
        HY_CUDA_TRY(cudaGetLastError());
    }
    uint32_t h_err = 0;
    HY_CUDA_TRY(cudaMemcpyAsync(&h_err, ctr + CTR_ERR, 4, cudaMemcpyDeviceToHost, s));
    HY_CUDA_TRY(cudaMemcpyAsync(d_root, ctr + CTR_ROOT, 4, cudaMemcpyDeviceToDevice, s));
    HY_CUDA_TRY(cudaStreamSynchronize(s));
    return h_err ? HY_ERR_STACK_OVERFLOW : HY_OK;
}

}  // namespace hy
