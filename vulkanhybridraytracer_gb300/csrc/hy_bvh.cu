// GPU build of the acceleration structure that replaces the driver's
// BLAS/TLAS builds (src/renderer.cpp:1696-1865, rebuilt each frame from
// src/vk_engine.cpp:172-187).
//
//   k_world_tris    M * v in world space (fixed unfused op order), triangle
//                   boxes and centroids
//   k_bounds        centroid bounds (min/max through order-preserving ints)
//   k_morton        30-bit Morton codes over the centroid bounds
//   k_radix_*       stable LSD radix sort (8-bit digits, warp-match ranking)
//   k_karras        Karras 2012 binary radix tree over (morton << 32 | id)
//                   (HY_BUILD_LBVH), or the binned-SAH tree of hy_sah.cu
//                   over the same order (HY_BUILD_SAH, the default)
//   k_refit         bottom-up boxes, last-arriver-computes (no waiting)
//   k_collapse_dp   slot budgets of the collapse by the surface area heuristic
//                   (bottom up, last arriver computes)
//   k_collapse_*    BFS collapse into compressed 8-wide nodes, one level per
//                   launch pair with prefix sums for deterministic numbering
//
// Every float op of the build is an explicit IEEE-rounded intrinsic, so the
// output arrays equal those of a CPU build of the same algorithm bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "hy_device.cuh"
#include "hy_internal.h"

namespace hy {

constexpr uint32_t kLeaf = 0x80000000u;

__device__ __forceinline__ int f2ord(float f) {
    int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float ord2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

// ---------------------------------------------------------------------------------
__global__ void k_world_tris(const HyVertex* __restrict__ verts, const uint32_t* __restrict__ idx,
                             const HyPrimitive* __restrict__ prims, const uint32_t* __restrict__ tri_prim,
                             const uint32_t* __restrict__ prim_tri0, const float* __restrict__ xf, uint32_t n,
                             float4* __restrict__ world, float* __restrict__ tribox, float4* __restrict__ cen) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    uint32_t p = tri_prim[t];
    HyPrimitive pr = prims[p];
    uint32_t local = t - prim_tri0[p];
    const float* M = xf + (size_t)pr.transform_id * 16;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int v = 0; v < 3; v++) {
        uint32_t vi = idx[pr.first_index + 3 * local + v] + pr.vertex_offset;
        const float* P = verts[vi].pos;
        float w[3];
#pragma unroll
        for (int r = 0; r < 3; r++) {
            float acc = __fmul_rn(M[0 * 4 + r], P[0]);
            acc = __fadd_rn(acc, __fmul_rn(M[1 * 4 + r], P[1]));
            acc = __fadd_rn(acc, __fmul_rn(M[2 * 4 + r], P[2]));
            acc = __fadd_rn(acc, M[3 * 4 + r]);
            w[r] = acc;
            lo[r] = fminf(lo[r], acc);
            hi[r] = fmaxf(hi[r], acc);
        }
        world[(size_t)t * 3 + v] = make_float4(w[0], w[1], w[2], 0.f);
    }
    float* b = tribox + (size_t)t * 6;
    for (int a = 0; a < 3; a++) { b[a] = lo[a]; b[3 + a] = hi[a]; }
    cen[t] = make_float4(__fmul_rn(__fadd_rn(lo[0], hi[0]), 0.5f), __fmul_rn(__fadd_rn(lo[1], hi[1]), 0.5f),
                         __fmul_rn(__fadd_rn(lo[2], hi[2]), 0.5f), 0.f);
}

__global__ void k_bounds_init(int* b) {
    if (threadIdx.x < 3) { b[threadIdx.x] = f2ord(INFINITY); b[3 + threadIdx.x] = f2ord(-INFINITY); }
}

__global__ void k_bounds(const float4* __restrict__ cen, uint32_t n, int* b) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
        float4 c = cen[t];
        lo[0] = fminf(lo[0], c.x); lo[1] = fminf(lo[1], c.y); lo[2] = fminf(lo[2], c.z);
        hi[0] = fmaxf(hi[0], c.x); hi[1] = fmaxf(hi[1], c.y); hi[2] = fmaxf(hi[2], c.z);
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int a = 0; a < 3; a++) {
            lo[a] = fminf(lo[a], __shfl_xor_sync(0xffffffffu, lo[a], o));
            hi[a] = fmaxf(hi[a], __shfl_xor_sync(0xffffffffu, hi[a], o));
        }
    if ((threadIdx.x & 31) == 0)
        for (int a = 0; a < 3; a++) { atomicMin(b + a, f2ord(lo[a])); atomicMax(b + 3 + a, f2ord(hi[a])); }
}

__device__ __forceinline__ uint32_t expand10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

__device__ __forceinline__ uint32_t morton_of(float4 c, const int* __restrict__ b) {
    float lo[3], inv[3];
    for (int a = 0; a < 3; a++) {
        lo[a] = ord2f(b[a]);
        float ext = __fsub_rn(ord2f(b[3 + a]), lo[a]);
        inv[a] = ext > 0.f ? __fdiv_rn(1024.0f, ext) : 0.f;
    }
    float cc[3] = {c.x, c.y, c.z};
    uint32_t q[3];
    for (int a = 0; a < 3; a++) {
        float v = __fmul_rn(__fsub_rn(cc[a], lo[a]), inv[a]);
        v = fminf(fmaxf(v, 0.f), 1023.f);
        q[a] = (uint32_t)v;
    }
    return (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
}

__global__ void k_morton(const float4* __restrict__ cen, uint32_t n, const int* __restrict__ b,
                         uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    keys[t] = morton_of(cen[t], b);
    vals[t] = t;
}

// the codes in leaf order after the SAH build reordered the ids
__global__ void k_morton_at(const float4* __restrict__ cen, uint32_t n, const int* __restrict__ b,
                            const uint32_t* __restrict__ ord, uint32_t* __restrict__ keys) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    keys[i] = morton_of(cen[ord[i]], b);
}

// ---------------------------------------------------------------------------------
// exclusive scan (three-phase: block sums, scan of sums, block scans)
// ---------------------------------------------------------------------------------
constexpr int SCAN_T = 256, SCAN_I = 8, SCAN_TILE = SCAN_T * SCAN_I;

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* sm, uint32_t& total) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sm[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t s = lane < (SCAN_T / 32) ? sm[lane] : 0u;
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += y;
        }
        if (lane < (SCAN_T / 32)) sm[lane] = s;
    }
    __syncthreads();
    total = sm[SCAN_T / 32 - 1];
    uint32_t base = w > 0 ? sm[w - 1] : 0u;
    __syncthreads();
    return base + x - v;
}

__global__ void k_scan_sums(const uint32_t* __restrict__ in, uint32_t n, uint32_t* __restrict__ sums) {
    __shared__ uint32_t sm[32];
    uint32_t base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_I, s = 0;
    for (int i = 0; i < SCAN_I; i++) if (base + i < n) s += in[base + i];
    uint32_t tot;
    block_excl_scan(s, sm, tot);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}
// single block: exclusive scan of the block sums in place, total to *total
__global__ void k_scan_top(uint32_t* sums, uint32_t nb, uint32_t* total) {
    __shared__ uint32_t sm[32];
    uint32_t carry = 0;
    for (uint32_t off = 0; off < nb; off += SCAN_T) {
        uint32_t i = off + threadIdx.x;
        uint32_t v = i < nb ? sums[i] : 0u, tot;
        uint32_t e = block_excl_scan(v, sm, tot);
        if (i < nb) sums[i] = carry + e;
        carry += tot;
    }
    if (threadIdx.x == 0 && total) *total = carry;
}
__global__ void k_scan_apply(const uint32_t* __restrict__ in, uint32_t n, const uint32_t* __restrict__ sums,
                             uint32_t* __restrict__ out) {
    __shared__ uint32_t sm[32];
    uint32_t base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_I;
    uint32_t v[SCAN_I], s = 0;
    for (int i = 0; i < SCAN_I; i++) { v[i] = base + i < n ? in[base + i] : 0u; s += v[i]; }
    uint32_t tot;
    uint32_t run = block_excl_scan(s, sm, tot) + sums[blockIdx.x];
    for (int i = 0; i < SCAN_I; i++) {
        if (base + i < n) out[base + i] = run;
        run += v[i];
    }
}

int scan_exclusive(HyCtx* c, const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* d_total) {
    uint32_t nb = (n + SCAN_TILE - 1) / SCAN_TILE;
    if (nb == 0) nb = 1;
    int rc = ctx_alloc(c, c->scan_tmp, (size_t)nb * 4);
    if (rc) return rc;
    uint32_t* sums = c->scan_tmp.as<uint32_t>();
    k_scan_sums<<<nb, SCAN_T, 0, c->stream>>>(in, n, sums);
    k_scan_top<<<1, SCAN_T, 0, c->stream>>>(sums, nb, d_total);
    k_scan_apply<<<nb, SCAN_T, 0, c->stream>>>(in, n, sums, out);
    HY_CUDA_TRY(cudaGetLastError());
    return HY_OK;
}

// ---------------------------------------------------------------------------------
// stable LSD radix sort, 8-bit digits
// ---------------------------------------------------------------------------------
constexpr int RS_WARPS = 8, RS_ROUNDS = 8, RS_TILE = RS_WARPS * 32 * RS_ROUNDS;

__device__ __forceinline__ void rs_count(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                         uint32_t (*cnt)[257]) {
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t base = blockIdx.x * RS_TILE + w * 32 * RS_ROUNDS;
    for (int r = 0; r < RS_ROUNDS; r++) {
        uint32_t i = base + r * 32 + lane;
        uint32_t d = i < n ? (keys[i] >> shift) & 0xffu : 256u;
        uint32_t m = __match_any_sync(0xffffffffu, d);
        if (d < 256u && lane == __ffs(m) - 1) cnt[w][d] += __popc(m);
        __syncwarp();
    }
}

__global__ void __launch_bounds__(256) k_radix_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                    uint32_t nblocks, uint32_t* __restrict__ hist) {
    __shared__ uint32_t cnt[RS_WARPS][257];
    for (int i = threadIdx.x; i < RS_WARPS * 257; i += blockDim.x) (&cnt[0][0])[i] = 0;
    __syncthreads();
    rs_count(keys, n, shift, cnt);
    __syncthreads();
    uint32_t d = threadIdx.x, s = 0;
    for (int w = 0; w < RS_WARPS; w++) s += cnt[w][d];
    hist[(size_t)d * nblocks + blockIdx.x] = s;
}

__global__ void __launch_bounds__(256) k_radix_scatter(const uint32_t* __restrict__ keys,
                                                       const uint32_t* __restrict__ vals, uint32_t n, int shift,
                                                       uint32_t nblocks, const uint32_t* __restrict__ offs,
                                                       uint32_t* __restrict__ okeys, uint32_t* __restrict__ ovals) {
    __shared__ uint32_t cnt[RS_WARPS][257];
    for (int i = threadIdx.x; i < RS_WARPS * 257; i += blockDim.x) (&cnt[0][0])[i] = 0;
    __syncthreads();
    rs_count(keys, n, shift, cnt);
    __syncthreads();
    {
        uint32_t d = threadIdx.x;
        uint32_t run = offs[(size_t)d * nblocks + blockIdx.x];
        for (int w = 0; w < RS_WARPS; w++) { uint32_t t = cnt[w][d]; cnt[w][d] = run; run += t; }
    }
    __syncthreads();
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t base = blockIdx.x * RS_TILE + w * 32 * RS_ROUNDS;
    uint32_t lt = (1u << lane) - 1u;
    for (int r = 0; r < RS_ROUNDS; r++) {
        uint32_t i = base + r * 32 + lane;
        bool ok = i < n;
        uint32_t k = ok ? keys[i] : 0u;
        uint32_t d = ok ? (k >> shift) & 0xffu : 256u;
        uint32_t m = __match_any_sync(0xffffffffu, d);
        uint32_t pos = ok ? cnt[w][d] + __popc(m & lt) : 0u;
        __syncwarp();
        if (ok) {
            okeys[pos] = k;
            ovals[pos] = vals[i];
            if (lane == __ffs(m) - 1) cnt[w][d] += __popc(m);
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------------
// Karras 2012
// ---------------------------------------------------------------------------------
__device__ __forceinline__ int kdelta(const uint32_t* mort, const uint32_t* ids, int64_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= n) return -1;
    uint64_t a = ((uint64_t)mort[i] << 32) | ids[i], b = ((uint64_t)mort[j] << 32) | ids[j];
    return __clzll(a ^ b);
}

// bvh2 node = 10 words: left, right, first, last, lo[3], hi[3]
__global__ void k_karras(const uint32_t* __restrict__ mort, const uint32_t* __restrict__ ids, uint32_t n,
                         uint32_t* __restrict__ bvh2, uint32_t* __restrict__ parent) {
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= (int64_t)n - 1) return;
    int64_t N = n;
    int d = (kdelta(mort, ids, N, i, i + 1) - kdelta(mort, ids, N, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = kdelta(mort, ids, N, i, i - d);
    int64_t lmax = 2;
    while (kdelta(mort, ids, N, i, i + lmax * d) > dmin) lmax *= 2;
    int64_t l = 0;
    for (int64_t t = lmax / 2; t >= 1; t /= 2)
        if (kdelta(mort, ids, N, i, i + (l + t) * d) > dmin) l += t;
    int64_t j = i + l * d;
    int dnode = kdelta(mort, ids, N, i, j);
    int64_t s = 0;
    for (int64_t div = 2;; div *= 2) {
        int64_t t = (l + div - 1) / div;
        if (kdelta(mort, ids, N, i, i + (s + t) * d) > dnode) s += t;
        if (t == 1) break;
    }
    int64_t gamma = i + s * d + min(d, 0);
    int64_t lo = min(i, j), hi = max(i, j);
    uint32_t left = (lo == gamma) ? (kLeaf | (uint32_t)gamma) : (uint32_t)gamma;
    uint32_t right = (hi == gamma + 1) ? (kLeaf | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
    uint32_t* nd = bvh2 + (size_t)i * 10;
    nd[0] = left; nd[1] = right; nd[2] = (uint32_t)lo; nd[3] = (uint32_t)hi;
    // parent: internal nodes at [0, n-1), leaves at [n-1, 2n-1)
    parent[(left & kLeaf) ? (n - 1 + (left & ~kLeaf)) : left] = (uint32_t)i;
    parent[(right & kLeaf) ? (n - 1 + (right & ~kLeaf)) : right] = (uint32_t)i;
    if (i == 0) parent[0] = 0xffffffffu;
}

__device__ __forceinline__ void child_box(uint32_t c, const uint32_t* bvh2, const uint32_t* order,
                                          const float* tribox, float lo[3], float hi[3]) {
    if (c & kLeaf) {
        const float* b = tribox + (size_t)order[c & ~kLeaf] * 6;
        for (int a = 0; a < 3; a++) { lo[a] = __ldcg(b + a); hi[a] = __ldcg(b + 3 + a); }
    } else {
        const uint32_t* nd = bvh2 + (size_t)c * 10;
        for (int a = 0; a < 3; a++) {
            lo[a] = __uint_as_float(__ldcg(nd + 4 + a));
            hi[a] = __uint_as_float(__ldcg(nd + 7 + a));
        }
    }
}

__global__ void k_refit(const uint32_t* __restrict__ order, const float* __restrict__ tribox, uint32_t n,
                        uint32_t* bvh2, const uint32_t* __restrict__ parent, uint32_t* flags) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    uint32_t p = parent[n - 1 + j];
    while (p != 0xffffffffu) {
        __threadfence();
        if (atomicAdd(flags + p, 1u) == 0u) return;  // the sibling's thread finishes this node
        __threadfence();
        uint32_t* nd = bvh2 + (size_t)p * 10;
        float l0[3], h0[3], l1[3], h1[3];
        child_box(__ldcg(nd + 0), bvh2, order, tribox, l0, h0);
        child_box(__ldcg(nd + 1), bvh2, order, tribox, l1, h1);
        for (int a = 0; a < 3; a++) {
            __stcg(nd + 4 + a, __float_as_uint(fminf(l0[a], l1[a])));
            __stcg(nd + 7 + a, __float_as_uint(fmaxf(h0[a], h1[a])));
        }
        p = parent[p];
    }
}

// ---------------------------------------------------------------------------------
// BVH8 collapse
// ---------------------------------------------------------------------------------
struct Ref { float lo[3], hi[3]; uint32_t count, first; };

__device__ __forceinline__ Ref load_ref(uint32_t r, const uint32_t* bvh2, const uint32_t* order,
                                        const float* tribox) {
    Ref o;
    if (r & kLeaf) {
        const float* b = tribox + (size_t)order[r & ~kLeaf] * 6;
        for (int a = 0; a < 3; a++) { o.lo[a] = b[a]; o.hi[a] = b[3 + a]; }
        o.count = 1;
        o.first = r & ~kLeaf;
    } else {
        const uint32_t* nd = bvh2 + (size_t)r * 10;
        for (int a = 0; a < 3; a++) { o.lo[a] = __uint_as_float(nd[4 + a]); o.hi[a] = __uint_as_float(nd[7 + a]); }
        o.count = nd[3] - nd[2] + 1;
        o.first = nd[2];
    }
    return o;
}

__device__ __forceinline__ float surface(const Ref& b) {
    float dx = __fsub_rn(b.hi[0], b.lo[0]), dy = __fsub_rn(b.hi[1], b.lo[1]), dz = __fsub_rn(b.hi[2], b.lo[2]);
    float a = __fmul_rn(dx, dy);
    a = __fadd_rn(a, __fmul_rn(dy, dz));
    a = __fadd_rn(a, __fmul_rn(dz, dx));
    return a;
}

// Slot budgets of the collapse (surface area heuristic), bottom up: f(n, i) =
// the lowest cost of representing subtree n by at most i slots of its parent
// (a leaf slot of <= kLeafMax triangles: area x triangles x kCostTri; an
// internal node: area x kCostNode + its own 8 slots); a one-triangle leaf
// costs area x kCostTri.  dpk[n * 9]: left share k of the node's own 8 slots;
// dpk[n * 9 + i]: the left share of i slots, 0 for "i - 1 slots".  The second
// child to finish computes its parent (as k_refit), reading the first's
// values through L2; the float ops and tie rule (first strict minimum in k
// order) are the oracle's.
constexpr float kCostNode = 1.0f, kCostTri = 0.5f;

__device__ __forceinline__ float dp_cost(uint32_t m, int i, const float* dpf, const uint32_t* order,
                                         const float* tribox) {
    if (m & kLeaf) return __fmul_rn(surface(load_ref(m, nullptr, order, tribox)), kCostTri);
    return __ldcg(dpf + (size_t)m * 8 + i - 1);
}

__global__ void k_collapse_dp(const uint32_t* __restrict__ order, const float* __restrict__ tribox, uint32_t n,
                              const uint32_t* __restrict__ bvh2, const uint32_t* __restrict__ parent,
                              uint32_t* flags, float* dpf, uint8_t* dpk) {
    uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    uint32_t p = parent[n - 1 + j];
    while (p != 0xffffffffu) {
        __threadfence();
        if (atomicAdd(flags + p, 1u) == 0u) return;  // the sibling's thread computes this node
        __threadfence();
        const uint32_t* nd = bvh2 + (size_t)p * 10;
        const uint32_t L = __ldcg(nd + 0), R = __ldcg(nd + 1);
        float fl[8], fr[8];
#pragma unroll
        for (int i = 1; i <= 8; i++) {
            fl[i - 1] = dp_cost(L, i, dpf, order, tribox);
            fr[i - 1] = dp_cost(R, i, dpf, order, tribox);
        }
        Ref nb;
        for (int a = 0; a < 3; a++) {
            nb.lo[a] = __uint_as_float(__ldcg(nd + 4 + a));
            nb.hi[a] = __uint_as_float(__ldcg(nd + 7 + a));
        }
        const float A = surface(nb);
        const uint32_t cnt = __ldcg(nd + 3) - __ldcg(nd + 2) + 1;
        float best8 = INFINITY;
        int bk = 1;
#pragma unroll
        for (int k = 1; k <= 7; k++) {
            const float v = __fadd_rn(fl[k - 1], fr[8 - k - 1]);
            if (v < best8) { best8 = v; bk = k; }
        }
        float f[8];
        f[0] = cnt <= (uint32_t)kLeafMax ? __fmul_rn(__fmul_rn(A, __uint2float_rn(cnt)), kCostTri)
                                         : __fadd_rn(__fmul_rn(A, kCostNode), best8);
        uint8_t* kd = dpk + (size_t)p * 9;
        kd[0] = (uint8_t)bk;
#pragma unroll
        for (int i = 2; i <= 8; i++) {
            float v = f[i - 2];
            int kk = 0;
            for (int k = 1; k < i; k++) {
                const float w = __fadd_rn(fl[k - 1], fr[i - k - 1]);
                if (w < v) { v = w; kk = k; }
            }
            f[i - 1] = v;
            kd[i] = (uint8_t)kk;
        }
        float* fo = dpf + (size_t)p * 8;
#pragma unroll
        for (int i = 0; i < 8; i++) __stcg(fo + i, f[i]);
        p = parent[p];
    }
}

// plan: 8 BVH2 refs per node in slot order (0xffffffff = empty)
__global__ void k_collapse_plan(const uint32_t* __restrict__ lvl, uint32_t m, const uint32_t* __restrict__ bvh2,
                                const uint32_t* __restrict__ order, const float* __restrict__ tribox,
                                const uint8_t* __restrict__ dpk, uint32_t* __restrict__ plan,
                                uint32_t* __restrict__ ni, uint32_t* __restrict__ nt) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    uint32_t r = lvl[k];
    // children: the node's 8 slots spread over its subtree by the slot budgets,
    // left subtree first
    uint32_t C[8];
    int nc = 0;
    if (r & kLeaf) {
        C[nc++] = r;
    } else {
        uint32_t sm_[8];
        int si_[8], sp = 0;
        const int k0 = dpk[(size_t)r * 9];
        sm_[sp] = bvh2[(size_t)r * 10 + 1]; si_[sp++] = 8 - k0;
        sm_[sp] = bvh2[(size_t)r * 10 + 0]; si_[sp++] = k0;
        while (sp > 0) {
            const uint32_t mm = sm_[--sp];
            int i = si_[sp];
            while (!(mm & kLeaf) && i > 1 && dpk[(size_t)mm * 9 + i] == 0) i--;
            if ((mm & kLeaf) || i == 1) { C[nc++] = mm; continue; }
            const int kk = dpk[(size_t)mm * 9 + i];
            sm_[sp] = bvh2[(size_t)mm * 10 + 1]; si_[sp++] = i - kk;
            sm_[sp] = bvh2[(size_t)mm * 10 + 0]; si_[sp++] = kk;
        }
    }
    Ref nb = load_ref(r, bvh2, order, tribox);
    float pc[3];
    for (int a = 0; a < 3; a++) pc[a] = __fmul_rn(__fadd_rn(nb.lo[a], nb.hi[a]), 0.5f);
    float cost[8][8];
    uint32_t cnt[8];
    for (int i = 0; i < nc; i++) {
        Ref cb = load_ref(C[i], bvh2, order, tribox);
        cnt[i] = cb.count;
        float dd[3];
        for (int a = 0; a < 3; a++) dd[a] = __fsub_rn(__fmul_rn(__fadd_rn(cb.lo[a], cb.hi[a]), 0.5f), pc[a]);
        for (int sl = 0; sl < 8; sl++) {
            float c0 = (sl & 1) ? dd[0] : -dd[0];
            float c1 = (sl & 2) ? dd[1] : -dd[1];
            float c2 = (sl & 4) ? dd[2] : -dd[2];
            cost[i][sl] = __fadd_rn(__fadd_rn(c0, c1), c2);
        }
    }
    int slot_of[8], child_in_slot[8];
    for (int i = 0; i < 8; i++) { slot_of[i] = -1; child_in_slot[i] = -1; }
    for (int it = 0; it < nc; it++) {
        int bi = -1, bs = -1;
        float bc = 0.f;
        for (int i = 0; i < nc; i++) {
            if (slot_of[i] >= 0) continue;
            for (int sl = 0; sl < 8; sl++) {
                if (child_in_slot[sl] >= 0) continue;
                if (bi < 0 || cost[i][sl] > bc) { bi = i; bs = sl; bc = cost[i][sl]; }
            }
        }
        slot_of[bi] = bs;
        child_in_slot[bs] = bi;
    }
    uint32_t n_int = 0, n_tri = 0;
    for (int sl = 0; sl < 8; sl++) {
        int i = child_in_slot[sl];
        plan[(size_t)k * 8 + sl] = i < 0 ? 0xffffffffu : C[i];
        if (i < 0) continue;
        if (cnt[i] > (uint32_t)kLeafMax) n_int++;
        else n_tri += cnt[i];
    }
    ni[k] = n_int;
    nt[k] = n_tri;
}

// Node origin p = the node box's lo corner, per-axis power-of-two scale 2^e
// with 255 * 2^e >= extent (extent and division rounded up), child boxes
// quantised outwards: floor((lo - p)_rd / 2^e), ceil((hi - p)_ru / 2^e).
__device__ __forceinline__ void quantize_node(const Ref& nb, const uint32_t* slots, const uint32_t* bvh2,
                                              const uint32_t* order, const float* tribox, uint32_t& e3,
                                              uint32_t qlo[3][2], uint32_t qhi[3][2]) {
    float inv_s[3];
    e3 = 0;
    for (int a = 0; a < 3; a++) {
        float ext = __fsub_ru(nb.hi[a], nb.lo[a]);
        float t = __fdiv_ru(ext, 255.0f);
        uint32_t tb = __float_as_uint(t);
        int E = (int)((tb >> 23) & 0xffu);
        int ex = (E == 0) ? -100 : (E - 127 + ((tb & 0x7fffffu) ? 1 : 0));
        ex = max(-100, min(100, ex));
        e3 |= (uint32_t)(ex + 127) << (8 * a);
        inv_s[a] = __uint_as_float((uint32_t)(127 - ex) << 23);
        qlo[a][0] = qlo[a][1] = qhi[a][0] = qhi[a][1] = 0;
    }
    for (int sl = 0; sl < 8; sl++) {
        uint32_t c = slots[sl];
        if (c == 0xffffffffu) continue;
        Ref cb = load_ref(c, bvh2, order, tribox);
        int wsel = sl >> 2, sh = (sl & 3) * 8;
        for (int a = 0; a < 3; a++) {
            float lo = floorf(__fmul_rn(__fsub_rd(cb.lo[a], nb.lo[a]), inv_s[a]));
            float hi = ceilf(__fmul_rn(__fsub_ru(cb.hi[a], nb.lo[a]), inv_s[a]));
            lo = fminf(fmaxf(lo, 0.f), 255.f);
            hi = fminf(fmaxf(hi, 0.f), 255.f);
            qlo[a][wsel] |= (uint32_t)lo << sh;
            qhi[a][wsel] |= (uint32_t)hi << sh;
        }
    }
}

__global__ void k_collapse_emit(uint32_t m, uint32_t level_start, uint32_t tri_start, uint32_t node_off,
                                uint32_t rec_off,
                                const uint32_t* __restrict__ lvl, const uint32_t* __restrict__ plan,
                                const uint32_t* __restrict__ ni_scan, const uint32_t* __restrict__ nt_scan,
                                const uint32_t* __restrict__ bvh2, const uint32_t* __restrict__ order,
                                const float* __restrict__ tribox, const float4* __restrict__ world,
                                Node8* __restrict__ nodes, float4* __restrict__ tris, uint32_t* __restrict__ next,
                                uint32_t* __restrict__ node_ref, uint32_t* __restrict__ node_plan) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= m) return;
    Ref nb = load_ref(lvl[k], bvh2, order, tribox);
    uint32_t child_base = node_off + level_start + m + ni_scan[k];
    uint32_t tri_base = rec_off + tri_start + nt_scan[k];
    const uint32_t* slots = plan + (size_t)k * 8;
    // kept for refits: the node's BVH2 subtree and its children in slot order
    node_ref[level_start + k] = lvl[k];
    for (int sl = 0; sl < 8; sl++) node_plan[(size_t)(level_start + k) * 8 + sl] = slots[sl];
    uint32_t e3, qlo[3][2], qhi[3][2];
    quantize_node(nb, slots, bvh2, order, tribox, e3, qlo, qhi);
    uint32_t imask = 0, meta[2] = {0, 0};
    uint32_t toff = 0, rank = 0;
    for (int sl = 0; sl < 8; sl++) {
        uint32_t c = slots[sl];
        if (c == 0xffffffffu) continue;
        Ref cb = load_ref(c, bvh2, order, tribox);
        int wsel = sl >> 2, sh = (sl & 3) * 8;
        if (cb.count > (uint32_t)kLeafMax) {
            imask |= 1u << sl;
            meta[wsel] |= 0x80u << sh;
            next[ni_scan[k] + rank] = c;
            rank++;
        } else {
            meta[wsel] |= ((cb.count << 5) | toff) << sh;
            for (uint32_t j = 0; j < cb.count; j++) {
                uint32_t tid = order[cb.first + j];
                float4* dst = tris + (size_t)(tri_base + toff + j) * 3;
                float4 v0 = world[(size_t)tid * 3], v1 = world[(size_t)tid * 3 + 1], v2 = world[(size_t)tid * 3 + 2];
                v0.w = __uint_as_float(tid);
                v1.w = 0.f;
                v2.w = 0.f;
                dst[0] = v0; dst[1] = v1; dst[2] = v2;
            }
            toff += cb.count;
        }
    }
    Node8 nd;
    nd.q[0] = make_uint4(__float_as_uint(nb.lo[0]), __float_as_uint(nb.lo[1]), __float_as_uint(nb.lo[2]),
                         e3 | (imask << 24));
    nd.q[1] = make_uint4(child_base, tri_base, meta[0], meta[1]);
    nd.q[2] = make_uint4(qlo[0][0], qlo[0][1], qlo[1][0], qlo[1][1]);
    nd.q[3] = make_uint4(qlo[2][0], qlo[2][1], qhi[0][0], qhi[0][1]);
    nd.q[4] = make_uint4(qhi[1][0], qhi[1][1], qhi[2][0], qhi[2][1]);
    nodes[node_off + level_start + k] = nd;
}

// Refit: the same topology, slot order and child/triangle bases; only the
// node origin, exponents and quantised child boxes are recomputed from the
// refitted binary tree.
__global__ void k_requantize(uint32_t n_nodes, const uint32_t* __restrict__ node_ref,
                             const uint32_t* __restrict__ node_plan, const uint32_t* __restrict__ bvh2,
                             const uint32_t* __restrict__ order, const float* __restrict__ tribox,
                             Node8* __restrict__ nodes) {
    uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n_nodes) return;
    Ref nb = load_ref(node_ref[k], bvh2, order, tribox);
    uint32_t e3, qlo[3][2], qhi[3][2];
    quantize_node(nb, node_plan + (size_t)k * 8, bvh2, order, tribox, e3, qlo, qhi);
    Node8& nd = nodes[k];
    const uint32_t imask = nd.q[0].w >> 24;
    nd.q[0] = make_uint4(__float_as_uint(nb.lo[0]), __float_as_uint(nb.lo[1]), __float_as_uint(nb.lo[2]),
                         e3 | (imask << 24));
    nd.q[2] = make_uint4(qlo[0][0], qlo[0][1], qlo[1][0], qlo[1][1]);
    nd.q[3] = make_uint4(qlo[2][0], qlo[2][1], qhi[0][0], qhi[0][1]);
    nd.q[4] = make_uint4(qhi[1][0], qhi[1][1], qhi[2][0], qhi[2][1]);
}

// packed triangles take their (new) world vertices by the id they carry
__global__ void k_repack_tris(uint32_t n, const float4* __restrict__ world, float4* __restrict__ tris) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4* t = tris + (size_t)i * 3;
    const uint32_t id = __float_as_uint(t[0].w);
    float4 v0 = world[(size_t)id * 3], v1 = world[(size_t)id * 3 + 1], v2 = world[(size_t)id * 3 + 2];
    v0.w = __uint_as_float(id);
    v1.w = 0.f;
    v2.w = 0.f;
    t[0] = v0; t[1] = v1; t[2] = v2;
}

// ---------------------------------------------------------------------------------
static inline uint32_t cdiv(uint32_t a, uint32_t b) { return (a + b - 1) / b; }

int world_tris_impl(HyCtx* c) {
    const uint32_t n = c->ntri;
    int rc;
    if ((rc = ctx_alloc(c, c->world, (size_t)n * 48))) return rc;
    if ((rc = ctx_alloc(c, c->tribox, (size_t)n * 24))) return rc;
    if ((rc = ctx_alloc(c, c->centroid, (size_t)n * 16))) return rc;
    k_world_tris<<<cdiv(n, 256), 256, 0, c->stream>>>(
        c->verts.as<HyVertex>(), c->idx.as<uint32_t>(), c->prims.as<HyPrimitive>(), c->tri_prim.as<uint32_t>(),
        c->prim_tri0.as<uint32_t>(), c->xf.as<float>(), n, c->world.as<float4>(), c->tribox.as<float>(),
        c->centroid.as<float4>());
    HY_CUDA_TRY(cudaGetLastError());
    return HY_OK;
}

// Binary tree (SAH or LBVH) -> BVH8 over the n items in c->world / c->tribox / c->centroid (three
// points per item: a triangle, or an instance box as (lo, hi, hi)).  Nodes go
// to nodes[node_off ...], leaf records to records rec_off ...; the emitted
// child and record indices include the offsets.  Records carry the item's
// index.  Leaves the sorted keys / ids in keys[0] / vals[0] and the binary tree
// in bvh2 (the refit of a one-level structure reuses them).
static int build_core(HyCtx* c, uint32_t n, uint32_t node_off, uint32_t rec_off, uint32_t* n_nodes,
                      uint32_t* depth_out) {
    if (n == 0) return HY_ERR_NOT_READY;
    int rc;
    const uint32_t nb_rs = cdiv(n, RS_TILE);
    if ((rc = ctx_alloc(c, c->keys[0], (size_t)n * 4)) || (rc = ctx_alloc(c, c->keys[1], (size_t)n * 4)) ||
        (rc = ctx_alloc(c, c->vals[0], (size_t)n * 4)) || (rc = ctx_alloc(c, c->vals[1], (size_t)n * 4)) ||
        (rc = ctx_alloc(c, c->bounds, 64)) || (rc = ctx_alloc(c, c->hist, (size_t)256 * nb_rs * 4 * 2)) ||
        (rc = ctx_alloc(c, c->total, 64)) ||
        (rc = ctx_alloc(c, c->bvh2, (size_t)std::max<uint32_t>(n - 1, 1) * 40)) ||
        (rc = ctx_alloc(c, c->parent, (size_t)(2 * n) * 4)) ||
        (rc = ctx_alloc(c, c->flags, (size_t)std::max<uint32_t>(n, 1) * 4)) ||
        (rc = ctx_alloc(c, c->lvl_ref[0], (size_t)n * 4)) || (rc = ctx_alloc(c, c->lvl_ref[1], (size_t)n * 4)) ||
        (rc = ctx_alloc(c, c->plan, (size_t)n * 32)) || (rc = ctx_alloc(c, c->ni, (size_t)n * 4)) ||
        (rc = ctx_alloc(c, c->nt, (size_t)n * 4)) || (rc = ctx_alloc(c, c->ni_scan, (size_t)n * 4)) ||
        (rc = ctx_alloc(c, c->nt_scan, (size_t)n * 4)) ||
        (rc = ctx_alloc(c, c->node_ref, (size_t)std::max<uint32_t>(n, 1) * 4)) ||
        (rc = ctx_alloc(c, c->node_plan, (size_t)std::max<uint32_t>(n, 1) * 32)) ||
        (rc = ctx_alloc(c, c->dp_cost, (size_t)std::max<uint32_t>(n, 1) * 32)) ||
        (rc = ctx_alloc(c, c->dp_k, (size_t)std::max<uint32_t>(n, 1) * 9)))
        return rc;
    cudaStream_t s = c->stream;
    int* bnd = c->bounds.as<int>();
    k_bounds_init<<<1, 32, 0, s>>>(bnd);
    k_bounds<<<std::min<uint32_t>(cdiv(n, 256), 4 * (uint32_t)c->num_sms), 256, 0, s>>>(c->centroid.as<float4>(), n,
                                                                                         bnd);
    k_morton<<<cdiv(n, 256), 256, 0, s>>>(c->centroid.as<float4>(), n, bnd, c->keys[0].as<uint32_t>(),
                                          c->vals[0].as<uint32_t>());
    uint32_t* hist = c->hist.as<uint32_t>();
    uint32_t* offs = hist + (size_t)256 * nb_rs;
    int cur = 0;
    for (int shift = 0; shift < 32; shift += 8) {
        k_radix_hist<<<nb_rs, 256, 0, s>>>(c->keys[cur].as<uint32_t>(), n, shift, nb_rs, hist);
        if ((rc = scan_exclusive(c, hist, offs, 256 * nb_rs, nullptr))) return rc;
        k_radix_scatter<<<nb_rs, 256, 0, s>>>(c->keys[cur].as<uint32_t>(), c->vals[cur].as<uint32_t>(), n, shift,
                                              nb_rs, offs, c->keys[cur ^ 1].as<uint32_t>(),
                                              c->vals[cur ^ 1].as<uint32_t>());
        cur ^= 1;
    }
    HY_CUDA_TRY(cudaGetLastError());
    // after 4 passes the sorted arrays are back in buffer 0
    const uint32_t* mort = c->keys[cur].as<uint32_t>();
    const uint32_t* ord = c->vals[cur].as<uint32_t>();
    uint32_t* bvh2 = c->bvh2.as<uint32_t>();
    // root reference of the collapse
    uint32_t root = n > 1 ? 0u : kLeaf;
    HY_CUDA_TRY(cudaMemcpyAsync(c->lvl_ref[0].p, &root, 4, cudaMemcpyHostToDevice, s));
    if (n > 1) {
        if (c->build_mode == HY_BUILD_SAH) {
            // ids reordered in place; the SAH tree writes its root id into lvl_ref[0]
            if ((rc = sah_tree_impl(c, n, c->vals[cur].as<uint32_t>(), c->vals[cur ^ 1].as<uint32_t>(), bvh2,
                                    c->parent.as<uint32_t>(), c->lvl_ref[0].as<uint32_t>())))
                return rc;
            k_morton_at<<<cdiv(n, 256), 256, 0, s>>>(c->centroid.as<float4>(), n, bnd, ord,
                                                     c->keys[cur].as<uint32_t>());
        } else {
            k_karras<<<cdiv(n - 1, 256), 256, 0, s>>>(mort, ord, n, bvh2, c->parent.as<uint32_t>());
        }
        HY_CUDA_TRY(cudaMemsetAsync(c->flags.p, 0, (size_t)n * 4, s));
        k_refit<<<cdiv(n, 256), 256, 0, s>>>(ord, c->tribox.as<float>(), n, bvh2, c->parent.as<uint32_t>(),
                                             c->flags.as<uint32_t>());
        HY_CUDA_TRY(cudaMemsetAsync(c->flags.p, 0, (size_t)n * 4, s));
        k_collapse_dp<<<cdiv(n, 256), 256, 0, s>>>(ord, c->tribox.as<float>(), n, bvh2, c->parent.as<uint32_t>(),
                                                   c->flags.as<uint32_t>(), c->dp_cost.as<float>(),
                                                   c->dp_k.as<uint8_t>());
    }
    HY_CUDA_TRY(cudaGetLastError());
    uint32_t level_start = 0, tri_start = 0, m = 1, depth = 0;
    int lv = 0;
    uint32_t* tot = c->total.as<uint32_t>();
    while (m > 0) {
        const uint32_t* lvl = c->lvl_ref[lv].as<uint32_t>();
        k_collapse_plan<<<cdiv(m, 128), 128, 0, s>>>(lvl, m, bvh2, ord, c->tribox.as<float>(),
                                                     c->dp_k.as<uint8_t>(), c->plan.as<uint32_t>(),
                                                     c->ni.as<uint32_t>(), c->nt.as<uint32_t>());
        if ((rc = scan_exclusive(c, c->ni.as<uint32_t>(), c->ni_scan.as<uint32_t>(), m, tot))) return rc;
        if ((rc = scan_exclusive(c, c->nt.as<uint32_t>(), c->nt_scan.as<uint32_t>(), m, tot + 1))) return rc;
        k_collapse_emit<<<cdiv(m, 128), 128, 0, s>>>(m, level_start, tri_start, node_off, rec_off, lvl,
                                                     c->plan.as<uint32_t>(),
                                                     c->ni_scan.as<uint32_t>(), c->nt_scan.as<uint32_t>(), bvh2, ord,
                                                     c->tribox.as<float>(), c->world.as<float4>(),
                                                     c->nodes.as<Node8>(), c->tris.as<float4>(),
                                                     c->lvl_ref[lv ^ 1].as<uint32_t>(), c->node_ref.as<uint32_t>(),
                                                     c->node_plan.as<uint32_t>());
        HY_CUDA_TRY(cudaGetLastError());
        uint32_t h_tot[2];
        HY_CUDA_TRY(cudaMemcpyAsync(h_tot, tot, 8, cudaMemcpyDeviceToHost, s));
        HY_CUDA_TRY(cudaStreamSynchronize(s));
        level_start += m;
        tri_start += h_tot[1];
        m = h_tot[0];
        lv ^= 1;
        depth++;
        if (depth > 256) return HY_ERR_TIMEOUT;
    }
    if (tri_start != n) return HY_ERR_CUDA;
    *n_nodes = level_start;
    *depth_out = depth;
    return HY_OK;
}

int bvh_build_impl(HyCtx* c, HyBvhStats* st) {
    const uint32_t n = c->ntri;
    if (n == 0) return HY_ERR_NOT_READY;
    int rc;
    c->bvh_ok = false;
    c->two_level = false;
    cudaEvent_t e0, e1;
    HY_CUDA_TRY(cudaEventCreate(&e0));
    HY_CUDA_TRY(cudaEventCreate(&e1));
    HY_CUDA_TRY(cudaEventRecord(e0, c->stream));
    if ((rc = world_tris_impl(c))) return rc;
    if ((rc = ctx_alloc(c, c->nodes, (size_t)std::max<uint32_t>(n, 1) * sizeof(Node8))) ||
        (rc = ctx_alloc(c, c->tris, (size_t)n * 48)))
        return rc;
    uint32_t n_nodes = 0, depth = 0;
    if ((rc = build_core(c, n, 0, 0, &n_nodes, &depth))) return rc;
    HY_CUDA_TRY(cudaEventRecord(e1, c->stream));
    HY_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->n_bvh8 = n_nodes;
    c->n_records = n;
    c->depth = depth;
    c->bvh_ok = true;
    int hb[6];
    HY_CUDA_TRY(cudaMemcpy(hb, c->bounds.p, 24, cudaMemcpyDeviceToHost));
    HyBvhStats out{};
    out.num_tris = n;
    out.num_bvh2_nodes = n > 1 ? n - 1 : 0;
    out.num_bvh8_nodes = n_nodes;
    out.depth = depth;
    out.build_ms = ms;
    for (int a = 0; a < 3; a++) {
        int lo = hb[a], hi = hb[3 + a];
        lo = lo >= 0 ? lo : lo ^ 0x7fffffff;
        hi = hi >= 0 ? hi : hi ^ 0x7fffffff;
        memcpy(&out.scene_lo[a], &lo, 4);
        memcpy(&out.scene_hi[a], &hi, 4);
    }
    c->last_build = out;
    if (st) *st = out;
    return HY_OK;
}

// Refit: new transforms, same topology.  Re-transforms the triangles, refits
// the binary tree and re-encodes every 8-wide node and triangle record level by
// level with the stored plan of the last build.
int bvh_refit_impl(HyCtx* c) {
    const uint32_t n = c->ntri;
    int rc;
    cudaStream_t s = c->stream;
    if ((rc = world_tris_impl(c))) return rc;
    if (n > 1) {
        HY_CUDA_TRY(cudaMemsetAsync(c->flags.p, 0, (size_t)n * 4, s));
        k_refit<<<cdiv(n, 256), 256, 0, s>>>(c->vals[0].as<uint32_t>(), c->tribox.as<float>(), n,
                                             c->bvh2.as<uint32_t>(), c->parent.as<uint32_t>(),
                                             c->flags.as<uint32_t>());
    }
    k_requantize<<<cdiv(c->n_bvh8, 128), 128, 0, s>>>(c->n_bvh8, c->node_ref.as<uint32_t>(),
                                                      c->node_plan.as<uint32_t>(), c->bvh2.as<uint32_t>(),
                                                      c->vals[0].as<uint32_t>(), c->tribox.as<float>(),
                                                      c->nodes.as<Node8>());
    k_repack_tris<<<cdiv(n, 256), 256, 0, s>>>(n, c->world.as<float4>(), c->tris.as<float4>());
    HY_CUDA_TRY(cudaGetLastError());
    HY_CUDA_TRY(cudaStreamSynchronize(s));
    return HY_OK;
}

// ---------------------------------------------------------------------------------
// Two-level structure: one BLAS per distinct mesh over its object-space
// triangles, a TLAS over the instance boxes (the driver's BLAS-per-primitive
// and TLAS builds of src/vk_mesh.cpp:424-492 and src/renderer.cpp:1696-1865).
// ---------------------------------------------------------------------------------

// object-space triangles of one mesh; x + 0 folds -0 into +0 so box bits do
// not depend on the sign of zero
__global__ void k_mesh_tris(const HyVertex* __restrict__ verts, const uint32_t* __restrict__ idx,
                            uint32_t first_index, uint32_t vertex_offset, uint32_t n, float4* __restrict__ world,
                            float* __restrict__ tribox, float4* __restrict__ cen) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int v = 0; v < 3; v++) {
        const float* P = verts[idx[first_index + 3 * t + v] + vertex_offset].pos;
        float w[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            w[a] = __fadd_rn(P[a], 0.0f);
            lo[a] = fminf(lo[a], w[a]);
            hi[a] = fmaxf(hi[a], w[a]);
        }
        world[(size_t)t * 3 + v] = make_float4(w[0], w[1], w[2], 0.f);
    }
    float* b = tribox + (size_t)t * 6;
    for (int a = 0; a < 3; a++) { b[a] = lo[a]; b[3 + a] = hi[a]; }
    cen[t] = make_float4(__fmul_rn(__fadd_rn(lo[0], hi[0]), 0.5f), __fmul_rn(__fadd_rn(lo[1], hi[1]), 0.5f),
                         __fmul_rn(__fadd_rn(lo[2], hi[2]), 0.5f), 0.f);
}

// smallest / largest vertex index a mesh's triangles use (out: min, max)
__global__ void k_mesh_vrange(const uint32_t* __restrict__ idx, uint32_t n, uint32_t* __restrict__ out) {
    uint32_t lo = 0xffffffffu, hi = 0;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t v = idx[k];
        lo = min(lo, v);
        hi = max(hi, v);
    }
    for (int o = 16; o > 0; o >>= 1) {
        lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    if ((threadIdx.x & 31) == 0) { atomicMin(out, lo); atomicMax(out + 1, hi); }
}

// doubles as order-preserving signed 64-bit keys (-0 below +0)
__device__ __forceinline__ long long d2ord(double x) {
    const long long b = __double_as_longlong(x);
    return b >= 0 ? b : b ^ 0x7fffffffffffffffll;
}
__device__ __forceinline__ double ord2d(long long k) {
    return __longlong_as_double(k >= 0 ? k : k ^ 0x7fffffffffffffffll);
}

__global__ void k_inst_box_init(uint32_t ninst, long long* __restrict__ keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ninst) return;
    for (int a = 0; a < 3; a++) {
        keys[(size_t)i * 6 + a] = d2ord(INFINITY);
        keys[(size_t)i * 6 + 3 + a] = d2ord(-INFINITY);
    }
}

// World box of an instance, one chunk (instance, first vertex, end vertex) of
// its mesh's vertex range per block: each vertex through the object->world
// matrix in double, ((m0 x + m1 y) + m2 z) + m3, min / max folded into the
// instance's keys (min and max are exact, so the order does not matter)
__global__ void __launch_bounds__(128) k_inst_box(const uint4* __restrict__ chunks,
                                                  const uint32_t* __restrict__ inst_prim,
                                                  const HyPrimitive* __restrict__ prims,
                                                  const HyVertex* __restrict__ verts, const float* __restrict__ xf,
                                                  long long* __restrict__ keys) {
    const uint4 ch = chunks[blockIdx.x];
    const float* M = xf + (size_t)prims[inst_prim[ch.x]].transform_id * 16;
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t v = ch.y + threadIdx.x; v < ch.z; v += blockDim.x) {
        const float* P = verts[v].pos;
#pragma unroll
        for (int r = 0; r < 3; r++) {
            double w = __dmul_rn((double)M[0 * 4 + r], (double)P[0]);
            w = __dadd_rn(w, __dmul_rn((double)M[1 * 4 + r], (double)P[1]));
            w = __dadd_rn(w, __dmul_rn((double)M[2 * 4 + r], (double)P[2]));
            w = __dadd_rn(w, (double)M[3 * 4 + r]);
            lo[r] = fmin(lo[r], w);
            hi[r] = fmax(hi[r], w);
        }
    }
    long long* k = keys + (size_t)ch.x * 6;
#pragma unroll
    for (int a = 0; a < 3; a++) {
        long long kl = d2ord(lo[a]), kh = d2ord(hi[a]);
        for (int o = 16; o > 0; o >>= 1) {
            kl = min(kl, __shfl_xor_sync(0xffffffffu, kl, o));
            kh = max(kh, __shfl_xor_sync(0xffffffffu, kh, o));
        }
        if ((threadIdx.x & 31) == 0) {
            atomicMin(k + a, kl);
            atomicMax(k + 3 + a, kh);
        }
    }
}

// Instance records and TLAS items.  Record: the world->object rows of the
// instance's transform, then (BLAS root node, first global triangle,
// primitive, 0).  Box: the vertex-range box, padded by 2^-16 of the extent
// plus 2^-20 of the largest magnitude plus 2^-60 per axis (room for the
// rounding of the world->object ray transform; the last term also makes the
// result independent of the sign of a zero) and rounded outwards to float.
__global__ void k_inst_setup(uint32_t ninst, const uint32_t* __restrict__ inst_prim,
                             const HyPrimitive* __restrict__ prims, const uint32_t* __restrict__ prim_mesh,
                             const uint32_t* __restrict__ blas_node0, const uint32_t* __restrict__ prim_tri0,
                             const float* __restrict__ xinv, const long long* __restrict__ keys,
                             float4* __restrict__ inst, float* __restrict__ inst_box, float4* __restrict__ world,
                             float* __restrict__ tribox, float4* __restrict__ cen) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ninst) return;
    const uint32_t p = inst_prim[i], m = prim_mesh[p], tf = prims[p].transform_id;
    const float* R = xinv + (size_t)tf * 12;
    for (int k = 0; k < 3; k++) inst[(size_t)i * 4 + k] = make_float4(R[4 * k], R[4 * k + 1], R[4 * k + 2], R[4 * k + 3]);
    inst[(size_t)i * 4 + 3] = make_float4(__uint_as_float(blas_node0[m]), __uint_as_float(prim_tri0[p]),
                                          __uint_as_float(p), 0.f);
    float bl[3], bh[3];
    for (int a = 0; a < 3; a++) {
        const double lo = ord2d(keys[(size_t)i * 6 + a]), hi = ord2d(keys[(size_t)i * 6 + 3 + a]);
        const double mag = fmax(fabs(lo), fabs(hi));
        const double pad =
            __dadd_rn(__dadd_rn(__dmul_rn(__dsub_rn(hi, lo), 0x1p-16), __dmul_rn(mag, 0x1p-20)), 0x1p-60);
        bl[a] = __double2float_rd(__dsub_rn(lo, pad));
        bh[a] = __double2float_ru(__dadd_rn(hi, pad));
        inst_box[(size_t)i * 6 + a] = bl[a];
        inst_box[(size_t)i * 6 + 3 + a] = bh[a];
        tribox[(size_t)i * 6 + a] = bl[a];
        tribox[(size_t)i * 6 + 3 + a] = bh[a];
    }
    world[(size_t)i * 3 + 0] = make_float4(bl[0], bl[1], bl[2], 0.f);
    world[(size_t)i * 3 + 1] = make_float4(bh[0], bh[1], bh[2], 0.f);
    world[(size_t)i * 3 + 2] = make_float4(bh[0], bh[1], bh[2], 0.f);
    cen[i] = make_float4(__fmul_rn(__fadd_rn(bl[0], bh[0]), 0.5f), __fmul_rn(__fadd_rn(bl[1], bh[1]), 0.5f),
                         __fmul_rn(__fadd_rn(bl[2], bh[2]), 0.5f), 0.f);
}

int tlas_build_impl(HyCtx* c) {
    const uint32_t ni = c->ninst;
    int rc;
    cudaStream_t s = c->stream;
    if ((rc = ctx_alloc(c, c->inst, (size_t)ni * 64)) || (rc = ctx_alloc(c, c->inst_box, (size_t)ni * 24)) ||
        (rc = ctx_alloc(c, c->inst_keys, (size_t)ni * 48)) ||
        (rc = ctx_alloc(c, c->world, (size_t)ni * 48)) || (rc = ctx_alloc(c, c->tribox, (size_t)ni * 24)) ||
        (rc = ctx_alloc(c, c->centroid, (size_t)ni * 16)))
        return rc;
    long long* keys = c->inst_keys.as<long long>();
    k_inst_box_init<<<cdiv(ni, 128), 128, 0, s>>>(ni, keys);
    k_inst_box<<<c->n_chunks, 128, 0, s>>>(c->inst_chunks.as<uint4>(), c->inst_prim.as<uint32_t>(),
                                           c->prims.as<HyPrimitive>(), c->verts.as<HyVertex>(), c->xf.as<float>(),
                                           keys);
    k_inst_setup<<<cdiv(ni, 128), 128, 0, s>>>(
        ni, c->inst_prim.as<uint32_t>(), c->prims.as<HyPrimitive>(), c->prim_mesh.as<uint32_t>(),
        c->blas_node0.as<uint32_t>(), c->prim_tri0.as<uint32_t>(), c->xinv.as<float>(), keys, c->inst.as<float4>(),
        c->inst_box.as<float>(), c->world.as<float4>(), c->tribox.as<float>(), c->centroid.as<float4>());
    HY_CUDA_TRY(cudaGetLastError());
    HY_CUDA_TRY(cudaMemsetAsync(c->nodes.p, 0, (size_t)c->tlas_region * sizeof(Node8), s));
    HY_CUDA_TRY(cudaMemsetAsync(c->tris.p, 0, (size_t)c->tlas_region * 48, s));
    uint32_t nn = 0, depth = 0;
    if ((rc = build_core(c, ni, 0, 0, &nn, &depth))) return rc;
    HY_CUDA_TRY(cudaStreamSynchronize(s));
    c->tlas_nodes = nn;
    c->tlas_depth = depth;
    c->depth = c->tlas_depth + c->blas_depth;
    return HY_OK;
}

int bvh_build_instanced_impl(HyCtx* c, HyBvhStats* st) {
    c->bvh_ok = false;
    c->two_level = false;
    const uint32_t np = c->nprims;
    if (c->h_prims.size() != np) return HY_ERR_NOT_READY;
    // distinct meshes in order of first use; one instance per primitive with triangles
    c->h_prim_mesh.assign(np, 0xffffffffu);
    c->h_mesh_prim.clear();
    c->h_inst_prim.clear();
    {
        // (first_index, index_count, vertex_offset) -> mesh, through 1024 hash buckets
        std::vector<std::vector<uint32_t>> bucket(1024);
        for (uint32_t p = 0; p < np; p++) {
            const HyPrimitive& pr = c->h_prims[p];
            if (pr.index_count / 3 == 0) continue;
            const uint64_t h = ((uint64_t)pr.first_index * 0x9E3779B97F4A7C15ull) ^
                               ((uint64_t)pr.index_count * 0xC2B2AE3D27D4EB4Full) ^ (uint64_t)pr.vertex_offset;
            std::vector<uint32_t>& b = bucket[(h >> 20) & 1023u];
            uint32_t m = 0xffffffffu;
            for (uint32_t cand : b) {
                const HyPrimitive& q = c->h_prims[c->h_mesh_prim[cand]];
                if (q.first_index == pr.first_index && q.index_count == pr.index_count &&
                    q.vertex_offset == pr.vertex_offset) { m = cand; break; }
            }
            if (m == 0xffffffffu) {
                m = (uint32_t)c->h_mesh_prim.size();
                c->h_mesh_prim.push_back(p);
                b.push_back(m);
            }
            c->h_prim_mesh[p] = m;
            c->h_inst_prim.push_back(p);
        }
    }
    c->ninst = (uint32_t)c->h_inst_prim.size();
    c->nblas = (uint32_t)c->h_mesh_prim.size();
    if (c->ninst == 0) return HY_ERR_NOT_READY;
    c->tlas_region = c->ninst;
    uint64_t node_cap = c->tlas_region, rec_cap = c->tlas_region;
    uint32_t max_nt = c->ninst;
    for (uint32_t m = 0; m < c->nblas; m++) {
        const uint32_t nt = c->h_prims[c->h_mesh_prim[m]].index_count / 3;
        node_cap += std::max<uint32_t>(nt, 1);
        rec_cap += nt;
        max_nt = std::max(max_nt, nt);
    }
    if (node_cap >= (1ull << 31) || rec_cap >= (1ull << 31)) return HY_ERR_TOO_LARGE;
    int rc;
    cudaStream_t s = c->stream;
    if ((rc = ctx_alloc(c, c->nodes, (size_t)node_cap * sizeof(Node8))) ||
        (rc = ctx_alloc(c, c->tris, (size_t)rec_cap * 48)) ||
        (rc = ctx_alloc(c, c->world, (size_t)max_nt * 48)) || (rc = ctx_alloc(c, c->tribox, (size_t)max_nt * 24)) ||
        (rc = ctx_alloc(c, c->centroid, (size_t)max_nt * 16)) ||
        (rc = ctx_alloc(c, c->mesh_vrange, (size_t)c->nblas * 8)) ||
        (rc = ctx_alloc(c, c->prim_mesh, (size_t)np * 4)) || (rc = ctx_alloc(c, c->inst_prim, (size_t)c->ninst * 4)) ||
        (rc = ctx_alloc(c, c->blas_node0, (size_t)c->nblas * 4)))
        return rc;
    cudaEvent_t e0, e1;
    HY_CUDA_TRY(cudaEventCreate(&e0));
    HY_CUDA_TRY(cudaEventCreate(&e1));
    HY_CUDA_TRY(cudaEventRecord(e0, s));
    HY_CUDA_TRY(cudaMemsetAsync(c->nodes.p, 0, (size_t)node_cap * sizeof(Node8), s));
    HY_CUDA_TRY(cudaMemsetAsync(c->tris.p, 0, (size_t)rec_cap * 48, s));
    HY_CUDA_TRY(cudaMemcpyAsync(c->prim_mesh.p, c->h_prim_mesh.data(), (size_t)np * 4, cudaMemcpyHostToDevice, s));
    std::vector<uint32_t> vr_init((size_t)c->nblas * 2);
    for (uint32_t m = 0; m < c->nblas; m++) { vr_init[2 * m] = 0xffffffffu; vr_init[2 * m + 1] = 0; }
    HY_CUDA_TRY(cudaMemcpyAsync(c->mesh_vrange.p, vr_init.data(), vr_init.size() * 4, cudaMemcpyHostToDevice, s));
    HY_CUDA_TRY(cudaMemcpyAsync(c->inst_prim.p, c->h_inst_prim.data(), (size_t)c->ninst * 4, cudaMemcpyHostToDevice,
                                s));
    uint32_t node_off = c->tlas_region, rec_off = c->tlas_region;
    c->h_blas_node0.assign(c->nblas, 0);
    c->blas_depth = 0;
    for (uint32_t m = 0; m < c->nblas; m++) {
        const HyPrimitive& pr = c->h_prims[c->h_mesh_prim[m]];
        const uint32_t nt = pr.index_count / 3;
        k_mesh_tris<<<cdiv(nt, 256), 256, 0, s>>>(c->verts.as<HyVertex>(), c->idx.as<uint32_t>(), pr.first_index,
                                                  pr.vertex_offset, nt, c->world.as<float4>(), c->tribox.as<float>(),
                                                  c->centroid.as<float4>());
        HY_CUDA_TRY(cudaGetLastError());
        uint32_t nn = 0, depth = 0;
        if ((rc = build_core(c, nt, node_off, rec_off, &nn, &depth))) return rc;
        k_mesh_vrange<<<std::min<uint32_t>(cdiv(nt * 3, 256), 4 * (uint32_t)c->num_sms), 256, 0, s>>>(
            c->idx.as<uint32_t>() + pr.first_index, nt * 3, c->mesh_vrange.as<uint32_t>() + (size_t)m * 2);
        HY_CUDA_TRY(cudaGetLastError());
        c->h_blas_node0[m] = node_off;
        node_off += nn;
        rec_off += nt;
        c->blas_depth = std::max(c->blas_depth, depth);
    }
    HY_CUDA_TRY(cudaMemcpyAsync(c->blas_node0.p, c->h_blas_node0.data(), (size_t)c->nblas * 4,
                                cudaMemcpyHostToDevice, s));
    // per-frame box work: each instance's vertex range in chunks of 1024 vertices
    std::vector<uint32_t> vr((size_t)c->nblas * 2);
    HY_CUDA_TRY(cudaMemcpyAsync(vr.data(), c->mesh_vrange.p, vr.size() * 4, cudaMemcpyDeviceToHost, s));
    HY_CUDA_TRY(cudaStreamSynchronize(s));
    std::vector<uint4> chunks;
    for (uint32_t i = 0; i < c->ninst; i++) {
        const uint32_t p = c->h_inst_prim[i], m = c->h_prim_mesh[p];
        const uint32_t v0 = c->h_prims[p].vertex_offset + vr[2 * m], v1 = c->h_prims[p].vertex_offset + vr[2 * m + 1] + 1;
        for (uint32_t v = v0; v < v1; v += 1024) chunks.push_back(make_uint4(i, v, std::min(v1, v + 1024), 0));
    }
    c->n_chunks = (uint32_t)chunks.size();
    if ((rc = ctx_alloc(c, c->inst_chunks, chunks.size() * sizeof(uint4)))) return rc;
    HY_CUDA_TRY(cudaMemcpyAsync(c->inst_chunks.p, chunks.data(), chunks.size() * sizeof(uint4),
                                cudaMemcpyHostToDevice, s));
    c->n_bvh8 = node_off;
    c->n_records = rec_off;
    if ((rc = tlas_build_impl(c))) return rc;
    HY_CUDA_TRY(cudaEventRecord(e1, s));
    HY_CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    c->two_level = true;
    c->bvh_ok = true;
    HyBvhStats out{};
    out.num_tris = c->ntri;
    out.num_bvh2_nodes = 0;
    out.num_bvh8_nodes = c->n_bvh8;
    out.depth = c->depth;
    out.build_ms = ms;
    // scene bounds: the union of the instance boxes
    std::vector<float> boxes((size_t)c->ninst * 6);
    HY_CUDA_TRY(cudaMemcpy(boxes.data(), c->inst_box.p, boxes.size() * 4, cudaMemcpyDeviceToHost));
    for (int a = 0; a < 3; a++) { out.scene_lo[a] = INFINITY; out.scene_hi[a] = -INFINITY; }
    for (uint32_t i = 0; i < c->ninst; i++)
        for (int a = 0; a < 3; a++) {
            out.scene_lo[a] = std::min(out.scene_lo[a], boxes[(size_t)i * 6 + a]);
            out.scene_hi[a] = std::max(out.scene_hi[a], boxes[(size_t)i * 6 + 3 + a]);
        }
    c->last_build = out;
    if (st) *st = out;
    return HY_OK;
}

}  // namespace hy
