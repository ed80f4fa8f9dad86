// ORACLE — test infrastructure only (see orc_math.hpp).
//
// CPU restatement of the acceleration structure that replaces the driver's
// BLAS/TLAS (src/renderer.cpp:1696-1865) and of its traversal (the hidden part
// of traceRayEXT at shadowRaygen.rgen:78, hybridRaygen.rgen:158,
// hybridHit.rchit:322).  The algorithm is written down here in plain C++ so the
// product's GPU build can be compared with it array for array:
//
//   1. world triangles: M * v with the fixed, unfused order ((m0 x + m1 y) + m2 z) + m3
//   2. 30-bit Morton codes of the AABB centroids over the centroid bounds
//   3. stable sort by Morton code (ties keep triangle order)
//   4. binary tree over that order, by the scene's build mode:
//      SAH  — top down, each range split where the binned surface area
//             heuristic is lowest (32 bins per axis over its centroid bounds),
//             the two sides stably partitioned (sah_tree below);
//      LBVH — Karras 2012 binary radix tree over the 64-bit keys (morton << 32 | id)
//   5. bottom-up box refit
//   6. BFS collapse into 8-wide nodes: each node's 8 slots spread over its
//      subtree by a surface-area-heuristic dynamic program over slot budgets,
//      then children assigned to octant slots by a greedy maximum of
//      dot(child centroid - node centroid, slot corner)
//   7. quantise child boxes to 8 bits per axis against a power-of-two scale
//      (Ylitie, Karras & Laine 2017 node format), rounding outwards
//
// Compiled with -ffp-contract=off -frounding-math: every float operation is a
// single IEEE-rounded op, as the CUDA build writes them with __f*_rn/_rd/_ru.
#include <algorithm>
#include <cfenv>
#include <cstdio>
#include <numeric>

#include "orc_scene.hpp"

namespace orc {

static inline float fmin2(float a, float b) { return std::fmin(a, b); }
static inline float fmax2(float a, float b) { return std::fmax(a, b); }

static float sub_dir(float a, float b, int mode) {
    std::fesetround(mode);
    volatile float va = a, vb = b;
    volatile float r = va - vb;
    std::fesetround(FE_TONEAREST);
    return r;
}
static float div_up(float a, float b) {
    std::fesetround(FE_UPWARD);
    volatile float va = a, vb = b;
    volatile float r = va / vb;
    std::fesetround(FE_TONEAREST);
    return r;
}

static void inverse4(const double* m, double* inv) {
    // cofactor expansion, column-major in and out
    double a[16];
    for (int i = 0; i < 16; i++) a[i] = m[i];
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

void scene_derive(Scene& s) {
    s.prim_tri0.resize(s.prims.size());
    uint32_t nt = 0;
    for (size_t p = 0; p < s.prims.size(); p++) { s.prim_tri0[p] = nt; nt += s.prims[p].index_count / 3; }
    s.ntri = nt;
    s.tri_prim.assign(nt, 0);
    for (size_t p = 0; p < s.prims.size(); p++)
        for (uint32_t k = 0; k < s.prims[p].index_count / 3; k++) s.tri_prim[s.prim_tri0[p] + k] = (uint32_t)p;
    derive_world(s);
    s.bvh_ok = false;
}

void derive_world(Scene& s) {
    // normal matrices: mat3(transpose(inverse(model))) (hybridHit.rchit:26, basic.vert:44)
    size_t nx = s.xf.size() / 16;
    s.nrm.assign(nx * 9, 0.f);
    for (size_t t = 0; t < nx; t++) {
        double m[16], inv[16];
        for (int i = 0; i < 16; i++) m[i] = s.xf[t * 16 + i];
        inverse4(m, inv);
        // nrm(r, c) = inv(c, r); column-major: nrm[c*3 + r] = inv[r*4 + c]
        for (int c = 0; c < 3; c++)
            for (int r = 0; r < 3; r++) s.nrm[t * 9 + c * 3 + r] = (float)inv[r * 4 + c];
    }
    s.world.assign((size_t)s.ntri * 9, 0.f);
    for (size_t p = 0; p < s.prims.size(); p++) {
        const HyPrimitive& pr = s.prims[p];
        const float* M = &s.xf[(size_t)pr.transform_id * 16];
        for (uint32_t k = 0; k < pr.index_count / 3; k++) {
            uint32_t t = s.prim_tri0[p] + k;
            for (int v = 0; v < 3; v++) {
                uint32_t vi = s.idx[pr.first_index + 3 * k + v] + pr.vertex_offset;
                const float* P = s.verts[vi].pos;
                for (int r = 0; r < 3; r++) {
                    float acc = M[0 * 4 + r] * P[0];
                    acc = acc + M[1 * 4 + r] * P[1];
                    acc = acc + M[2 * 4 + r] * P[2];
                    acc = acc + M[3 * 4 + r];
                    s.world[(size_t)t * 9 + v * 3 + r] = acc;
                }
            }
        }
    }
}

static inline uint32_t expand10(uint32_t v) {
    v &= 0x3ffu;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

static inline int clz64(uint64_t x) { return x ? __builtin_clzll(x) : 64; }

struct Box { float lo[3], hi[3]; };

// boxes of the binary tree, bottom-up (the union is order independent)
static void refit_bvh2(Bvh& B, const std::vector<Box>& tb) {
    const uint32_t n = B.n;
    if (n < 2) return;
    std::vector<uint32_t> stack;
    std::vector<uint8_t> done(n - 1, 0);
    stack.push_back(B.root);
    while (!stack.empty()) {
        uint32_t i = stack.back();
        Bvh2Node& nd = B.bvh2[i];
        bool ready = true;
        for (uint32_t c : {nd.left, nd.right})
            if (!(c & kLeafBit) && !done[c]) { stack.push_back(c); ready = false; }
        if (!ready) continue;
        stack.pop_back();
        for (int a = 0; a < 3; a++) {
            float lo2[2], hi2[2];
            int k = 0;
            for (uint32_t c : {nd.left, nd.right}) {
                if (c & kLeafBit) {
                    const Box& b = tb[B.order[c & ~kLeafBit]];
                    lo2[k] = b.lo[a]; hi2[k] = b.hi[a];
                } else {
                    lo2[k] = B.bvh2[c].lo[a]; hi2[k] = B.bvh2[c].hi[a];
                }
                k++;
            }
            nd.lo[a] = fmin2(lo2[0], lo2[1]);
            nd.hi[a] = fmax2(hi2[0], hi2[1]);
        }
        done[i] = 1;
    }
}

static std::vector<Box> tri_boxes(const Scene& s) {
    std::vector<Box> tb(s.ntri);
    for (uint32_t t = 0; t < s.ntri; t++) {
        const float* w = &s.world[(size_t)t * 9];
        for (int a = 0; a < 3; a++) {
            tb[t].lo[a] = fmin2(fmin2(w[a], w[3 + a]), w[6 + a]);
            tb[t].hi[a] = fmax2(fmax2(w[a], w[3 + a]), w[6 + a]);
        }
    }
    return tb;
}

static Box ref_box_of(const Bvh& B, const std::vector<Box>& tb, uint32_t r) {
    if (r & kLeafBit) return tb[B.order[r & ~kLeafBit]];
    Box b;
    for (int a = 0; a < 3; a++) { b.lo[a] = B.bvh2[r].lo[a]; b.hi[a] = B.bvh2[r].hi[a]; }
    return b;
}

// Node origin p = the node box's lo corner, per-axis power-of-two scale 2^e
// with 255 * 2^e >= extent (extent and division rounded up), child boxes
// quantised outwards.  Writes w[0..2], the exponent bytes of w[3] (keeping
// its internal mask byte) and w[8..19].
static void quantize_node(const Bvh& B, const std::vector<Box>& tb, uint32_t ref, const uint32_t* slots,
                          uint32_t* w) {
    Box nb = ref_box_of(B, tb, ref);
    uint32_t e3 = 0;
    float inv_s[3];
    for (int a = 0; a < 3; a++) {
        w[a] = fbits(nb.lo[a]);
        float ext = sub_dir(nb.hi[a], nb.lo[a], FE_UPWARD);
        float t = div_up(ext, 255.0f);
        uint32_t tb_ = fbits(t);
        int E = (int)((tb_ >> 23) & 0xffu);
        int ex = (E == 0) ? -100 : (E - 127 + ((tb_ & 0x7fffffu) ? 1 : 0));
        ex = std::max(-100, std::min(100, ex));
        e3 |= (uint32_t)(ex + 127) << (8 * a);
        inv_s[a] = bitsf((uint32_t)(127 - ex) << 23);
    }
    w[3] = (w[3] & 0xff000000u) | e3;
    uint8_t qlo[3][8], qhi[3][8];
    std::memset(qlo, 0, sizeof(qlo));
    std::memset(qhi, 0, sizeof(qhi));
    for (int sl = 0; sl < 8; sl++) {
        if (slots[sl] == 0xffffffffu) continue;
        Box cb = ref_box_of(B, tb, slots[sl]);
        for (int a = 0; a < 3; a++) {
            float lo = std::floor(sub_dir(cb.lo[a], nb.lo[a], FE_DOWNWARD) * inv_s[a]);
            float hi = std::ceil(sub_dir(cb.hi[a], nb.lo[a], FE_UPWARD) * inv_s[a]);
            qlo[a][sl] = (uint8_t)fmin2(fmax2(lo, 0.f), 255.f);
            qhi[a][sl] = (uint8_t)fmin2(fmax2(hi, 0.f), 255.f);
        }
    }
    auto pack4 = [](const uint8_t* b) {
        return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24);
    };
    for (int a = 0; a < 3; a++) {
        w[8 + 2 * a] = pack4(qlo[a]);
        w[9 + 2 * a] = pack4(qlo[a] + 4);
        w[14 + 2 * a] = pack4(qhi[a]);
        w[15 + 2 * a] = pack4(qhi[a] + 4);
    }
}

static inline float surface(const Box& b) {
    float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    float a = dx * dy;
    a = a + dy * dz;
    a = a + dz * dx;
    return a;
}

// ---- top-down binned SAH (HY_BUILD_SAH) --------------------------------------
// Min and max run on order-preserving integer keys of the float bits (-0 below
// +0, NaNs beyond the infinities), so they are exact and independent of the
// order the GPU's atomics apply them in.
constexpr int kSahBins = 32;
static inline int32_t okey(float x) {
    const int32_t b = (int32_t)fbits(x);
    return b >= 0 ? b : b ^ 0x7fffffff;
}
static inline float unkey(int32_t k) { return bitsf((uint32_t)(k >= 0 ? k : k ^ 0x7fffffff)); }

// bin of a centroid coordinate: floor((c - lo) * (32 / extent)) clamped to
// [0, 31] (a NaN goes to bin 0)
static inline int sah_bin(float c, float lo, float scale) {
    const float v = (c - lo) * scale;
    return v >= 0.f ? (v < (float)kSahBins ? (int)v : kSahBins - 1) : 0;
}

// surface area / 2 of a box given as keys: dx dy + dy dz + dz dx
static inline float area_keys(const int32_t* lo, const int32_t* hi) {
    const float dx = unkey(hi[0]) - unkey(lo[0]), dy = unkey(hi[1]) - unkey(lo[1]),
                dz = unkey(hi[2]) - unkey(lo[2]);
    float a = dx * dy;
    a = a + dy * dz;
    a = a + dz * dx;
    return a;
}

// Binary tree over B.order (Morton sorted on entry; permuted by the stable
// partitions).  Each range [f, l] of c >= 2 items:
//   centroid bounds (keys); an axis takes part when hi - lo > 0, its scale
//   32 / (hi - lo); per axis and bin: item count and box (keys);
//   for each axis and q = 0..30: left = bins 0..q, right = bins q+1..31, both
//   non-empty, cost = (area(left) * count(left) + area(right) * count(right)) + 0;
//   the first strictly lowest finite cost in (axis, q) order wins; the items
//   with bin <= q move to the front, order kept on both sides, m = f +
//   count(left).  No candidate: m = f + c / 2, order unchanged.
// The range's node is node m - 1 (split positions are distinct, so every index
// in [0, n - 1) is used once); a one-item side is the leaf at its position.
static void sah_tree(Bvh& B, const std::vector<Box>& tb, const std::vector<float>& cen) {
    const uint32_t n = B.n;
    B.bvh2.assign(n - 1, Bvh2Node());
    struct Task { uint32_t f, l, parent, side; };
    std::vector<Task> st;
    st.push_back({0, n - 1, 0xffffffffu, 0});
    std::vector<uint32_t> tmp(n);
    while (!st.empty()) {
        const Task T = st.back();
        st.pop_back();
        const uint32_t f = T.f, l = T.l, c = l - f + 1;
        int32_t klo[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, khi[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
        for (uint32_t i = f; i <= l; i++)
            for (int a = 0; a < 3; a++) {
                const int32_t k = okey(cen[(size_t)B.order[i] * 3 + a]);
                klo[a] = std::min(klo[a], k);
                khi[a] = std::max(khi[a], k);
            }
        float clo[3], scale[3];
        bool ok[3];
        for (int a = 0; a < 3; a++) {
            clo[a] = unkey(klo[a]);
            const float ext = unkey(khi[a]) - clo[a];
            ok[a] = ext > 0.f;
            scale[a] = ok[a] ? (float)kSahBins / ext : 0.f;
        }
        uint32_t cnt[3][kSahBins] = {};
        int32_t blo[3][kSahBins][3], bhi[3][kSahBins][3];
        for (int a = 0; a < 3; a++)
            for (int q = 0; q < kSahBins; q++)
                for (int k = 0; k < 3; k++) { blo[a][q][k] = INT32_MAX; bhi[a][q][k] = INT32_MIN; }
        for (uint32_t i = f; i <= l; i++) {
            const uint32_t t = B.order[i];
            for (int a = 0; a < 3; a++) {
                if (!ok[a]) continue;
                const int q = sah_bin(cen[(size_t)t * 3 + a], clo[a], scale[a]);
                cnt[a][q]++;
                for (int k = 0; k < 3; k++) {
                    blo[a][q][k] = std::min(blo[a][q][k], okey(tb[t].lo[k]));
                    bhi[a][q][k] = std::max(bhi[a][q][k], okey(tb[t].hi[k]));
                }
            }
        }
        int best_a = -1, best_q = -1;
        uint32_t best_lc = 0;
        float best = INFINITY;
        for (int a = 0; a < 3; a++) {
            if (!ok[a]) continue;
            uint32_t rc[kSahBins];
            int32_t rlo[kSahBins][3], rhi[kSahBins][3];
            uint32_t acc = 0;
            int32_t alo[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, ahi[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
            for (int q = kSahBins - 1; q >= 0; q--) {
                acc += cnt[a][q];
                for (int k = 0; k < 3; k++) {
                    alo[k] = std::min(alo[k], blo[a][q][k]);
                    ahi[k] = std::max(ahi[k], bhi[a][q][k]);
                    rlo[q][k] = alo[k];
                    rhi[q][k] = ahi[k];
                }
                rc[q] = acc;
            }
            uint32_t lc = 0;
            int32_t llo[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, lhi[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
            for (int q = 0; q + 1 < kSahBins; q++) {
                lc += cnt[a][q];
                for (int k = 0; k < 3; k++) {
                    llo[k] = std::min(llo[k], blo[a][q][k]);
                    lhi[k] = std::max(lhi[k], bhi[a][q][k]);
                }
                const uint32_t r = rc[q + 1];
                if (lc == 0 || r == 0) continue;
                const float t1 = area_keys(llo, lhi) * (float)lc;
                const float t2 = area_keys(rlo[q + 1], rhi[q + 1]) * (float)r;
                const float cost = (t1 + t2) + 0.f;
                if (cost < best) { best = cost; best_a = a; best_q = q; best_lc = lc; }
            }
        }
        uint32_t m;
        if (best_a >= 0) {
            uint32_t nl = 0, nr = 0;
            m = f + best_lc;
            for (uint32_t i = f; i <= l; i++) {
                const uint32_t t = B.order[i];
                if (sah_bin(cen[(size_t)t * 3 + best_a], clo[best_a], scale[best_a]) <= best_q) tmp[f + nl++] = t;
                else tmp[m + nr++] = t;
            }
            std::copy(tmp.begin() + f, tmp.begin() + l + 1, B.order.begin() + f);
        } else {
            m = f + c / 2;
        }
        const uint32_t id = m - 1;
        Bvh2Node& nd = B.bvh2[id];
        nd.first = f;
        nd.last = l;
        if (T.parent == 0xffffffffu) B.root = id;
        else if (T.side) B.bvh2[T.parent].right = id;
        else B.bvh2[T.parent].left = id;
        if (m - f == 1) nd.left = kLeafBit | f;
        else st.push_back({f, m - 1, id, 0});
        if (l - m + 1 == 1) nd.right = kLeafBit | m;
        else st.push_back({m, l, id, 1});
    }
}

// LBVH -> BVH8 over n items of three points each (9 floats: a triangle, or an
// instance box as (lo, hi, hi)); an item's box is the min/max of its points.
// Records hold the item's points and its index; node and record numbers in the
// emitted nodes are offset by node_off / rec_off (BLASes and the TLAS of the
// two-level structure share one node array and one record array).
static void build_core(const float* items, uint32_t n, Bvh& B, uint32_t node_off, uint32_t rec_off, uint32_t mode) {
    B = Bvh();
    B.n = n;
    if (n == 0) return;
    std::vector<Box> tb(n);
    std::vector<float> cen((size_t)n * 3);
    for (int a = 0; a < 3; a++) { B.slo[a] = INFINITY; B.shi[a] = -INFINITY; }
    for (uint32_t t = 0; t < n; t++) {
        const float* w = &items[(size_t)t * 9];
        for (int a = 0; a < 3; a++) {
            tb[t].lo[a] = fmin2(fmin2(w[a], w[3 + a]), w[6 + a]);
            tb[t].hi[a] = fmax2(fmax2(w[a], w[3 + a]), w[6 + a]);
            float c = (tb[t].lo[a] + tb[t].hi[a]) * 0.5f;
            cen[(size_t)t * 3 + a] = c;
            B.slo[a] = fmin2(B.slo[a], c);
            B.shi[a] = fmax2(B.shi[a], c);
        }
    }
    float inv[3];
    for (int a = 0; a < 3; a++) {
        float ext = B.shi[a] - B.slo[a];
        inv[a] = ext > 0.f ? 1024.0f / ext : 0.f;
    }
    std::vector<uint32_t> code(n);
    for (uint32_t t = 0; t < n; t++) {
        uint32_t q[3];
        for (int a = 0; a < 3; a++) {
            float v = (cen[(size_t)t * 3 + a] - B.slo[a]) * inv[a];
            v = fmin2(fmax2(v, 0.f), 1023.f);
            q[a] = (uint32_t)v;
        }
        code[t] = (expand10(q[0]) << 2) | (expand10(q[1]) << 1) | expand10(q[2]);
    }
    B.order.resize(n);
    std::iota(B.order.begin(), B.order.end(), 0u);
    std::stable_sort(B.order.begin(), B.order.end(), [&](uint32_t a, uint32_t b) { return code[a] < code[b]; });
    B.morton.resize(n);
    std::vector<uint64_t> key(n);
    for (uint32_t i = 0; i < n; i++) {
        B.morton[i] = code[B.order[i]];
        key[i] = ((uint64_t)B.morton[i] << 32) | B.order[i];
    }
    if (mode == HY_BUILD_SAH) {
        B.root = n > 1 ? 0u : kLeafBit;
        if (n > 1) {
            sah_tree(B, tb, cen);
            refit_bvh2(B, tb);
        }
        for (uint32_t i = 0; i < n; i++) B.morton[i] = code[B.order[i]];
    }
    // ---- Karras 2012 ----
    auto delta = [&](int64_t i, int64_t j) -> int {
        if (j < 0 || j >= (int64_t)n) return -1;
        return clz64(key[i] ^ key[j]);
    };
    if (mode == HY_BUILD_LBVH && n > 1) {
        B.root = 0;
        B.bvh2.resize(n - 1);
        for (int64_t i = 0; i < (int64_t)n - 1; i++) {
            int d = (delta(i, i + 1) - delta(i, i - 1)) >= 0 ? 1 : -1;
            int dmin = delta(i, i - d);
            int64_t lmax = 2;
            while (delta(i, i + lmax * d) > dmin) lmax *= 2;
            int64_t l = 0;
            for (int64_t t = lmax / 2; t >= 1; t /= 2)
                if (delta(i, i + (l + t) * d) > dmin) l += t;
            int64_t j = i + l * d;
            int dnode = delta(i, j);
            int64_t sp = 0;
            for (int64_t div = 2;; div *= 2) {
                int64_t t = (l + div - 1) / div;
                if (delta(i, i + (sp + t) * d) > dnode) sp += t;
                if (t == 1) break;
            }
            int64_t gamma = i + sp * d + std::min(d, 0);
            int64_t lo = std::min(i, j), hi = std::max(i, j);
            Bvh2Node& nd = B.bvh2[i];
            nd.left = (lo == gamma) ? (kLeafBit | (uint32_t)gamma) : (uint32_t)gamma;
            nd.right = (hi == gamma + 1) ? (kLeafBit | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
            nd.first = (uint32_t)lo;
            nd.last = (uint32_t)hi;
        }
        refit_bvh2(B, tb);
    }
    auto ref_box = [&](uint32_t r) -> Box {
        if (r & kLeafBit) return tb[B.order[r & ~kLeafBit]];
        Box b;
        for (int a = 0; a < 3; a++) { b.lo[a] = B.bvh2[r].lo[a]; b.hi[a] = B.bvh2[r].hi[a]; }
        return b;
    };
    auto ref_count = [&](uint32_t r) -> uint32_t {
        if (r & kLeafBit) return 1;
        return B.bvh2[r].last - B.bvh2[r].first + 1;
    };
    auto ref_first = [&](uint32_t r) -> uint32_t {
        if (r & kLeafBit) return r & ~kLeafBit;
        return B.bvh2[r].first;
    };
    // ---- slot budgets of the collapse (surface area heuristic) ----
    // f(n, i): the lowest cost of representing subtree n by at most i slots of
    // its parent, a slot being a leaf of <= kLeafMax triangles (area x triangles
    // x kCostTri) or an internal node (area x kCostNode + its own 8 slots); a
    // one-triangle leaf costs area x kCostTri.  Split choices: how many of the
    // i slots go to the left child, or 0 for "f(n, i - 1)"; a node's own 8 slots
    // (k to the left, 8 - k to the right) at [n * 9].  Float ops in the written
    // order; the first strict minimum in k order wins.
    std::vector<float> dpf;
    std::vector<uint8_t> dpk;
    if (n > 1) {
        dpf.assign((size_t)(n - 1) * 8, 0.f);
        dpk.assign((size_t)(n - 1) * 9, 0);
        auto f = [&](uint32_t m, int i) -> float {
            if (m & kLeafBit) return surface(tb[B.order[m & ~kLeafBit]]) * kCostTri;
            return dpf[(size_t)m * 8 + i - 1];
        };
        std::vector<uint32_t> st{B.root};
        std::vector<uint8_t> done(n - 1, 0);
        while (!st.empty()) {
            const uint32_t m = st.back();
            bool ready = true;
            for (uint32_t c : {B.bvh2[m].left, B.bvh2[m].right})
                if (!(c & kLeafBit) && !done[c]) { st.push_back(c); ready = false; }
            if (!ready) continue;
            st.pop_back();
            const uint32_t L = B.bvh2[m].left, R = B.bvh2[m].right;
            const float A = surface(ref_box(m));
            const uint32_t cnt = B.bvh2[m].last - B.bvh2[m].first + 1;
            float best8 = INFINITY;
            int bk = 1;
            for (int k = 1; k <= 7; k++) {
                const float v = f(L, k) + f(R, 8 - k);
                if (v < best8) { best8 = v; bk = k; }
            }
            dpk[(size_t)m * 9] = (uint8_t)bk;
            dpf[(size_t)m * 8] = cnt <= (uint32_t)kLeafMax ? (A * (float)cnt) * kCostTri : A * kCostNode + best8;
            for (int i = 2; i <= 8; i++) {
                float v = dpf[(size_t)m * 8 + i - 2];
                int kk = 0;
                for (int k = 1; k < i; k++) {
                    const float w = f(L, k) + f(R, i - k);
                    if (w < v) { v = w; kk = k; }
                }
                dpf[(size_t)m * 8 + i - 1] = v;
                dpk[(size_t)m * 9 + i] = (uint8_t)kk;
            }
            done[m] = 1;
        }
    }
    // ---- BFS collapse to BVH8 ----
    std::vector<uint32_t> queue;       // BVH2 ref of each BVH8 node, BFS order
    std::vector<uint32_t> level;       // level of each node
    queue.push_back(n > 1 ? B.root : (kLeafBit | 0u));
    level.push_back(0);
    uint32_t tri_count = 0;
    B.tris.assign((size_t)n * 12, 0.f);
    for (size_t k = 0; k < queue.size(); k++) {
        uint32_t r = queue[k];
        // children list
        // children: the node's 8 slots spread over its subtree by the budget
        // choices, left subtree first
        uint32_t C[8];
        int nc = 0;
        if (r & kLeafBit) {
            C[nc++] = r;
        } else {
            uint32_t sm_[8];
            int si_[8], sp = 0;
            const int k0 = dpk[(size_t)r * 9];
            sm_[sp] = B.bvh2[r].right; si_[sp++] = 8 - k0;
            sm_[sp] = B.bvh2[r].left; si_[sp++] = k0;
            while (sp > 0) {
                const uint32_t m = sm_[--sp];
                int i = si_[sp];
                while (!(m & kLeafBit) && i > 1 && dpk[(size_t)m * 9 + i] == 0) i--;
                if ((m & kLeafBit) || i == 1) { C[nc++] = m; continue; }
                const int k = dpk[(size_t)m * 9 + i];
                sm_[sp] = B.bvh2[m].right; si_[sp++] = i - k;
                sm_[sp] = B.bvh2[m].left; si_[sp++] = k;
            }
        }
        // slot assignment
        Box nb = ref_box(r);
        float pc[3];
        for (int a = 0; a < 3; a++) pc[a] = (nb.lo[a] + nb.hi[a]) * 0.5f;
        float cost[8][8];
        for (int i = 0; i < nc; i++) {
            Box cb = ref_box(C[i]);
            float dd[3];
            for (int a = 0; a < 3; a++) dd[a] = (cb.lo[a] + cb.hi[a]) * 0.5f - pc[a];
            for (int sl = 0; sl < 8; sl++) {
                float c0 = (sl & 1) ? dd[0] : -dd[0];
                float c1 = (sl & 2) ? dd[1] : -dd[1];
                float c2 = (sl & 4) ? dd[2] : -dd[2];
                cost[i][sl] = (c0 + c1) + c2;
            }
        }
        int slot_of[8];
        int child_in_slot[8];
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
        // encode
        Bvh8Node node;
        std::memset(&node, 0, sizeof(node));
        uint32_t slots[8];
        for (int sl = 0; sl < 8; sl++) slots[sl] = child_in_slot[sl] < 0 ? 0xffffffffu : C[child_in_slot[sl]];
        B.node_ref.push_back(r);
        B.node_plan.insert(B.node_plan.end(), slots, slots + 8);
        uint32_t imask = 0;
        uint8_t meta[8] = {0};
        uint32_t child_base = (uint32_t)queue.size();
        uint32_t tri_base = tri_count;
        uint32_t toff = 0;
        for (int sl = 0; sl < 8; sl++) {
            int i = child_in_slot[sl];
            if (i < 0) continue;
            uint32_t c = C[i];
            uint32_t cnt = ref_count(c);
            if (cnt > (uint32_t)kLeafMax) {
                imask |= 1u << sl;
                meta[sl] = 0x80;
                queue.push_back(c);
                level.push_back(level[k] + 1);
            } else {
                meta[sl] = (uint8_t)((cnt << 5) | toff);
                uint32_t f = ref_first(c);
                for (uint32_t j = 0; j < cnt; j++) {
                    uint32_t tid = B.order[f + j];
                    float* dst = &B.tris[(size_t)(tri_count + toff + j) * 12];
                    const float* w = &items[(size_t)tid * 9];
                    dst[0] = w[0]; dst[1] = w[1]; dst[2] = w[2]; dst[3] = bitsf(tid);
                    dst[4] = w[3]; dst[5] = w[4]; dst[6] = w[5]; dst[7] = 0.f;
                    dst[8] = w[6]; dst[9] = w[7]; dst[10] = w[8]; dst[11] = 0.f;
                }
                toff += cnt;
            }
        }
        tri_count += toff;
        node.w[3] = imask << 24;
        quantize_node(B, tb, r, slots, node.w);
        node.w[4] = node_off + child_base;
        node.w[5] = rec_off + tri_base;
        auto pack4 = [](const uint8_t* b) { return (uint32_t)b[0] | ((uint32_t)b[1] << 8) | ((uint32_t)b[2] << 16) | ((uint32_t)b[3] << 24); };
        node.w[6] = pack4(meta); node.w[7] = pack4(meta + 4);
        B.bvh8.push_back(node);
    }
    (void)ref_box;
    B.depth = level.empty() ? 0 : level.back() + 1;
}

void bvh_build(Scene& s) {
    s.two_level = false;
    s.two = Bvh2L();
    build_core(s.world.data(), s.ntri, s.bvh, 0, 0, s.build_mode);
    s.bvh_ok = s.ntri > 0;
}

// New transforms, same topology: re-transformed triangles, refitted binary
// tree, every 8-wide node re-quantised with its stored slot plan, packed
// triangles rewritten (the GPU refit computes exactly this).
static void tlas_build(Scene& s);

void bvh_refit(Scene& s) {
    Bvh& B = s.bvh;
    if (!s.bvh_ok) return;
    if (s.two_level) { tlas_build(s); return; }
    std::vector<Box> tb = tri_boxes(s);
    refit_bvh2(B, tb);
    for (size_t k = 0; k < B.bvh8.size(); k++) quantize_node(B, tb, B.node_ref[k], &B.node_plan[k * 8], B.bvh8[k].w);
    for (uint32_t i = 0; i < B.n; i++) {
        float* dst = &B.tris[(size_t)i * 12];
        const uint32_t tid = fbits(dst[3]);
        const float* w = &s.world[(size_t)tid * 9];
        dst[0] = w[0]; dst[1] = w[1]; dst[2] = w[2];
        dst[4] = w[3]; dst[5] = w[4]; dst[6] = w[5];
        dst[8] = w[6]; dst[9] = w[7]; dst[10] = w[8];
    }
}

// ---- watertight ray/triangle test (Woop, Benthin & Wald, JCGT 2013) -----------
struct RayPre {
    float o[3], d[3];
    int kx, ky, kz;
    float Sx, Sy, Sz;
};

static RayPre ray_pre(const float o[3], const float d[3]) {
    RayPre r;
    for (int a = 0; a < 3; a++) { r.o[a] = o[a]; r.d[a] = d[a]; }
    float ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
    r.kz = (ax > ay) ? ((ax > az) ? 0 : 2) : ((ay > az) ? 1 : 2);
    r.kx = r.kz + 1; if (r.kx == 3) r.kx = 0;
    r.ky = r.kx + 1; if (r.ky == 3) r.ky = 0;
    if (d[r.kz] < 0.f) std::swap(r.kx, r.ky);
    r.Sx = d[r.kx] / d[r.kz];
    r.Sy = d[r.ky] / d[r.kz];
    r.Sz = 1.0f / d[r.kz];
    return r;
}

// returns true and t/b1/b2 when the triangle is hit with tmin <= t <= tmax
static bool tri_test(const RayPre& r, const float* v0, const float* v1, const float* v2, float tmin, float tmax,
                     float& t, float& b1, float& b2) {
    float A[3], Bv[3], Cv[3];
    for (int a = 0; a < 3; a++) { A[a] = v0[a] - r.o[a]; Bv[a] = v1[a] - r.o[a]; Cv[a] = v2[a] - r.o[a]; }
    float Ax = A[r.kx] - r.Sx * A[r.kz], Ay = A[r.ky] - r.Sy * A[r.kz];
    float Bx = Bv[r.kx] - r.Sx * Bv[r.kz], By = Bv[r.ky] - r.Sy * Bv[r.kz];
    float Cx = Cv[r.kx] - r.Sx * Cv[r.kz], Cy = Cv[r.ky] - r.Sy * Cv[r.kz];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.f || V == 0.f || W == 0.f) {
        double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
        U = (float)(CxBy - CyBx);
        double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
        V = (float)(AxCy - AyCx);
        double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
        W = (float)(BxAy - ByAx);
    }
    if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
    float det = U + V;
    det = det + W;
    if (det == 0.f) return false;
    float Az = r.Sz * A[r.kz], Bz = r.Sz * Bv[r.kz], Cz = r.Sz * Cv[r.kz];
    float T = U * Az;
    T = T + V * Bz;
    T = T + W * Cz;
    float tt = T / det;
    if (!(tt >= tmin && tt <= tmax)) return false;
    t = tt;
    b1 = V / det;
    b2 = W / det;
    return true;
}

static inline bool better(float t, uint32_t id, const Hit& h) {
    return t < h.t || (t == h.t && id < h.id);
}

static Hit trace_brute(const Scene& s, const float o[3], const float d[3], float tmin, float tmax, bool any_hit,
                       Counters* c) {
    Hit h{tmax, HY_NO_HIT, 0.f, 0.f};
    RayPre r = ray_pre(o, d);
    for (uint32_t t = 0; t < s.ntri; t++) {
        const float* w = &s.world[(size_t)t * 9];
        float tt, b1, b2;
        if (c) c->tris++;
        if (tri_test(r, w, w + 3, w + 6, tmin, h.id == HY_NO_HIT ? tmax : h.t, tt, b1, b2)) {
            if (h.id == HY_NO_HIT || better(tt, t, h)) h = Hit{tt, t, b1, b2};
            if (any_hit) return h;
        }
    }
    return h;
}

static inline uint8_t byte_of(const uint32_t* w, int word0, int slot) {
    return (uint8_t)(w[word0 + (slot >> 2)] >> ((slot & 3) * 8));
}

// Plane distances of both walks, as the kernels compute them: plane
// byte q as q * 2^-24 (the kernels convert it from a subnormal half, exactly)
// times the node scale over d scaled by 2^24, plus org, in one fma: q * adj +
// org rounded once, the value fma(q, adj, org) gives (unless adj * 2^24
// overflows, which both sides then share).
static const struct PlaneValues24 {
    float v[256];
    PlaneValues24() { for (int q = 0; q < 256; q++) v[q] = (float)q * 5.9604644775390625e-8f; }
} kPlane24;

static Hit trace_bvh8(const Scene& s, const float o[3], const float d[3], float tmin, float tmax, bool any_hit,
                      Counters* c) {
    const Bvh& B = s.bvh;
    Hit h{tmax, HY_NO_HIT, 0.f, 0.f};
    RayPre r = ray_pre(o, d);
    float invd[3];
    for (int a = 0; a < 3; a++) {
        float dd = std::fabs(d[a]) > 1e-20f ? d[a] : std::copysign(1e-20f, d[a]);
        invd[a] = 1.0f / dd;
    }
    uint32_t near = (invd[0] < 0.f ? 1u : 0u) | (invd[1] < 0.f ? 2u : 0u) | (invd[2] < 0.f ? 4u : 0u);
    // child rank = slot ^ ord: front to back for closest hits; any-hit rays
    // in the scene's order (anyhit_flip)
    const uint32_t ord = any_hit ? near ^ anyhit_flip(s) : near;
    uint32_t stk_base[kStackMax], stk_bits[kStackMax];
    int sp = 0;
    uint32_t g_base = 0, g_bits = 1u << 24;  // one rank bit, empty slot mask: the root alone
    float cur_tmax = tmax;
    for (uint32_t iter = 0;; iter++) {
        if (iter >= kMaxIters) { if (c) c->status |= HY_STATUS_TIMEOUT; break; }
        if ((g_bits & 0xff000000u) == 0) {
            if (sp == 0) break;
            --sp;
            g_base = stk_base[sp];
            g_bits = stk_bits[sp];
        }
        uint32_t rb = (uint32_t)__builtin_ctz(g_bits >> 24);
        g_bits &= ~(1u << (24 + rb));
        uint32_t sl = rb ^ ord;
        uint32_t idx = g_base + (uint32_t)__builtin_popcount(g_bits & 0xffu & ((1u << sl) - 1u));
        if (g_bits & 0xff000000u) {
            if (sp >= kStackMax) { if (c) c->status |= HY_STATUS_STACK_OVERFLOW; break; }
            stk_base[sp] = g_base;
            stk_bits[sp] = g_bits;
            sp++;
        }
        const uint32_t* w = B.bvh8[idx].w;
        if (c) c->nodes++;
        float adj24[3], org[3];
        for (int a = 0; a < 3; a++) {
            uint32_t ea = (w[3] >> (8 * a)) & 0xffu;
            float sc = bitsf(ea << 23);
            adj24[a] = (sc * invd[a]) * 16777216.0f;
            org[a] = (bitsf(w[a]) - o[a]) * invd[a];
        }
        uint32_t imask = w[3] >> 24;
        uint32_t hit_int = 0, hit_tri = 0;
        for (int slot = 0; slot < 8; slot++) {
            uint8_t m = byte_of(w, 6, slot);
            if (m == 0) continue;
            float tn[3], tf[3];
            for (int a = 0; a < 3; a++) {
                float ql = kPlane24.v[byte_of(w, 8 + 2 * a, slot)];
                float qh = kPlane24.v[byte_of(w, 14 + 2 * a, slot)];
                float lo = invd[a] < 0.f ? qh : ql;
                float hi = invd[a] < 0.f ? ql : qh;
                tn[a] = std::fma(lo, adj24[a], org[a]);
                tf[a] = std::fma(hi, adj24[a], org[a]);
            }
            float tnear = fmax2(fmax2(tn[0], tn[1]), fmax2(tn[2], tmin));
            float tfar = fmin2(fmin2(tf[0], tf[1]), fmin2(tf[2], cur_tmax));
            if (!(tnear <= tfar * 1.0000003f)) continue;
            if (imask & (1u << slot)) hit_int |= 1u << (slot ^ ord);
            else hit_tri |= ((1u << (m >> 5)) - 1u) << (m & 31u);
        }
        uint32_t tri_base = w[5];
        while (hit_tri) {
            uint32_t b = (uint32_t)__builtin_ctz(hit_tri);
            hit_tri &= hit_tri - 1u;
            const float* tr = &B.tris[(size_t)(tri_base + b) * 12];
            uint32_t id = fbits(tr[3]);
            if (c) c->tris++;
            float tt, b1, b2;
            if (tri_test(r, tr, tr + 4, tr + 8, tmin, cur_tmax, tt, b1, b2)) {
                if (h.id == HY_NO_HIT || better(tt, id, h)) { h = Hit{tt, id, b1, b2}; cur_tmax = tt; }
                if (any_hit) return h;
            }
        }
        g_base = w[4];
        g_bits = (hit_int << 24) | imask;
    }
    return h;
}

// ---- two-level structure ------------------------------------------------------

static inline float round_down_f(double x) {
    float f = (float)x;
    return ((double)f > x) ? std::nextafter(f, -INFINITY) : f;
}
static inline float round_up_f(double x) {
    float f = (float)x;
    return ((double)f < x) ? std::nextafter(f, INFINITY) : f;
}

// World box of an instance: the vertices of its mesh's vertex range (from the
// smallest to the largest vertex its triangles use) through the
// object->world matrix M (column-major) in double, each coordinate
// ((m0 x + m1 y) + m2 z) + m3; min / max, then padded by 2^-16 of the extent
// plus 2^-20 of the largest magnitude plus 2^-60 per axis (room for the
// rounding of the world->object ray transform; the last term also makes the
// result independent of the sign of a zero) and rounded outwards to float.
static void instance_box(const Scene& s, uint32_t v0, uint32_t v1, const float* M, float* out6) {
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t v = v0; v < v1; v++) {
        const float* P = s.verts[v].pos;
        for (int r = 0; r < 3; r++) {
            double w = (double)M[0 * 4 + r] * (double)P[0];
            w = w + (double)M[1 * 4 + r] * (double)P[1];
            w = w + (double)M[2 * 4 + r] * (double)P[2];
            w = w + (double)M[3 * 4 + r];
            lo[r] = std::fmin(lo[r], w);
            hi[r] = std::fmax(hi[r], w);
        }
    }
    for (int a = 0; a < 3; a++) {
        const double mag = std::fmax(std::fabs(lo[a]), std::fabs(hi[a]));
        const double pad = ((hi[a] - lo[a]) * 0x1p-16 + mag * 0x1p-20) + 0x1p-60;
        out6[a] = round_down_f(lo[a] - pad);
        out6[3 + a] = round_up_f(hi[a] + pad);
    }
}

// world->object rows of every transform: rows of inverse(M) rounded to float
static void derive_xinv(Scene& s) {
    const size_t nx = s.xf.size() / 16;
    s.two.xinv.assign(nx * 12, 0.f);
    for (size_t t = 0; t < nx; t++) {
        double m[16], inv[16];
        for (int i = 0; i < 16; i++) m[i] = s.xf[t * 16 + i];
        inverse4(m, inv);
        for (int r = 0; r < 3; r++)
            for (int k = 0; k < 4; k++) s.two.xinv[t * 12 + r * 4 + k] = (float)inv[k * 4 + r];
    }
}

// instance records and TLAS (the per-frame part: transforms only)
static void tlas_build(Scene& s) {
    Bvh2L& T = s.two;
    derive_xinv(s);
    T.inst.assign((size_t)T.ninst * 16, 0.f);
    T.inst_box.assign((size_t)T.ninst * 6, 0.f);
    std::vector<float> items((size_t)T.ninst * 9);
    for (uint32_t i = 0; i < T.ninst; i++) {
        const uint32_t p = T.inst_prim[i], m = T.prim_mesh[p];
        const uint32_t tf = s.prims[p].transform_id;
        float* I = &T.inst[(size_t)i * 16];
        for (int k = 0; k < 12; k++) I[k] = T.xinv[(size_t)tf * 12 + k];
        I[12] = bitsf(T.blas_node0[m]);
        I[13] = bitsf(s.prim_tri0[p]);
        I[14] = bitsf(p);
        float* b = &T.inst_box[(size_t)i * 6];
        instance_box(s, T.mesh_vrange[2 * m], T.mesh_vrange[2 * m + 1], &s.xf[(size_t)tf * 16], b);
        float* it = &items[(size_t)i * 9];
        for (int a = 0; a < 3; a++) { it[a] = b[a]; it[3 + a] = b[3 + a]; it[6 + a] = b[3 + a]; }
    }
    Bvh tl;
    build_core(items.data(), T.ninst, tl, 0, 0, s.build_mode);
    T.tlas_nodes = (uint32_t)tl.bvh8.size();
    T.tlas_depth = tl.depth;
    for (uint32_t k = 0; k < T.tlas_region; k++) std::memset(T.nodes[k].w, 0, 80);
    for (uint32_t k = 0; k < T.tlas_nodes; k++) T.nodes[k] = tl.bvh8[k];
    std::fill(T.tris.begin(), T.tris.begin() + (size_t)T.tlas_region * 12, 0.f);
    std::copy(tl.tris.begin(), tl.tris.end(), T.tris.begin());
}

void bvh_build_instanced(Scene& s) {
    s.bvh = Bvh();
    s.bvh_ok = false;
    s.two_level = false;
    Bvh2L& T = s.two;
    T = Bvh2L();
    const uint32_t np = (uint32_t)s.prims.size();
    T.prim_mesh.assign(np, 0xffffffffu);
    for (uint32_t p = 0; p < np; p++) {
        const HyPrimitive& pr = s.prims[p];
        if (pr.index_count / 3 == 0) continue;
        uint32_t m = 0;
        for (; m < T.nblas; m++) {
            const HyPrimitive& q = s.prims[T.mesh_prim[m]];
            if (q.first_index == pr.first_index && q.index_count == pr.index_count &&
                q.vertex_offset == pr.vertex_offset)
                break;
        }
        if (m == T.nblas) { T.mesh_prim.push_back(p); T.nblas++; }
        T.prim_mesh[p] = m;
        T.inst_prim.push_back(p);
    }
    T.ninst = (uint32_t)T.inst_prim.size();
    if (T.ninst == 0) return;
    T.tlas_region = T.ninst;
    T.nodes.assign(T.tlas_region, Bvh8Node{});
    T.tris.assign((size_t)T.tlas_region * 12, 0.f);
    T.mesh_vrange.assign((size_t)T.nblas * 2, 0u);
    uint32_t rec = T.tlas_region;
    for (uint32_t m = 0; m < T.nblas; m++) {
        const HyPrimitive& pr = s.prims[T.mesh_prim[m]];
        const uint32_t nt = pr.index_count / 3;
        std::vector<float> items((size_t)nt * 9);
        for (uint32_t k = 0; k < nt; k++)
            for (int v = 0; v < 3; v++) {
                const float* P = s.verts[s.idx[pr.first_index + 3 * k + v] + pr.vertex_offset].pos;
                for (int a = 0; a < 3; a++) items[(size_t)k * 9 + v * 3 + a] = P[a] + 0.0f;  // -0 -> +0
            }
        const uint32_t node0 = (uint32_t)T.nodes.size();
        Bvh b;
        build_core(items.data(), nt, b, node0, rec, s.build_mode);
        T.blas_node0.push_back(node0);
        T.blas_rec0.push_back(rec);
        T.blas_nodes.push_back((uint32_t)b.bvh8.size());
        T.nodes.insert(T.nodes.end(), b.bvh8.begin(), b.bvh8.end());
        T.tris.insert(T.tris.end(), b.tris.begin(), b.tris.end());
        T.blas_depth = std::max(T.blas_depth, b.depth);
        // vertex range the mesh's triangles use
        uint32_t vmin = 0xffffffffu, vmax = 0;
        for (uint32_t k = 0; k < nt * 3; k++) {
            vmin = std::min(vmin, s.idx[pr.first_index + k]);
            vmax = std::max(vmax, s.idx[pr.first_index + k]);
        }
        T.mesh_vrange[2 * m] = pr.vertex_offset + vmin;
        T.mesh_vrange[2 * m + 1] = pr.vertex_offset + vmax + 1;
        rec += nt;
    }
    tlas_build(s);
    s.two_level = true;
    s.bvh_ok = true;
}

struct RayState {
    RayPre p;
    float invd[3];
    uint32_t near;
};

static RayState ray_state(const float o[3], const float d[3]) {
    RayState r;
    r.p = ray_pre(o, d);
    for (int a = 0; a < 3; a++) {
        float dd = std::fabs(d[a]) > 1e-20f ? d[a] : std::copysign(1e-20f, d[a]);
        r.invd[a] = 1.0f / dd;
    }
    r.near = (r.invd[0] < 0.f ? 1u : 0u) | (r.invd[1] < 0.f ? 2u : 0u) | (r.invd[2] < 0.f ? 4u : 0u);
    return r;
}

// box tests of one node: internal children hit (rank order) and leaf records
// hit (plane distances as in trace_bvh8)
static void node_hits(const uint32_t* w, const RayState& r, uint32_t ord, float tmin, float tmax,
                      uint32_t& hit_int, uint32_t& hit_tri) {
    float adj24[3], org[3];
    for (int a = 0; a < 3; a++) {
        uint32_t ea = (w[3] >> (8 * a)) & 0xffu;
        adj24[a] = (bitsf(ea << 23) * r.invd[a]) * 16777216.0f;
        org[a] = (bitsf(w[a]) - r.p.o[a]) * r.invd[a];
    }
    const uint32_t imask = w[3] >> 24;
    hit_int = 0;
    hit_tri = 0;
    for (int slot = 0; slot < 8; slot++) {
        uint8_t m = byte_of(w, 6, slot);
        if (m == 0) continue;
        float tn[3], tf[3];
        for (int a = 0; a < 3; a++) {
            float ql = kPlane24.v[byte_of(w, 8 + 2 * a, slot)];
            float qh = kPlane24.v[byte_of(w, 14 + 2 * a, slot)];
            float lo = r.invd[a] < 0.f ? qh : ql;
            float hi = r.invd[a] < 0.f ? ql : qh;
            tn[a] = std::fma(lo, adj24[a], org[a]);
            tf[a] = std::fma(hi, adj24[a], org[a]);
        }
        float tnear = fmax2(fmax2(tn[0], tn[1]), fmax2(tn[2], tmin));
        float tfar = fmin2(fmin2(tf[0], tf[1]), fmin2(tf[2], tmax));
        if (!(tnear <= tfar * 1.0000003f)) continue;
        if (imask & (1u << slot)) hit_int |= 1u << (slot ^ ord);
        else hit_tri |= ((1u << (m >> 5)) - 1u) << (m & 31u);
    }
}

// Two-level walk, step for step the product's: a TLAS leaf hands its hit
// instance entries over one at a time; entering one saves the pending TLAS
// group on the stack, moves the ray into object space
// (((r0 x + r1 y) + r2 z) + t per row; the direction without t) and walks
// the BLAS above the saved stack height; leaving it restores the world ray.
// Hit ids are global triangle ids (the instance's first triangle + the
// record's index in its mesh); t is shared by both levels (the direction is
// not renormalised).
static Hit trace_2l(const Scene& s, const float o[3], const float d[3], float tmin, float tmax, bool any_hit,
                    Counters* c) {
    const Bvh2L& T = s.two;
    Hit h{tmax, HY_NO_HIT, 0.f, 0.f};
    const RayState rw = ray_state(o, d);
    RayState r = rw;
    uint32_t stk_base[kStackMax], stk_bits[kStackMax];
    int sp = 0, sp_base = 0;
    bool level = false;
    uint32_t inst_base = 0, inst_bits = 0, id_off = 0;
    uint32_t g_base = 0, g_bits = 1u << 24;
    const uint32_t flip = any_hit ? anyhit_flip(s) : 0u;  // rank order as in trace_bvh8
    float cur_tmax = tmax;
    const uint32_t nrec = (uint32_t)(T.tris.size() / 12), nnodes = (uint32_t)T.nodes.size();
    for (uint32_t iter = 0;; iter++) {
        if (iter >= kMaxIters) { if (c) c->status |= HY_STATUS_TIMEOUT; break; }
        bool done = false;
        for (;;) {
            if (!level && inst_bits) {
                if (g_bits & 0xff000000u) {
                    if (sp >= kStackMax) { if (c) c->status |= HY_STATUS_STACK_OVERFLOW; done = true; break; }
                    stk_base[sp] = g_base;
                    stk_bits[sp] = g_bits;
                    sp++;
                }
                const uint32_t b = (uint32_t)__builtin_ctz(inst_bits);
                inst_bits &= inst_bits - 1u;
                const uint32_t rec = inst_base + b;
                if (rec >= nrec) { if (c) c->status |= HY_STATUS_BAD_INDEX; done = true; break; }
                const uint32_t iid = fbits(T.tris[(size_t)rec * 12 + 3]);
                if (iid >= T.ninst) { if (c) c->status |= HY_STATUS_BAD_INDEX; done = true; break; }
                const float* I = &T.inst[(size_t)iid * 16];
                float oo[3], dd[3];
                for (int k = 0; k < 3; k++) {
                    const float* R = I + 4 * k;
                    float a = R[0] * rw.p.o[0];
                    a = a + R[1] * rw.p.o[1];
                    a = a + R[2] * rw.p.o[2];
                    oo[k] = a + R[3];
                    float e = R[0] * rw.p.d[0];
                    e = e + R[1] * rw.p.d[1];
                    dd[k] = e + R[2] * rw.p.d[2];
                }
                r = ray_state(oo, dd);
                level = true;
                sp_base = sp;
                id_off = fbits(I[13]);
                g_base = fbits(I[12]);
                g_bits = 1u << 24;
                break;
            }
            if (g_bits & 0xff000000u) break;
            if (level && sp == sp_base) { level = false; r = rw; continue; }
            if (sp == 0) { done = true; break; }
            --sp;
            g_base = stk_base[sp];
            g_bits = stk_bits[sp];
        }
        if (done) break;
        const uint32_t rb = (uint32_t)__builtin_ctz(g_bits >> 24);
        g_bits &= ~(1u << (24 + rb));
        const uint32_t sl = rb ^ r.near ^ flip;
        const uint32_t idx = g_base + (uint32_t)__builtin_popcount(g_bits & 0xffu & ((1u << sl) - 1u));
        if (g_bits & 0xff000000u) {
            if (sp >= kStackMax) { if (c) c->status |= HY_STATUS_STACK_OVERFLOW; break; }
            stk_base[sp] = g_base;
            stk_bits[sp] = g_bits;
            sp++;
        }
        if (idx >= nnodes) { if (c) c->status |= HY_STATUS_BAD_INDEX; break; }
        const uint32_t* w = T.nodes[idx].w;
        if (c) c->nodes++;
        uint32_t hit_int, hit_tri;
        node_hits(w, r, r.near ^ flip, tmin, cur_tmax, hit_int, hit_tri);
        const uint32_t tri_base = w[5];
        if (!level) {
            inst_base = tri_base;
            inst_bits = hit_tri;
        } else {
            while (hit_tri) {
                uint32_t b = (uint32_t)__builtin_ctz(hit_tri);
                hit_tri &= hit_tri - 1u;
                if (tri_base + b >= nrec) { if (c) c->status |= HY_STATUS_BAD_INDEX; return h; }
                const float* tr = &T.tris[(size_t)(tri_base + b) * 12];
                const uint32_t id = id_off + fbits(tr[3]);
                if (c) c->tris++;
                float tt, b1, b2;
                if (tri_test(r.p, tr, tr + 4, tr + 8, tmin, cur_tmax, tt, b1, b2)) {
                    if (h.id == HY_NO_HIT || better(tt, id, h)) { h = Hit{tt, id, b1, b2}; cur_tmax = tt; }
                    if (any_hit) return h;
                }
            }
        }
        g_base = w[4];
        g_bits = (hit_int << 24) | (w[3] >> 24);
    }
    return h;
}

Hit trace(const Scene& s, const float o[3], const float d[3], float tmin, float tmax, bool any_hit, int mode,
          Counters* c) {
    if (mode == 1 && s.bvh_ok) {
        if (s.two_level) return trace_2l(s, o, d, tmin, tmax, any_hit, c);
        return trace_bvh8(s, o, d, tmin, tmax, any_hit, c);
    }
    return trace_brute(s, o, d, tmin, tmax, any_hit, c);
}

}  // namespace orc
