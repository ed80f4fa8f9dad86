"""CPU tests of the binned-SAH build (HY_BUILD_SAH, the default) in the oracle:
an independent numpy restatement of every node's split decision, the tree's
numbering and ranges, traversal against brute force, and fewer node visits
than the LBVH on shadow-like rays."""
import numpy as np
import pytest

import pyoracle as po
from vulkanhybridraytracer_gb300 import scenes

LEAF = 0x80000000
BINS = 32
F32 = np.float32


def okey(x: np.ndarray) -> np.ndarray:
    """Order-preserving int32 key of float32 bits (-0 below +0)."""
    b = np.ascontiguousarray(x, F32).view(np.int32).astype(np.int64)
    return np.where(b >= 0, b, b ^ 0x7FFFFFFF)


def unkey(k) -> np.ndarray:
    k = np.asarray(k, np.int64)
    return np.where(k >= 0, k, k ^ 0x7FFFFFFF).astype(np.int32).view(F32)


def area(lo_k, hi_k):
    lo, hi = unkey(lo_k), unkey(hi_k)
    d = (hi - lo).astype(F32)
    a = (d[..., 0] * d[..., 1]).astype(F32)
    a = (a + (d[..., 1] * d[..., 2]).astype(F32)).astype(F32)
    return (a + (d[..., 2] * d[..., 0]).astype(F32)).astype(F32)


def sah_decision(cen: np.ndarray, box: np.ndarray):
    """(axis, q, left mask) of the split of one range, or None (no candidate):
    32 bins per axis over the centroid bounds, cost area(L) n(L) + area(R) n(R),
    the first strictly lowest finite cost in (axis, q) order."""
    ck = okey(cen)
    lo = unkey(ck.min(0))
    ext = (unkey(ck.max(0)) - lo).astype(F32)
    best, pick = np.inf, None
    blo, bhi = okey(box[:, :3]), okey(box[:, 3:])
    for a in range(3):
        if not ext[a] > 0:
            continue
        scale = F32(BINS) / ext[a]
        v = ((cen[:, a] - lo[a]).astype(F32) * scale).astype(F32)
        q = np.where(v >= 0, np.where(v < BINS, np.floor(np.where(v >= 0, v, 0)), BINS - 1), 0).astype(np.int64)
        cnt = np.bincount(q, minlength=BINS)
        lo_b = np.full((BINS, 3), 2**31 - 1, np.int64)
        hi_b = np.full((BINS, 3), -(2**31), np.int64)
        np.minimum.at(lo_b, q, blo)
        np.maximum.at(hi_b, q, bhi)
        lc, rc = np.cumsum(cnt)[:-1], np.cumsum(cnt[::-1])[::-1][1:]
        llo, lhi = np.minimum.accumulate(lo_b)[:-1], np.maximum.accumulate(hi_b)[:-1]
        rlo = np.minimum.accumulate(lo_b[::-1])[::-1][1:]
        rhi = np.maximum.accumulate(hi_b[::-1])[::-1][1:]
        with np.errstate(invalid="ignore", over="ignore"):
            t1 = (area(llo, lhi) * lc.astype(F32)).astype(F32)
            t2 = (area(rlo, rhi) * rc.astype(F32)).astype(F32)
            cost = ((t1 + t2).astype(F32) + F32(0)).astype(F32)
        for k in range(BINS - 1):
            if lc[k] and rc[k] and np.isfinite(cost[k]) and cost[k] < best:
                best, pick = cost[k], (a, k, q <= k)
    return pick


def tri_boxes(world: np.ndarray):
    w = world.reshape(-1, 3, 3)
    lo, hi = w.min(1), w.max(1)
    cen = ((lo + hi).astype(F32) * F32(0.5)).astype(F32)
    return cen, np.concatenate([lo, hi], 1).astype(F32)


def build(wl, mode):
    o = po.OracleScene()
    o.set_scene(wl.scene)
    o.set_build_mode(mode)
    info = o.build_bvh()
    return o, info


@pytest.fixture(scope="module")
def sah_small(oracle_lib):
    wl = scenes.small(0, 64, 64)
    o, info = build(wl, po.HY_BUILD_SAH)
    return wl, o, info


def test_sah_tree_numbering_and_ranges(sah_small):
    """Node m - 1 splits its range before position m; every index of [0, n-1)
    is one node; children partition their parent; boxes are the children's union."""
    wl, o, info = sah_small
    n = info["num_tris"]
    morton, order, bvh2, bvh8, tris = o.download_bvh(info["num_bvh8_nodes"])
    assert sorted(order.tolist()) == list(range(n))
    roots = np.nonzero((bvh2[:, 2] == 0) & (bvh2[:, 3] == n - 1))[0]
    assert len(roots) == 1
    seen = np.zeros(n - 1, bool)
    seen[roots[0]] = True
    box = bvh2[:, 4:10].view(F32)
    cen, tb = tri_boxes(o.world_tris())
    for i in range(n - 1):
        left, right, f, la = (int(v) for v in bvh2[i, :4])
        lr = (left & ~LEAF, left & ~LEAF) if left & LEAF else (int(bvh2[left, 2]), int(bvh2[left, 3]))
        rr = (right & ~LEAF, right & ~LEAF) if right & LEAF else (int(bvh2[right, 2]), int(bvh2[right, 3]))
        assert lr[0] == f and rr[1] == la and lr[1] + 1 == rr[0]
        assert i == rr[0] - 1  # node id = split position - 1
        for ch in (left, right):
            if not ch & LEAF:
                assert not seen[ch]
                seen[ch] = True
        cb = [tb[order[c & ~LEAF]] if c & LEAF else box[c] for c in (left, right)]
        assert np.array_equal(box[i, :3], np.minimum(cb[0][:3], cb[1][:3]))
        assert np.array_equal(box[i, 3:], np.maximum(cb[0][3:], cb[1][3:]))
    assert seen.all()
    # morton: the code of each triangle in leaf order (no longer sorted)
    assert len(morton) == n and not np.all(np.diff(morton.astype(np.int64)) >= 0)


def test_sah_split_decisions_restated(sah_small):
    """Every node's split equals an independent numpy restatement of the binned
    SAH (computed from the set of triangles in its range, which does not depend
    on their order), and ranges without a candidate split at their middle."""
    wl, o, info = sah_small
    n = info["num_tris"]
    _, order, bvh2, _, _ = o.download_bvh(info["num_bvh8_nodes"])
    cen, tb = tri_boxes(o.world_tris())
    medians = 0
    for i in range(n - 1):
        f, la = int(bvh2[i, 2]), int(bvh2[i, 3])
        m = i + 1
        ids = order[f:la + 1]
        d = sah_decision(cen[ids], tb[ids])
        if d is None:
            assert m == f + (la - f + 1) // 2
            medians += 1
        else:
            _, _, left = d
            assert m == f + int(left.sum())
            assert set(order[f:m].tolist()) == set(ids[left].tolist())
    assert medians < n // 100


def test_sah_degenerate_inputs(oracle_lib):
    """Coincident centroids (median splits), points and duplicates: the tree is
    complete and traversal equals brute force."""
    rng = np.random.default_rng(7)
    for n in (2, 3, 5, 33, 700):
        v = np.zeros((3 * n, 11), np.float32)
        base = rng.uniform(-1, 1, (n, 3))
        base[n // 2:] = base[0]
        for t in range(n):
            for k in range(3):
                v[3 * t + k, 0:3] = base[t] + (rng.uniform(-0.5, 0.5, 3) if t % 5 else 0)
                v[3 * t + k, 4] = 1
        idx = np.arange(3 * n, dtype=np.uint32)
        prims = np.array([[0, 3 * n, 0, 0, 0, 0]], np.uint32)
        xf = np.eye(4, dtype=np.float32).reshape(1, 16)
        from vulkanhybridraytracer_gb300.scene import Material
        o = po.OracleScene()
        o.set_scene_arrays(v, idx, prims, xf, Material().to_shader(0)[None], np.zeros((0, 12), np.float32))
        info = o.build_bvh()
        _, order, bvh2, _, _ = o.download_bvh(info["num_bvh8_nodes"])
        assert sorted(order.tolist()) == list(range(n))
        r = np.zeros((2000, 8), np.float32)
        r[:, 0:3] = rng.uniform(-2, 2, (2000, 3))
        d = rng.normal(size=(2000, 3))
        r[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
        r[:, 3], r[:, 7] = 1e-3, 100.0
        for any_hit in (False, True):
            hb, _ = o.trace(r, any_hit, po.TRACE_BRUTE)
            hv, _ = o.trace(r, any_hit, po.TRACE_BVH8)
            if any_hit:
                assert np.array_equal(hb.view(np.uint32)[:, 1] != 0xFFFFFFFF, hv.view(np.uint32)[:, 1] != 0xFFFFFFFF)
            else:
                assert np.array_equal(hb.view(np.uint32), hv.view(np.uint32))


def test_sah_fewer_visits_than_lbvh(oracle_lib):
    """Shadow-like rays (surface points towards lights above the scene): the
    SAH structure makes fewer node visits than the LBVH, the same occlusion."""
    wl = scenes.hd(width=96, height=54, n_spheres=16, terrain_n=128)
    rng = np.random.default_rng(11)
    k = 6000
    res = {}
    for mode in (po.HY_BUILD_SAH, po.HY_BUILD_LBVH):
        o, _ = build(wl, mode)
        if mode == po.HY_BUILD_SAH:
            w = o.world_tris().reshape(-1, 3, 3)
            pick = rng.integers(0, len(w), k)
            bary = rng.dirichlet((1, 1, 1), k).astype(F32)
            org = np.einsum("kv,kva->ka", bary, w[pick]).astype(F32)
            tgt = np.stack([rng.uniform(-30, 30, k), rng.uniform(8, 16, k), rng.uniform(-30, 30, k)], 1)
            d = tgt - org
            dist = np.linalg.norm(d, axis=1)
            rays = np.zeros((k, 8), F32)
            rays[:, 0:3], rays[:, 4:7], rays[:, 3], rays[:, 7] = org, d / dist[:, None], 1e-3, dist
        o.set_anyhit_order(po.HY_ANYHIT_FAR_FIRST)
        h, cnt = o.trace(rays, True)
        res[mode] = (h.view(np.uint32)[:, 1] != 0xFFFFFFFF, cnt[:, 0].mean())
        if mode == po.HY_BUILD_SAH:  # far first still makes fewer visits than near first
            o.set_anyhit_order(po.HY_ANYHIT_NEAR_FIRST)
            hn, cn = o.trace(rays, True)
            assert np.array_equal(hn.view(np.uint32)[:, 1] != 0xFFFFFFFF, res[mode][0])
            assert cnt[:, 0].mean() < cn[:, 0].mean()
    assert np.array_equal(res[po.HY_BUILD_SAH][0], res[po.HY_BUILD_LBVH][0])
    assert res[po.HY_BUILD_SAH][1] < 0.9 * res[po.HY_BUILD_LBVH][1]


def _surface32(lo, hi):
    d = (np.asarray(hi, F32) - np.asarray(lo, F32)).astype(F32)
    a = F32(d[0] * d[1])
    a = F32(a + F32(d[1] * d[2]))
    return F32(a + F32(d[2] * d[0]))


def test_collapse_slot_budgets_restated(sah_small):
    """Every 8-wide node's children are its binary subtree spread over 8 slots by the
    surface-area program (leaf slot: area x triangles x 0.5; internal node: area +
    its own 8 slots; first strict minimum in split order), restated here in numpy
    float32 from the downloaded binary tree and compared as sets of triangles."""
    wl, o, info = sah_small
    n = info["num_tris"]
    _, order, bvh2, bvh8, tris = o.download_bvh(info["num_bvh8_nodes"])
    box = bvh2[:, 4:10].view(F32)
    w = o.world_tris().reshape(-1, 3, 3)
    tlo, thi = w.min(1), w.max(1)
    ids = tris[:, 3].view(np.uint32)

    memo = {}

    def f(m):  # the 8 costs f(m, 1..8)
        if m & LEAF:
            t = order[m & ~LEAF]
            return [F32(_surface32(tlo[t], thi[t]) * F32(0.5))] * 8, None
        if m in memo:
            return memo[m]
        L, R, first, last = (int(v) for v in bvh2[m, :4])
        fl, _ = f(L)
        fr, _ = f(R)
        A = _surface32(box[m, :3], box[m, 3:])
        cnt = last - first + 1
        best8, bk = np.float32(np.inf), 1
        for k in range(1, 8):
            v = F32(fl[k - 1] + fr[8 - k - 1])
            if v < best8:
                best8, bk = v, k
        fv = [F32(F32(A * F32(cnt)) * F32(0.5)) if cnt <= 3 else F32(F32(A * F32(1.0)) + best8)]
        kk = [bk, 0]
        for i in range(2, 9):
            v, ki = fv[i - 2], 0
            for k in range(1, i):
                w_ = F32(fl[k - 1] + fr[i - k - 1])
                if w_ < v:
                    v, ki = w_, k
            fv.append(v)
            kk.append(ki)
        memo[m] = (fv, kk)
        return memo[m]

    def expand(m, i, out):
        while not (m & LEAF) and i > 1 and f(m)[1][i] == 0:
            i -= 1
        if (m & LEAF) or i == 1:
            out.append(m)
            return
        k = f(m)[1][i]
        expand(int(bvh2[m, 0]), k, out)
        expand(int(bvh2[m, 1]), i - k, out)

    import sys
    sys.setrecursionlimit(10000)

    def tri_set(ref):
        if ref & LEAF:
            return frozenset([int(order[ref & ~LEAF])])
        return frozenset(int(t) for t in order[bvh2[ref, 2]:bvh2[ref, 3] + 1])

    node_of_set = {tri_set(m): m for m in range(n - 1)}

    def bvh8_children(k):
        w8 = bvh8[k]
        meta = list(w8[6:8].view(np.uint8))
        base, tbase, rank, kids = int(w8[4]), int(w8[5]), 0, []
        for sl in range(8):
            mb = int(meta[sl])
            if mb == 0:
                continue
            if mb == 0x80:
                kids.append(("node", base + rank))
                rank += 1
            else:
                c, off = mb >> 5, mb & 31
                kids.append(("tris", frozenset(int(t) for t in ids[tbase + off:tbase + off + c])))
        return kids

    sets8 = {}

    def subtree_set(k):
        if k not in sets8:
            s = set()
            for kind, v in bvh8_children(k):
                s |= subtree_set(v) if kind == "node" else v
            sets8[k] = frozenset(s)
        return sets8[k]

    for k in range(len(bvh8)):
        whole = subtree_set(k)
        m = node_of_set[whole]
        want = []
        expand(int(bvh2[m, 1]), 8 - f(m)[1][0], want)
        left = []
        expand(int(bvh2[m, 0]), f(m)[1][0], left)
        want = {tri_set(r) for r in left + want}
        got = {subtree_set(v) if kind == "node" else v for kind, v in bvh8_children(k)}
        assert got == want, k
