"""Two-level structure: one BLAS per distinct mesh under a TLAS over the
primitives, the driver's BLAS/TLAS split (src/vk_mesh.cpp:424-492,
src/renderer.cpp:1696-1865) with the per-frame TLAS update of
src/vk_engine.cpp:172-187.

CPU: the oracle's two-level walk agrees with brute force over the world
triangles (rays in object space differ from world-space tests only in the
rounding of the ray transform), the TLAS update equals a fresh build, and the
layout is what the C ABI documents.  GPU (through the C ABI): node, record and
instance arrays bit-exact with the oracle, hits and traversal counts
bit-exact, the hybrid pass within the pass's radiance bars.
"""
import numpy as np
import pytest

import pyoracle as po
from vulkanhybridraytracer_gb300 import _lib as L
from vulkanhybridraytracer_gb300 import scenes
from vulkanhybridraytracer_gb300.scene import Material

NO_HIT = 0xFFFFFFFF


def _moved(xf, step):
    """Move and turn every sphere (transform 1..); keep the ground."""
    out = xf.copy().reshape(-1, 4, 4)
    ang = 0.3 * step
    for t in range(1, len(out)):
        c, s = np.float32(np.cos(ang + t)), np.float32(np.sin(ang + t))
        rot = np.array([[c, 0, -s], [0, 1, 0], [s, 0, c]], np.float32)
        out[t, :3, :3] = rot @ out[t, :3, :3]
        out[t, 3, 0] += np.float32(1.5 * np.cos(ang + t))
        out[t, 3, 1] += np.float32(0.5 * np.sin(ang * 2 + t))
        out[t, 3, 2] += np.float32(1.5 * np.sin(ang + t))
    return out.reshape(-1, 16)


def _rays(n, seed, lo=-7, hi=7):
    rng = np.random.default_rng(seed)
    org = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    org[:, 1] = rng.uniform(0.1, 4, n)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[::7] = [0, -1, 0]           # axis-aligned directions (zero components)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3], r[:, 3], r[:, 4:7], r[:, 7] = org, 0.001, d, 1000.0
    r[::11, 7] = 0.5              # short rays
    return r


def _oracle(wl, instanced=True):
    verts, idx, prims, xf, mats, lights = wl.scene.pack()
    o = po.OracleScene()
    o.set_scene(wl.scene)
    lay = o.build_bvh_instanced() if instanced else o.build_bvh()
    return o, lay, xf


def _agree(hv, hb, any_hit):
    iv, ib = hv[:, 1].view(np.uint32), hb[:, 1].view(np.uint32)
    if any_hit:
        return np.mean((iv == NO_HIT) == (ib == NO_HIT))
    return np.mean(iv == ib)


def test_oracle_layout(oracle_lib):
    wl = scenes.small(0, 32, 32)
    o, lay, xf = _oracle(wl)
    # 16 spheres share one icosphere; the ground quad is the other mesh
    assert lay["two_level"] == 1 and lay["num_instances"] == 17 and lay["num_blas"] == 2
    assert lay["tlas_region"] == 17 and 1 <= lay["tlas_nodes"] <= 17
    L_, nodes, recs, inst, boxes = o.download_bvh_instanced()
    assert L_ == lay
    assert lay["num_records"] == 17 + 2 + 320
    # unused tail of the TLAS region is zero; instance entries name each instance once
    assert not nodes[lay["tlas_nodes"]:17].any()
    ids = recs[:17, 3].view(np.uint32)
    assert sorted(ids.tolist()) == list(range(17))
    # instance records: BLAS roots inside the node array, first triangles of their primitives
    meta = inst[:, 12:16].view(np.uint32)
    assert np.all(meta[:, 0] >= 17) and np.all(meta[:, 0] < lay["num_nodes"])
    assert meta[0, 1] == 0 and np.all(np.diff(meta[1:, 1].astype(np.int64)) == 320)
    assert len(set(meta[1:, 0].tolist())) == 1            # the shared sphere BLAS
    # instance boxes contain the world triangles of their primitive
    world = o.world_tris().reshape(-1, 3, 3)
    tri0 = [0] + [2 + 320 * k for k in range(16)]
    cnt = [2] + [320] * 16
    for i in range(17):
        w = world[tri0[i]:tri0[i] + cnt[i]].reshape(-1, 3)
        assert np.all(w.min(0) >= boxes[i, :3]) and np.all(w.max(0) <= boxes[i, 3:])


@pytest.mark.parametrize("any_hit", [False, True])
def test_oracle_two_level_matches_brute(oracle_lib, any_hit):
    wl = scenes.small(0, 32, 32)
    o, lay, xf = _oracle(wl)
    rays = _rays(30000, 3)
    hb, _ = o.trace(rays, any_hit, po.TRACE_BRUTE)
    hv, cv = o.trace(rays, any_hit, po.TRACE_BVH8)
    assert _agree(hv, hb, any_hit) >= 0.9999
    if not any_hit:
        same = (hv[:, 1].view(np.uint32) == hb[:, 1].view(np.uint32)) & (hb[:, 1].view(np.uint32) != NO_HIT)
        # t in both frames: |dt| within a few ulps of the ray's coordinates
        assert np.max(np.abs(hv[same, 0] - hb[same, 0])) <= 1e-5
        np.testing.assert_allclose(hv[same, 2:], hb[same, 2:], atol=1e-4)
    # the walk visits both levels: more than the TLAS alone
    assert cv[:, 0].mean() > 1.0


def test_oracle_tlas_update_equals_fresh_build(oracle_lib):
    wl = scenes.small(0, 32, 32)
    verts, idx, prims, xf, mats, lights = wl.scene.pack()
    o = po.OracleScene()
    o.set_scene_arrays(verts, idx, prims, xf, mats, lights)
    o.build_bvh_instanced()
    for step in (1, 3):
        x2 = _moved(xf, step)
        o.refit_bvh(x2)
        f = po.OracleScene()
        f.set_scene_arrays(verts, idx, prims, x2, mats, lights)
        f.build_bvh_instanced()
        a, b = o.download_bvh_instanced(), f.download_bvh_instanced()
        assert a[0] == b[0]
        for x, y in zip(a[1:], b[1:]):
            assert np.array_equal(x.view(np.uint32), y.view(np.uint32))
        rays = _rays(20000, 20 + step)
        hb, _ = o.trace(rays, False, po.TRACE_BRUTE)
        hv, _ = o.trace(rays, False, po.TRACE_BVH8)
        assert _agree(hv, hb, False) >= 0.9999


def test_oracle_two_level_pass_close_to_flat(oracle_lib):
    """The hybrid pass over the two-level structure stays within the radiance
    bars of the same pass over the flattened one."""
    wl = scenes.small(0, 48, 48)
    cam = wl.camera(1.0)
    res = []
    for inst in (False, True):
        o, _, _ = _oracle(wl, inst)
        planes = o.gbuffer(cam, wl.width, wl.height)
        nl = len(wl.scene.lights)
        hist = np.full((nl, wl.height, wl.width), 128, np.uint8)
        of, o8, osh, ost = o.forward(planes, cam, po.cfg_dict(4, 1, L.HY_RNG_DECORRELATED, 1, 0), hist,
                                     L.HY_ACCUM_U8)
        res.append((of, hist))
    (fa, ha), (fb, hb) = res
    assert np.mean(ha != hb) <= 1e-3
    err = np.abs(fa[..., :3].astype(np.float64) - fb[..., :3])
    rms = np.sqrt((err ** 2).sum() / max((fa[..., :3].astype(np.float64) ** 2).sum(), 1e-30))
    assert rms <= 1e-3


# ---------------------------------------------------------------------------- GPU


def _gpu_pair(wl):
    from vulkanhybridraytracer_gb300.hybrid import HybridContext
    ctx = HybridContext(0)
    ctx.set_scene(wl.scene)
    gi = ctx.build_bvh(instanced=True)
    o = po.OracleScene()
    o.set_scene(wl.scene)
    o.build_bvh_instanced()
    return ctx, gi, o


def _assert_same_structure(ctx, o):
    g = ctx.download_bvh_instanced()
    r = o.download_bvh_instanced()
    assert g[0] == r[0], (g[0], r[0])
    for name, a, b in zip(["nodes", "records", "instances", "boxes"], g[1:], r[1:]):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), name


@pytest.mark.gpu
def test_gpu_instanced_bitexact(gpu_lib, oracle_lib):
    wl = scenes.small(0, 32, 32)
    ctx, gi, o = _gpu_pair(wl)
    assert gi["num_tris"] == wl.scene.num_tris
    _assert_same_structure(ctx, o)
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("any_hit", [False, True])
def test_gpu_instanced_trace_bitexact(gpu_lib, oracle_lib, any_hit):
    import torch
    wl = scenes.small(0, 32, 32)
    ctx, gi, o = _gpu_pair(wl)
    assert ctx.anyhit_order() == L.HY_ANYHIT_NEAR_FIRST  # AUTO on a two-level structure
    rays = _rays(50000, 7)
    hg, sg = ctx.trace(torch.from_numpy(rays).cuda(), any_hit, count=True)
    ho, co = o.trace(rays, any_hit)
    assert np.array_equal(hg.cpu().numpy().view(np.uint32), ho.view(np.uint32))
    assert sg["nodes_visited"] == int(co[:, 0].sum()) and sg["tris_tested"] == int(co[:, 1].sum())
    assert sg["error_flags"] == 0
    ctx.close()


@pytest.mark.gpu
def test_gpu_instanced_tlas_update_bitexact(gpu_lib, oracle_lib):
    import torch
    wl = scenes.small(0, 32, 32)
    verts, idx, prims, xf, mats, lights = wl.scene.pack()
    ctx, gi, o = _gpu_pair(wl)
    for step in (1, 4):
        x2 = _moved(xf, step)
        ctx.refit_bvh(x2)
        o.refit_bvh(x2)
        _assert_same_structure(ctx, o)
        rays = _rays(20000, 30 + step)
        hg, sg = ctx.trace(torch.from_numpy(rays).cuda(), False, count=True)
        ho, co = o.trace(rays, False)
        assert np.array_equal(hg.cpu().numpy().view(np.uint32), ho.view(np.uint32))
        assert sg["nodes_visited"] == int(co[:, 0].sum())
    ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("rng_mode,spp,flags", [(L.HY_RNG_REFERENCE, 1, 0), (L.HY_RNG_DECORRELATED, 4, 0),
                                                (L.HY_RNG_DECORRELATED, 4, L.HY_FLAG_PIXEL_PARALLEL)])
def test_gpu_instanced_pass_parity(gpu_lib, oracle_lib, rng_mode, spp, flags):
    """Shadow (lane-group and pixel-parallel kernels), accumulation and shading
    with mirror/glass bounces over the two-level structure, against the
    oracle's pass over the same structure."""
    from test_gpu_parity import Pair, check_parity, run_both
    wl = scenes.small(0, 64, 64)
    for i in (2, 5):
        wl.scene.materials[i] = Material(4, (0.9, 0.95, 1.0, 1), 1.0, 0.0, 1.5)
    wl.scene.materials[3] = Material(3, (0.8, 0.8, 0.8, 1), 1.0, 0.05, 1.0)
    wl.max_bounces = 4
    p = Pair(wl, build=False)
    p.gi = p.ctx.build_bvh(instanced=True)
    p.oi = p.orc.build_bvh_instanced()
    for frame in (0, 2):
        g, o = run_both(p, frame, spp, rng_mode, L.HY_ACCUM_U8, flags=flags)
        check_parity(g, o, L.HY_ACCUM_U8)
    p.ctx.close()


@pytest.mark.gpu
def test_gpu_instanced_unsupported_paths(gpu_lib, oracle_lib):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    wl = scenes.small(0, 32, 32)
    ctx, gi, o = _gpu_pair(wl)
    cam = wl.camera(1.0)
    planes = ctx.gbuffer(cam, 32, 32)
    hist = torch.zeros((len(wl.scene.lights), 32, 32), dtype=torch.uint8, device="cuda")
    with pytest.raises(L.HyError) as e:
        ctx.forward(planes, cam, pass_config(4, 1, L.HY_RNG_DECORRELATED, 1, L.HY_FLAG_RAY_POOL), hist)
    assert e.value.code == L.HY_ERR_UNSUPPORTED
    with pytest.raises(L.HyError):
        ctx.download_bvh(gi["num_bvh8_nodes"])     # morton / order / bvh2 do not exist here
    # a one-level build on the same context replaces the two-level one
    ctx.build_bvh()
    assert ctx.bvh_layout()["two_level"] == 0
    ctx.close()


@pytest.mark.gpu
def test_gpu_instanced_pathtrace_parity(gpu_lib, oracle_lib):
    """The path-traced mode (camera rays, closesthit shading, shadow rays at every
    hit) over the two-level structure against the oracle's over the same one."""
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    wl = scenes.small_glass(64, 48)
    ctx, gi, o = _gpu_pair(wl)
    try:
        img = torch.zeros((wl.height, wl.width, 4), dtype=torch.uint8, device="cuda")
        out = torch.zeros((wl.height, wl.width, 4), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        img_o = np.zeros((wl.height, wl.width, 4), np.uint8)
        for frame in (-1.0, 1.0):
            cam = wl.camera(frame)
            img, st = ctx.pathtrace(cam, wl.width, wl.height, pass_config(4, 8, L.HY_RNG_DECORRELATED), img,
                                    out_f=out)
            img_o, out_o, st_o = o.pathtrace(cam, wl.width, wl.height,
                                             po.cfg_dict(spp=4, max_bounces=8, rng_mode=L.HY_RNG_DECORRELATED), img_o)
            got = out.cpu().numpy()[..., :3].astype(np.float64)
            ref = out_o[..., :3].astype(np.float64)
            err = np.abs(got - ref)
            rms = np.sqrt((err ** 2).sum() / max((ref ** 2).sum(), 1e-30))
            assert rms <= 1e-3, (frame, rms)
            assert np.mean(err.max(-1) > 1e-2) <= 2e-3
            assert st["error_flags"] == 0
            assert abs(st["shadow_rays"] - st_o["shadow_rays"]) <= 1e-3 * st_o["shadow_rays"] + 4
    finally:
        ctx.close()


@pytest.mark.gpu
def test_gpu_instanced_batch_equals_per_view(gpu_lib, oracle_lib):
    """A batch mixing a two-level scene and a one-level one (tile streams, graph
    replay) equals the views rendered one by one, bit for bit."""
    import torch
    from vulkanhybridraytracer_gb300.hybrid import HybridContext, pass_config
    wa, wb = scenes.small(0, 48, 40), scenes.small_glass(40, 32)
    ca, cb = HybridContext(0), HybridContext(0)
    ca.set_scene(wa.scene)
    ca.build_bvh(instanced=True)
    cb.set_scene(wb.scene)
    cb.build_bvh()
    runner = HybridContext(0)
    try:
        views = []
        for si, (c, wl, spp, rng_mode) in enumerate(((ca, wa, 4, L.HY_RNG_DECORRELATED), (cb, wb, 1, L.HY_RNG_REFERENCE),
                                                      (ca, wa, 1, L.HY_RNG_REFERENCE))):
            cam = wl.scene.camera.rt_camera(wl.width, wl.height, 3.0)
            planes = c.gbuffer(cam, wl.width, wl.height)
            hist = torch.full((len(wl.scene.lights), wl.height, wl.width), 90, dtype=torch.uint8, device="cuda")
            views.append(dict(scene=0 if c is ca else 1, planes=planes, camera=cam,
                              config=pass_config(spp, 4, rng_mode, 3, 0), hist=hist,
                              out_8=torch.zeros((wl.height, wl.width, 4), dtype=torch.uint8, device="cuda")))
        torch.cuda.synchronize()
        ref = []
        for v in views:
            h = v["hist"].clone()
            o = torch.zeros_like(v["out_8"])
            torch.cuda.synchronize()
            (ca if v["scene"] == 0 else cb).forward(v["planes"], v["camera"], v["config"], h, out_8=o)
            ref.append((h, o))
        torch.cuda.synchronize()
        st = runner.batch_forward([ca, cb], views, graph=True)
        torch.cuda.synchronize()
        assert st["error_flags"] == 0
        for v, (h, o) in zip(views, ref):
            assert torch.equal(v["hist"], h) and torch.equal(v["out_8"], o)
        with pytest.raises(L.HyError) as e:
            runner.batch_forward([ca, cb], views, tuning=pass_config(1, flags=L.HY_FLAG_LANE_GROUPS))
        assert e.value.code == L.HY_ERR_UNSUPPORTED
    finally:
        runner.close()
        ca.close()
        cb.close()
