"""BVH refit: new transforms, same topology (the per-frame TLAS update of
src/vk_engine.cpp:172-187, built with ALLOW_UPDATE).  The refitted tree stays
correct (traversal == brute force) and the GPU refit equals the oracle's
array for array."""
import numpy as np
import pytest

import pyoracle as po
from vulkanhybridraytracer_gb300 import scenes


def _moved(xf, step):
    """Move every sphere (transform 1..) along a circle; keep the ground."""
    out = xf.copy().reshape(-1, 4, 4)
    ang = 0.3 * step
    for t in range(1, len(out)):
        out[t, 3, 0] += np.float32(1.5 * np.cos(ang + t))
        out[t, 3, 1] += np.float32(0.5 * np.sin(ang * 2 + t))
        out[t, 3, 2] += np.float32(1.5 * np.sin(ang + t))
    return out.reshape(-1, 16)


def _rays(n, seed):
    rng = np.random.default_rng(seed)
    org = rng.uniform(-7, 7, (n, 3)).astype(np.float32)
    org[:, 1] = rng.uniform(0.1, 4, n)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3], r[:, 3], r[:, 4:7], r[:, 7] = org, 0.001, d, 1000.0
    return r


def test_oracle_refit_traversal_correct(oracle_lib):
    wl = scenes.small(0, 32, 32)
    verts, idx, prims, xf, mats, lights = wl.scene.pack()
    o = po.OracleScene()
    o.set_scene_arrays(verts, idx, prims, xf, mats, lights)
    o.build_bvh()
    for step in (1, 2, 5):
        o.refit_bvh(_moved(xf, step))
        rays = _rays(3000, step)
        hb, _ = o.trace(rays, False, po.TRACE_BRUTE)
        hv, _ = o.trace(rays, False, po.TRACE_BVH8)
        assert np.array_equal(hb.view(np.uint32), hv.view(np.uint32))
    # refit with the original transforms restores the original structure exactly
    o2 = po.OracleScene()
    o2.set_scene_arrays(verts, idx, prims, xf, mats, lights)
    info = o2.build_bvh()
    o.refit_bvh(xf)
    a = o.download_bvh(info["num_bvh8_nodes"])
    b = o2.download_bvh(info["num_bvh8_nodes"])
    for x, y in zip(a, b):
        assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


@pytest.mark.gpu
def test_gpu_refit_bitexact(gpu_lib, oracle_lib):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import HybridContext
    wl = scenes.small(0, 32, 32)
    verts, idx, prims, xf, mats, lights = wl.scene.pack()
    ctx = HybridContext(0)
    ctx.set_scene_arrays(verts, idx, prims, xf, mats, lights)
    gi = ctx.build_bvh()
    o = po.OracleScene()
    o.set_scene_arrays(verts, idx, prims, xf, mats, lights)
    o.build_bvh()
    for step in (1, 4):
        x2 = _moved(xf, step)
        ctx.refit_bvh(x2)
        o.refit_bvh(x2)
        g = ctx.download_bvh(gi["num_bvh8_nodes"])
        r = o.download_bvh(gi["num_bvh8_nodes"])
        for name, a, b in zip(["morton", "order", "bvh2", "bvh8", "tris"], g, r):
            assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), name
        rays = _rays(20000, 10 + step)
        hg, sg = ctx.trace(torch.from_numpy(rays).cuda(), False, count=True)
        ho, co = o.trace(rays, False)
        assert np.array_equal(hg.cpu().numpy().view(np.uint32), ho.view(np.uint32))
        assert sg["nodes_visited"] == int(co[:, 0].sum())
    ctx.close()
