"""The large combined configuration's scene family at a reduced size:
rotated and scaled instances of icospheres and displaced tori over the
terrain, 1024 materials, 64 area lights x 1 decorrelated sample, 2 bounces.
BVH bit-exact with the CPU build, the frame within the radiance bars of the
oracle, the adjoint over all materials and lights within 1e-3 of the FP64
CPU adjoint, and the frame batched with a second view equal to the views
rendered one by one."""
import numpy as np
import pytest

from vulkanhybridraytracer_gb300 import _lib as L
from vulkanhybridraytracer_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def large(gpu_lib, oracle_lib):
    from vulkanhybridraytracer_gb300.hybrid import HybridContext
    wl = scenes.large(4, 96, 64, n_instances=96, terrain_n=64)
    ctx = HybridContext(0)
    ctx.set_scene(wl.scene)
    info = ctx.build_bvh()
    o = oracle_lib.OracleScene()
    o.set_scene(wl.scene)
    oinfo = o.build_bvh()
    yield wl, ctx, o, info, oinfo
    ctx.close()


def test_large_bvh_bitexact(large):
    wl, ctx, o, info, oinfo = large
    assert info["num_bvh8_nodes"] == oinfo["num_bvh8_nodes"] and info["depth"] == oinfo["depth"]
    g = ctx.download_bvh(info["num_bvh8_nodes"])
    r = o.download_bvh(oinfo["num_bvh8_nodes"])
    for a, b in zip(g, r):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_large_forward_vs_oracle(large, oracle_lib):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    wl, ctx, o, _, _ = large
    po = oracle_lib
    cam = wl.camera(1.0)
    planes = o.gbuffer(cam, wl.width, wl.height)
    nl = len(wl.scene.lights)
    hist0 = np.zeros((nl, wl.height, wl.width), np.float32)
    hist_g = torch.from_numpy(hist0.copy()).cuda()
    out = torch.zeros((wl.height, wl.width, 4), device="cuda")
    pg = [torch.from_numpy(p).cuda() for p in planes]
    torch.cuda.synchronize()
    ctx.forward(pg, cam, pass_config(1, wl.max_bounces, L.HY_RNG_DECORRELATED, 0, L.HY_FLAG_NO_ACCUM), hist_g,
                L.HY_ACCUM_F32, out_f=out)
    ref, _, _, _ = o.forward(planes, cam, po.cfg_dict(spp=1, max_bounces=wl.max_bounces, rng_mode=1,
                                                       flags=L.HY_FLAG_NO_ACCUM), hist0.copy(), 1)
    got = out.cpu().numpy()[..., :3].astype(np.float64)
    ref = ref[..., :3].astype(np.float64)
    err = np.abs(got - ref)
    # a shadow ray that CUDA's sinf/cosf moves by an ulp may flip: bound those texels
    flips = err.max(-1) > 1e-2
    assert np.mean(flips) <= 5e-3
    keep = ~flips
    assert np.sqrt((err[keep] ** 2).sum() / (ref[keep] ** 2).sum()) <= 1e-3


def test_large_adjoint_vs_fp64(large, oracle_lib):
    import torch
    from vulkanhybridraytracer_gb300 import diffrender
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    wl, ctx, o, _, _ = large
    cam = wl.camera(0.0)
    planes = ctx.gbuffer(cam, wl.width, wl.height)
    nl = len(wl.scene.lights)
    shadow = torch.zeros((nl, wl.height, wl.width), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    cfg = pass_config(1, wl.max_bounces, L.HY_RNG_DECORRELATED)
    ctx.shadow_pass(planes, cam, cfg, shadow, L.HY_ACCUM_F32)
    rng = np.random.default_rng(9)
    w = torch.from_numpy(rng.normal(size=(wl.height, wl.width, 4)).astype(np.float32)).cuda()
    torch.cuda.synchronize()
    gm, gl, _ = ctx.backward(planes, cam, cfg, shadow, w, L.HY_ACCUM_F32)
    _, _, _, _, mats, lights = wl.scene.pack()
    go = oracle_lib.GradOracle(o, [p.cpu().numpy() for p in planes], cam,
                               oracle_lib.cfg_dict(spp=1, max_bounces=wl.max_bounces, rng_mode=1),
                               shadow.cpu().numpy(), 1)
    gm64, gl64 = go.adjoint(diffrender.material_params(mats).astype(np.float64),
                            diffrender.light_params(lights).astype(np.float64),
                            w.cpu().numpy()[..., :3].astype(np.float64))
    g64 = np.concatenate([gm64.ravel(), gl64.ravel()])
    g = np.concatenate([gm.cpu().numpy().ravel(), gl.cpu().numpy().ravel()]).astype(np.float64)
    scale = np.abs(g64).max()
    rel = np.abs(g - g64) / np.maximum(np.abs(g64), 1e-2 * scale)
    assert g.size == 1024 * 5 + 64 * 4
    assert rel.max() <= 1e-3, (int(np.argmax(rel)), g[np.argmax(rel)], g64[np.argmax(rel)])


def test_large_batch_equals_views(large):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    from vulkanhybridraytracer_gb300.scene import Camera
    wl, ctx, o, _, _ = large
    nl = len(wl.scene.lights)
    cams = [wl.camera(2.0), Camera((30.0, 15.0, 30.0), (0.0, 0.0, 0.0), 60.0).rt_camera(48, 32, 2.0)]
    sizes = [(wl.width, wl.height), (48, 32)]
    views, ref = [], []
    for cam, (w, h) in zip(cams, sizes):
        planes = ctx.gbuffer(cam, w, h)
        hist = torch.zeros((nl, h, w), dtype=torch.uint8, device="cuda")
        hist2 = torch.zeros((nl, h, w), dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        cfg = pass_config(1, wl.max_bounces, L.HY_RNG_DECORRELATED, 0)
        a = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")
        b = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        ctx.forward(planes, cam, cfg, hist2, L.HY_ACCUM_U8, out_8=b)
        ref.append((b, hist2))
        views.append(dict(scene=0, planes=planes, camera=cam, config=cfg, hist=hist, out_8=a))
    ctx.batch_forward([ctx], views)
    for v, (b, hist2) in zip(views, ref):
        assert torch.equal(v["out_8"], b) and torch.equal(v["hist"], hist2)
