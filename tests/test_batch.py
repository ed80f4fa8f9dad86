"""Batched form: many views over several scenes in one persistent launch
(hy_batch_forward), against the same views run one by one through
hy_hybrid_forward.  Both use the same per-view rays, so histories and
images must agree bit for bit, with and without graph replay."""
import numpy as np
import pytest

from vulkanhybridraytracer_gb300 import _lib as L
from vulkanhybridraytracer_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def two_scenes(gpu_lib):
    from vulkanhybridraytracer_gb300.hybrid import HybridContext
    a = scenes.small(0, 8, 8)
    b = scenes.small_glass(8, 8)
    b.scene.lights = b.scene.lights[:1] + [b.scene.lights[0].__class__(0, (1, 0.5, 0.2), (-3, 5, 1), 15.0, 500.0, 0.3)] * 2
    ctxs = []
    for wl in (a, b):
        c = HybridContext(0)
        c.set_scene(wl.scene)
        c.build_bvh()
        ctxs.append((c, wl))
    runner = HybridContext(0)
    yield runner, ctxs
    runner.close()
    for c, _ in ctxs:
        c.close()


def _views(ctxs, frame0, seed=0):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    rng = np.random.default_rng(seed)
    specs = [(0, 96, 64, 1, L.HY_RNG_REFERENCE, 1, 0), (1, 80, 80, 4, L.HY_RNG_DECORRELATED, 8, 0),
             (0, 120, 40, 16, L.HY_RNG_DECORRELATED, 1, 0), (1, 33, 57, 3, L.HY_RNG_DECORRELATED, 8, 0),
             (0, 64, 64, 8, L.HY_RNG_DECORRELATED, 1, L.HY_FLAG_NO_ACCUM), (1, 72, 48, 1, L.HY_RNG_REFERENCE, 8, 0)]
    views = []
    for i, (si, w, h, spp, rng_mode, bounces, flags) in enumerate(specs):
        c, wl = ctxs[si]
        frame = frame0 + i if i != 3 else 0   # view 3 is on its reset frame
        cam = wl.scene.camera.rt_camera(w, h, float(frame))
        planes = c.gbuffer(cam, w, h)
        nl = len(wl.scene.lights) if i != 2 else 1   # view 2 uses only the scene's first light
        hist = torch.from_numpy(rng.integers(0, 256, (nl, h, w)).astype(np.uint8)).cuda()
        views.append(dict(scene=si, planes=planes, camera=cam, config=pass_config(spp, bounces, rng_mode, frame, flags),
                          hist=hist, out_f=torch.zeros((h, w, 4), device="cuda"),
                          out_8=torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")))
    return views


@pytest.mark.parametrize("graph,sched", [(False, 0), (True, 0), (False, L.HY_FLAG_LANE_GROUPS),
                                         (True, L.HY_FLAG_LANE_GROUPS)])
def test_batch_equals_per_view(two_scenes, graph, sched):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    runner, ctxs = two_scenes
    tuning = pass_config(1, flags=sched)
    scene_ctx = [c for c, _ in ctxs]
    for rep in range(3):   # the graph is captured once, then replayed with new frames
        views = _views(ctxs, 3 + 5 * rep, seed=rep)
        ref = []
        for v in views:
            h = v["hist"].clone()
            of, o8 = torch.zeros_like(v["out_f"]), torch.zeros_like(v["out_8"])
            torch.cuda.synchronize()   # the library runs on its own streams
            st = scene_ctx[v["scene"]].forward(v["planes"], v["camera"], v["config"], h, out_f=of, out_8=o8)
            ref.append((h, of, o8, st))
        torch.cuda.synchronize()
        st = runner.batch_forward(scene_ctx, views, graph=graph, tuning=tuning)
        torch.cuda.synchronize()
        assert st["error_flags"] == 0
        for v, (h, of, o8, st1) in zip(views, ref):
            assert torch.equal(v["hist"], h)
            assert torch.equal(v["out_f"], of)
            assert torch.equal(v["out_8"], o8)
        tot = sum(r[3]["shadow_rays"] for r in ref)
        assert st["shadow_rays"] == tot


def _per_view(scene_ctx, views):
    import torch
    ref = []
    for v in views:
        h = v["hist"].clone()
        of, o8 = torch.zeros_like(v["out_f"]), torch.zeros_like(v["out_8"])
        torch.cuda.synchronize()
        scene_ctx[v["scene"]].forward(v["planes"], v["camera"], v["config"], h, out_f=of, out_8=o8)
        ref.append((h, of, o8))
    torch.cuda.synchronize()
    return ref


@pytest.mark.parametrize("block,minb,depth", [(64, 8, 0), (256, 6, 32), (128, 8, 16), (64, 6, 8), (256, 8, 0)])
def test_batch_launch_shapes_equal_per_view(two_scenes, block, minb, depth):
    """Every launch shape of the batch's tile-stream kernel (threads per block,
    register cap, shared-memory stack entries) writes the views' histories and
    images bit for bit as the per-view passes do."""
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    runner, ctxs = two_scenes
    scene_ctx = [c for c, _ in ctxs]
    views = _views(ctxs, 11, seed=7)
    ref = _per_view(scene_ctx, views)
    tuning = pass_config(1, queue_chunk=2, block_size=block, min_blocks=minb, stack_depth=depth)
    for graph in (False, True):
        vs = [dict(v, hist=v["hist"].clone(), out_f=torch.zeros_like(v["out_f"]), out_8=torch.zeros_like(v["out_8"]))
              for v in views]
        torch.cuda.synchronize()
        st = runner.batch_forward(scene_ctx, vs, graph=graph, tuning=tuning)
        torch.cuda.synchronize()
        assert st["error_flags"] == 0
        for v, (h, of, o8) in zip(vs, ref):
            assert torch.equal(v["hist"], h) and torch.equal(v["out_f"], of) and torch.equal(v["out_8"], o8)


def test_batch_rejects_unknown_shapes(two_scenes):
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    runner, ctxs = two_scenes
    views = _views(ctxs, 2)
    for kw in (dict(block_size=96), dict(stack_depth=12), dict(min_blocks=7), dict(queue_chunk=2048)):
        with pytest.raises(L.HyError) as e:
            runner.batch_forward([c for c, _ in ctxs], views, tuning=pass_config(1, **kw))
        assert e.value.code == L.HY_ERR_INVALID_ARG, kw
    with pytest.raises(L.HyError) as e:   # counting launches run the default shape only
        runner.batch_forward([c for c, _ in ctxs], views,
                             tuning=pass_config(1, flags=L.HY_FLAG_COUNT_TRAVERSAL, block_size=256))
    assert e.value.code == L.HY_ERR_UNSUPPORTED


def test_batch_autotune_returns_a_shape_that_renders_the_same(two_scenes):
    """hy_batch_autotune (the C-ABI tuner): a shape from the tuning space, whose batch
    equals the per-view passes."""
    import torch
    from vulkanhybridraytracer_gb300 import autotune
    runner, ctxs = two_scenes
    scene_ctx = [c for c, _ in ctxs]
    views = _views(ctxs, 21, seed=3)
    scratch = [dict(v, hist=v["hist"].clone()) for v in views]   # tuning overwrites histories
    t, ms = runner.batch_autotune(scene_ctx, scratch, reps=1)
    assert ms > 0
    assert t.queue_chunk in (1, 2, 4, 8, 16, 32) and t.block_size in (64, 128, 256)
    assert t.min_blocks in (6, 8) and t.stack_depth in (0, 8, 16, 32)
    ref = _per_view(scene_ctx, views)
    shape = {"chunk": t.queue_chunk, "block": t.block_size, "min_blocks": t.min_blocks, "stack_depth": t.stack_depth}
    st = runner.batch_forward(scene_ctx, views, tuning=autotune.tuning_config(shape))
    torch.cuda.synchronize()
    assert st["error_flags"] == 0
    for v, (h, of, o8) in zip(views, ref):
        assert torch.equal(v["hist"], h) and torch.equal(v["out_f"], of) and torch.equal(v["out_8"], o8)


@pytest.mark.parametrize("frame", [0, 4])
def test_batched_view_against_oracle(gpu_lib, oracle_lib, frame):
    """A view rendered inside a batch (next to a view of another scene) against the
    CPU oracle directly, with the parity bars of the single-view pass."""
    import torch
    from test_gpu_parity import Pair, check_parity
    from vulkanhybridraytracer_gb300.hybrid import HybridContext, pass_config
    import pyoracle as po
    p = Pair(scenes.small(0, 64, 48))
    other = HybridContext(0)
    glass = scenes.small_glass(40, 24)
    other.set_scene(glass.scene)
    other.build_bvh()
    runner = HybridContext(0)
    try:
        wl = p.wl
        W, H, nl = wl.width, wl.height, len(wl.scene.lights)
        cam = wl.camera(float(frame))
        planes_np = p.orc.gbuffer(cam, W, H)
        rng = np.random.default_rng(frame + 5)
        hist0 = rng.integers(0, 256, (nl, H, W)).astype(np.uint8)
        cfg = pass_config(4, 2, L.HY_RNG_DECORRELATED, frame, L.HY_FLAG_GGX_REFLECTION)
        v0 = dict(scene=0, planes=[torch.from_numpy(x).cuda() for x in planes_np], camera=cam, config=cfg,
                  hist=torch.from_numpy(hist0.copy()).cuda(), out_f=torch.zeros((H, W, 4), device="cuda"),
                  out_8=torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda"))
        gcam = glass.camera(2.0)
        v1 = dict(scene=1, planes=other.gbuffer(gcam, 40, 24), camera=gcam,
                  config=pass_config(2, 8, L.HY_RNG_DECORRELATED, 2),
                  hist=torch.zeros((len(glass.scene.lights), 24, 40), dtype=torch.uint8, device="cuda"),
                  out_f=torch.zeros((24, 40, 4), device="cuda"),
                  out_8=torch.zeros((24, 40, 4), dtype=torch.uint8, device="cuda"))
        torch.cuda.synchronize()
        st = runner.batch_forward([p.ctx, other], [v0, v1], tuning=pass_config(1, block_size=256, stack_depth=8))
        torch.cuda.synchronize()
        hist_o = hist0.copy()
        ocfg = po.cfg_dict(4, 2, L.HY_RNG_DECORRELATED, frame, L.HY_FLAG_GGX_REFLECTION)
        of, o8, osh, ost = p.orc.forward(planes_np, cam, ocfg, hist_o, L.HY_ACCUM_U8)
        hg = v0["hist"].cpu().numpy()
        of_g = p.orc.shade(planes_np, cam, ocfg, np.ascontiguousarray(hg), L.HY_ACCUM_U8)[0]
        g = (v0["out_f"].cpu().numpy(), v0["out_8"].cpu().numpy(), hg,
             dict(st, shadow_rays=ost["shadow_rays"], reflection_rays=ost["reflection_rays"]))
        check_parity(g, (of, o8, hist_o, osh, ost, of_g), L.HY_ACCUM_U8)
        assert st["error_flags"] == 0
    finally:
        other.close()
        runner.close()
        p.ctx.close()
