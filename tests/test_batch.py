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
