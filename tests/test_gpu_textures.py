"""Material textures on the GPU (hy_scene_set_textures): the G-buffer producer
against the oracle, the hybrid and path-traced shading against the
reference's own shader output on the textured workload
(tests/golden/ref_textured_small.npz), the adjoint against the FP64 CPU
adjoint, and the validation of texture ids."""
from pathlib import Path

import numpy as np
import pytest

from vulkanhybridraytracer_gb300 import _lib as L
from vulkanhybridraytracer_gb300 import scenes

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def tex(gpu_lib, oracle_lib):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import HybridContext
    fx = dict(np.load(GOLD / "ref_textured_small.npz"))
    wl = scenes.small_textured(48, 40)
    ctx = HybridContext(0)
    ctx.set_scene(wl.scene)
    ctx.build_bvh()
    o = oracle_lib.OracleScene()
    o.set_scene(wl.scene)
    o.build_bvh()
    planes = [torch.from_numpy(np.ascontiguousarray(fx[f"plane{i}"])).cuda() for i in range(6)]
    torch.cuda.synchronize()
    yield ctx, o, fx, wl, planes
    ctx.close()


def test_textured_gbuffer_matches_oracle(tex):
    ctx, o, fx, wl, _ = tex
    cam = wl.camera(1.0)
    g = [p.cpu().numpy() for p in ctx.gbuffer(cam, wl.width, wl.height)]
    r = o.gbuffer(cam, wl.width, wl.height)
    for i in (0, 2, 3, 4, 5):
        assert np.array_equal(g[i], r[i]), f"plane {i}"
    np.testing.assert_allclose(g[1], r[1], atol=2e-6)
    assert g[5][..., :3].max() > 0  # emissive texels


def test_textured_shade_vs_reference(tex):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    ctx, o, fx, wl, planes = tex
    hist = torch.from_numpy(np.ascontiguousarray(fx["shadow_spp2"])).cuda()
    out = torch.zeros((wl.height, wl.width, 4), device="cuda")
    torch.cuda.synchronize()
    st = ctx.shade_pass(planes, fx["camera"], pass_config(2, 8, L.HY_RNG_REFERENCE, 3), hist, L.HY_ACCUM_U8,
                        out_f=out)
    ref = fx["hybrid_rgba"][..., :3].astype(np.float64)
    got = out.cpu().numpy()[..., :3].astype(np.float64)
    err = np.abs(got - ref)
    assert st["reflection_rays"] > 0
    assert np.sqrt((err ** 2).sum() / (ref ** 2).sum()) <= 1e-3
    assert np.mean(err.max(-1) > 1e-2) <= 2e-3


def test_textured_pathtrace_vs_reference(tex):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    ctx, o, fx, wl, _ = tex
    img = torch.zeros((wl.height, wl.width, 4), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    for f in (0, 2):
        img, _ = ctx.pathtrace(fx[f"pt_camera_f{f}"], wl.width, wl.height, pass_config(2, 8, L.HY_RNG_REFERENCE),
                               img)
        d = np.abs(img.cpu().numpy().astype(int) - fx[f"pt_image_f{f}"].astype(int)).max(-1)
        assert np.mean(d > 0) <= 5e-3 and np.mean(d > 2) <= 1e-3, f


def test_textured_backward_vs_fp64_adjoint(gpu_lib, oracle_lib):
    import torch
    from vulkanhybridraytracer_gb300 import diffrender
    wl = scenes.small_textured(64, 48)
    r = diffrender.DiffRenderer(wl.scene, wl.camera(0.0), wl.width, wl.height, spp=4, max_bounces=wl.max_bounces)
    try:
        mp0, lp0 = r.params0
        img, state = r.render(mp0, lp0)
        rng = np.random.default_rng(3)
        w = torch.from_numpy(rng.normal(size=(wl.height, wl.width, 4)).astype(np.float32)).cuda()
        w[..., 3] = 0
        gm, gl, _ = r.backward(state, w)
        torch.cuda.synchronize()
        planes, shadow = state
        sc = oracle_lib.OracleScene()
        sc.set_scene(wl.scene)
        sc.build_bvh()
        go = oracle_lib.GradOracle(sc, [p.cpu().numpy() for p in planes], wl.camera(0.0),
                                   oracle_lib.cfg_dict(spp=4, max_bounces=wl.max_bounces, rng_mode=1),
                                   shadow.cpu().numpy(), 1)
        gm64, gl64 = go.adjoint(mp0.astype(np.float64), lp0.astype(np.float64),
                                w.cpu().numpy()[..., :3].astype(np.float64))
        g64 = np.concatenate([gm64.ravel(), gl64.ravel()])
        g = np.concatenate([gm.cpu().numpy().ravel(), gl.cpu().numpy().ravel()]).astype(np.float64)
        scale = np.abs(g64).max()
        rel = np.abs(g - g64) / np.maximum(np.abs(g64), 1e-2 * scale)
        assert rel.max() <= 1e-3, (int(np.argmax(rel)), g[np.argmax(rel)], g64[np.argmax(rel)])
        # material 0's diffuse comes from a texture: no gradient to its diffuse colour
        assert np.all(gm.cpu().numpy()[0, :3] == 0)
    finally:
        r.close()


def test_missing_texture_is_rejected(gpu_lib):
    from vulkanhybridraytracer_gb300.hybrid import HybridContext, pass_config
    wl = scenes.small_textured(16, 16)
    ctx = HybridContext(0)
    try:
        ctx.set_scene(wl.scene)
        ctx.build_bvh()
        ctx.set_textures(wl.scene.textures[:1])  # materials name textures 1 and 2 too
        with pytest.raises(L.HyError) as e:
            ctx.pathtrace(wl.camera(0.0), 16, 16, pass_config(1, 2))
        assert e.value.code == L.HY_ERR_INVALID_ARG
        ctx.set_textures(wl.scene.textures)
        ctx.pathtrace(wl.camera(0.0), 16, 16, pass_config(1, 2))
    finally:
        ctx.close()
