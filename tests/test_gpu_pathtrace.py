"""Path-traced mode (hy_pathtrace_pass) against the reference's own shader
output (tests/golden/ref_pathtrace_small.npz) and the CPU oracle, through the
C ABI.  The GPU traverses its BVH8 and uses CUDA's cosf/sinf and fused
multiply-adds in shading; the bars: the 8-bit accumulated image equal on
>= 99.5 % of pixels and within 2 levels elsewhere except a few decision
flips, the frame's float colour within 1e-3 relative RMS."""
from pathlib import Path

import numpy as np
import pytest

from vulkanhybridraytracer_gb300 import _lib as L
from vulkanhybridraytracer_gb300 import scenes

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def _ctx(wl):
    from vulkanhybridraytracer_gb300.hybrid import HybridContext
    ctx = HybridContext(0)
    ctx.set_scene(wl.scene)
    ctx.build_bvh()
    return ctx


def _img_close(got, ref, frac=5e-3):
    d = np.abs(got.astype(int) - ref.astype(int)).max(-1)
    return np.mean(d > 0) <= frac and np.mean(d > 2) <= 1e-3


def test_pathtrace_vs_reference_fixture(gpu_lib):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    fx = dict(np.load(GOLD / "ref_pathtrace_small.npz"))
    wl = scenes.small_glass()
    ctx = _ctx(wl)
    try:
        img = torch.zeros((wl.height, wl.width, 4), dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()  # the library runs on its own stream
        for f in (0, 2, 3):
            img, st = ctx.pathtrace(fx[f"camera_f{f}"], wl.width, wl.height,
                                    pass_config(2, 8, L.HY_RNG_REFERENCE), img)
            assert st["reflection_rays"] > 0 and st["shadow_rays"] > 0 and st["error_flags"] == 0
            assert _img_close(img.cpu().numpy(), fx[f"image_f{f}"]), f
    finally:
        ctx.close()


@pytest.mark.parametrize("rng", [L.HY_RNG_REFERENCE, L.HY_RNG_DECORRELATED])
@pytest.mark.parametrize("which", ["small", "glass"])
def test_pathtrace_vs_oracle(gpu_lib, oracle_lib, rng, which):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    po = oracle_lib
    wl = scenes.small(0, 96, 64) if which == "small" else scenes.small_glass(64, 48)
    ctx = _ctx(wl)
    o = po.OracleScene()
    o.set_scene(wl.scene)
    o.build_bvh()
    try:
        img = torch.zeros((wl.height, wl.width, 4), dtype=torch.uint8, device="cuda")
        out = torch.zeros((wl.height, wl.width, 4), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        img_o = np.zeros((wl.height, wl.width, 4), np.uint8)
        for frame in (-1.0, 1.0, 2.0):
            cam = wl.camera(frame)
            img, st = ctx.pathtrace(cam, wl.width, wl.height, pass_config(4, 8, rng), img, out_f=out)
            img_o, out_o, st_o = o.pathtrace(cam, wl.width, wl.height, po.cfg_dict(spp=4, max_bounces=8, rng_mode=rng),
                                             img_o)
            got = out.cpu().numpy()[..., :3].astype(np.float64)
            ref = out_o[..., :3].astype(np.float64)
            err = np.abs(got - ref)
            rms = np.sqrt((err ** 2).sum() / max((ref ** 2).sum(), 1e-30))
            assert rms <= 1e-3, (frame, rms)
            assert np.mean(err.max(-1) > 1e-2) <= 2e-3
            assert _img_close(img.cpu().numpy(), img_o), frame
            assert abs(st["shadow_rays"] - st_o["shadow_rays"]) <= 1e-3 * st_o["shadow_rays"] + 4
            assert abs(st["reflection_rays"] - st_o["reflection_rays"]) <= 1e-3 * st_o["reflection_rays"] + 4
    finally:
        ctx.close()


def test_pathtrace_store_then_mean(gpu_lib):
    """frame < 0 stores the frame's colour; frame >= 0 mixes with weight 1 / (1 + frame)."""
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    wl = scenes.small(0, 40, 24)
    ctx = _ctx(wl)
    try:
        out = torch.zeros((wl.height, wl.width, 4), dtype=torch.float32, device="cuda")
        img = torch.full((wl.height, wl.width, 4), 77, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        img, _ = ctx.pathtrace(wl.camera(-1.0), wl.width, wl.height, pass_config(1, 8), img, out_f=out)
        c = np.clip(out.cpu().numpy()[..., :3], 0, 1)
        expect = np.rint(c * 255).astype(np.uint8)[..., ::-1]  # B, G, R
        assert np.array_equal(img.cpu().numpy()[..., :3], expect)
        assert np.all(img.cpu().numpy()[..., 3] == 255)
        before = img.cpu().numpy().astype(np.float64)
        img, _ = ctx.pathtrace(wl.camera(0.0), wl.width, wl.height, pass_config(1, 8), img, out_f=out)
        # frame 0: weight 1, the image is the new frame whatever it held
        c = np.clip(out.cpu().numpy()[..., :3], 0, 1)
        assert np.abs(img.cpu().numpy()[..., :3].astype(int) - np.rint(c * 255)[..., ::-1]).max() <= 1
        assert before.shape == img.shape
    finally:
        ctx.close()


def test_post_resolve_vs_reference(gpu_lib):
    """postFragment.frag on the GPU (hy_post_resolve) against the reference's output: CUDA's
    powf and libm may round a value to the other side of an 8-bit step."""
    import torch
    from vulkanhybridraytracer_gb300.hybrid import HybridContext
    fx = dict(np.load(GOLD / "ref_post_small.npz"))
    ctx = HybridContext(0)
    try:
        img = torch.from_numpy(fx["image"]).cuda()
        f = torch.from_numpy((fx["image"][..., [2, 1, 0, 3]].astype(np.float32) / np.float32(255.0))).cuda()
        torch.cuda.synchronize()
        for src in (img, f):
            got = ctx.post(src).cpu().numpy().astype(int)
            d = np.abs(got - fx["post"].astype(int))
            assert d.max() <= 1 and np.mean(d > 0) <= 1e-2
    finally:
        ctx.close()


def test_pathtrace_argument_errors(gpu_lib):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    wl = scenes.small(0, 16, 16)
    ctx = _ctx(wl)
    try:
        with pytest.raises(L.HyError) as e:
            ctx.pathtrace(wl.camera(0.0), 0, 16, pass_config(1, 8))
        assert e.value.code == L.HY_ERR_INVALID_ARG
        bad = torch.zeros(16 * 16 * 4 + 1, dtype=torch.uint8, device="cuda")[1:]
        with pytest.raises(L.HyError) as e:
            ctx.pathtrace(wl.camera(0.0), 16, 16, pass_config(1, 8), bad)
        assert e.value.code == L.HY_ERR_INVALID_ARG
    finally:
        ctx.close()


@pytest.mark.parametrize("rng,minb", [(L.HY_RNG_REFERENCE, 0), (L.HY_RNG_DECORRELATED, 0),
                                      (L.HY_RNG_DECORRELATED, 4), (L.HY_RNG_DECORRELATED, 5)])
def test_pathtrace_tile_streams_equal_per_lane(gpu_lib, rng, minb):
    """The warp-cooperative kernel (each hit's shadow rays as tile streams, the
    default) traces the same rays as one lane per pixel (HY_FLAG_PIXEL_PARALLEL):
    equal ray counts and, up to the rounding of fused multiply-adds the compiler
    places differently in the two kernels, the same colours."""
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    wl = scenes.small_glass(64, 48)
    ctx = _ctx(wl)
    try:
        outs = []
        for flags in (0, L.HY_FLAG_PIXEL_PARALLEL):
            img = torch.zeros((wl.height, wl.width, 4), dtype=torch.uint8, device="cuda")
            out = torch.zeros((wl.height, wl.width, 4), dtype=torch.float32, device="cuda")
            torch.cuda.synchronize()
            img, st = ctx.pathtrace(wl.camera(-1.0), wl.width, wl.height,
                                    pass_config(4, 8, rng, flags=flags, min_blocks=minb), img, out_f=out)
            outs.append((img.cpu().numpy(), out.cpu().numpy(), st))
        (ia, fa, sa), (ib, fb, sb) = outs
        assert sa["shadow_rays"] == sb["shadow_rays"] > 0
        assert sa["reflection_rays"] == sb["reflection_rays"]
        assert sa["error_flags"] == 0
        np.testing.assert_allclose(fa, fb, rtol=1e-5, atol=1e-6)
        assert np.abs(ia.astype(int) - ib.astype(int)).max() <= 1
    finally:
        ctx.close()
