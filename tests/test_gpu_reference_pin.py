"""The CUDA path against outputs of the reference's own shader code
(tests/golden/ref_pass_small.npz, see tests/golden/make_golden.py), through
the C ABI.  The GPU traverses its BVH8 and uses CUDA's cosf/sinf, the fixture
came from brute-force traversal and libm: shadow decisions may differ on
exact ties/edges (<= 1e-4 of texels, the bar of every other parity test),
radiance within 1e-3 relative RMS."""
from pathlib import Path

import numpy as np
import pytest

from vulkanhybridraytracer_gb300 import _lib as L
from vulkanhybridraytracer_gb300 import scenes

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def setup(gpu_lib):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import HybridContext
    fx = dict(np.load(GOLD / "ref_pass_small.npz"))
    wl = scenes.small_glass()
    ctx = HybridContext(0)
    ctx.set_scene(wl.scene)
    ctx.build_bvh()
    planes = [torch.from_numpy(np.ascontiguousarray(fx[f"plane{i}"])).cuda() for i in range(6)]
    yield ctx, fx, planes, wl
    ctx.close()


@pytest.mark.parametrize("spp", [1, 4])
def test_gpu_shadow_pass_vs_reference(setup, spp):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    ctx, fx, planes, wl = setup
    nl, H, W = fx[f"shadow_spp{spp}"].shape
    sh = torch.zeros((nl, H, W), dtype=torch.uint8, device="cuda")
    ctx.shadow_pass(planes, fx["camera"], pass_config(spp, 8, L.HY_RNG_REFERENCE, 3), sh, L.HY_ACCUM_U8)
    assert np.mean(sh.cpu().numpy() != fx[f"shadow_spp{spp}"]) <= 1e-4


def test_gpu_shade_pass_vs_reference(setup):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    ctx, fx, planes, wl = setup
    hist = torch.from_numpy(np.ascontiguousarray(fx["shadow_spp4"])).cuda()
    out = torch.zeros((wl.height, wl.width, 4), device="cuda")
    st = ctx.shade_pass(planes, fx["camera"], pass_config(4, 8, L.HY_RNG_REFERENCE, 3), hist, L.HY_ACCUM_U8,
                        out_f=out)
    ref = fx["hybrid_rgba"]
    got = out.cpu().numpy()
    err = np.abs(got[..., :3].astype(np.float64) - ref[..., :3])
    rms = np.sqrt((err ** 2).sum() / (ref[..., :3].astype(np.float64) ** 2).sum())
    assert st["reflection_rays"] > 0
    assert rms <= 1e-3, rms
    assert err.max() <= 1e-2, err.max()


def test_gpu_blur_vs_reference(setup):
    import torch
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    ctx, fx, planes, wl = setup
    m = fx["blur_motion"]
    H, W = m.shape[:2]
    bp = [torch.zeros((H, W, 4), device="cuda") for _ in range(6)]
    bp[3] = torch.from_numpy(np.ascontiguousarray(m)).cuda()
    h = torch.from_numpy(fx["blur_hist0"].copy()).cuda()
    src = torch.from_numpy(fx["blur_in"].copy()).cuda()
    ctx.accumulate_pass(bp, pass_config(accum_frame=0), src, h, L.HY_ACCUM_U8)
    assert np.array_equal(h.cpu().numpy(), fx["blur_after_frame0"])
    ctx.accumulate_pass(bp, pass_config(accum_frame=3), src, h, L.HY_ACCUM_U8)
    assert np.array_equal(h.cpu().numpy(), fx["blur_after_frame3"])
