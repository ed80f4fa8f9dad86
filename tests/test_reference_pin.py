"""The oracle against the reference's own shader code.

tests/golden/ref_kat.json and ref_pass_small.npz hold outputs of the
reference's helpers.glsl / shadowRaygen.rgen / blur.comp / hybridRaygen.rgen
+ hybridHit.rchit + miss.rmiss + shadow.rmiss, compiled as C++ from the
reference checkout (oracle/glsl_ref) and generated by
tests/golden/make_golden.py.  The oracle must reproduce them bit for bit.
Where the reference checkout is present the pin is also re-run live on
fresh random inputs."""
import json
from pathlib import Path

import numpy as np
import pytest

import pyoracle as po
from vulkanhybridraytracer_gb300 import scenes

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def fx():
    return dict(np.load(GOLD / "ref_pass_small.npz"))


@pytest.fixture(scope="module")
def glass_orc(oracle_lib):
    wl = scenes.small_glass()
    o = po.OracleScene()
    o.set_scene(wl.scene)
    o.build_bvh()
    return wl, o


def test_kat_sample_disk_and_brdf(oracle_lib):
    kat = json.loads((GOLD / "ref_kat.json").read_text())
    for e in kat["sampleDisk"]:
        got = po.sample_disk(e["radius"], np.float32(e["pos"]), np.float32(e["L"]), e["seed"])
        assert np.array_equal(got, np.float32(e["dir"])), e
    for e in kat["brdf"]:
        got = po.brdf(np.float32(e["N"]), np.float32(e["V"]), np.float32(e["L"]), e["roughness"], np.float32(e["F0"]),
                      e["cos"])
        assert np.array_equal(got, np.float32(e["D_G_F"])), e


def _planes(fx):
    return [np.ascontiguousarray(fx[f"plane{i}"]) for i in range(6)]


@pytest.mark.parametrize("mode", [po.TRACE_BRUTE, po.TRACE_BVH8])
@pytest.mark.parametrize("spp", [1, 4])
def test_shadow_pass_equals_reference(glass_orc, fx, mode, spp):
    wl, o = glass_orc
    sh, _ = o.shadow_pass(_planes(fx), fx["camera"], po.cfg_dict(spp=spp, rng_mode=0), 0, mode)
    ref = fx[f"shadow_spp{spp}"]
    if mode == po.TRACE_BRUTE:
        assert np.array_equal(sh, ref)
    else:  # BVH8 traversal: the same hits except exact ties/edges
        assert np.mean(sh != ref) <= 1e-3


def test_blur_equals_reference(oracle_lib, fx):
    o = po.OracleScene()
    m = fx["blur_motion"]
    H, W = m.shape[:2]
    planes = [np.zeros((H, W, 4), np.float32)] * 3 + [np.ascontiguousarray(m)] + [np.zeros((H, W, 4), np.float32)] * 2
    h = fx["blur_hist0"].copy()
    o.accumulate(planes, po.cfg_dict(accum_frame=0), fx["blur_in"].copy(), h, 0)
    assert np.array_equal(h, fx["blur_after_frame0"])
    o.accumulate(planes, po.cfg_dict(accum_frame=3), fx["blur_in"].copy(), h, 0)
    assert np.array_equal(h, fx["blur_after_frame3"])


@pytest.mark.parametrize("mode", [po.TRACE_BRUTE, po.TRACE_BVH8])
def test_hybrid_pass_equals_reference(glass_orc, fx, mode):
    wl, o = glass_orc
    hist = np.ascontiguousarray(fx["shadow_spp4"])
    out, _, st = o.shade(_planes(fx), fx["camera"], po.cfg_dict(spp=4, max_bounces=8, rng_mode=0), hist, 0, mode)
    ref = fx["hybrid_rgba"]
    assert st["reflection_rays"] > 0 and st["hit_shadow_rays"] > 0
    if mode == po.TRACE_BRUTE:
        assert np.array_equal(out, ref)
    else:
        err = np.abs(out[..., :3].astype(np.float64) - ref[..., :3])
        rms = np.sqrt((err ** 2).sum() / (ref[..., :3].astype(np.float64) ** 2).sum())
        assert rms <= 1e-3 and np.mean(err > 1e-2) <= 1e-3


def test_live_pin_against_reference_shaders(oracle_lib):
    """Runs the reference's shaders compiled from the checkout on a fresh frame."""
    import sys
    sys.path.insert(0, str(Path(po.__file__).resolve().parent / "glsl_ref"))
    import pyref
    if not pyref.available():
        pytest.skip("reference checkout not present")
    wl = scenes.small_glass(40, 32)
    o = po.OracleScene()
    o.set_scene(wl.scene)
    rs = pyref.RefScene(wl.scene)
    for frame in (0.0, 11.0):
        cam = wl.camera(frame)
        planes = o.gbuffer(cam, wl.width, wl.height, po.TRACE_BRUTE)
        for spp in (1, 3):
            sh, _ = o.shadow_pass(planes, cam, po.cfg_dict(spp=spp, rng_mode=0), 0, po.TRACE_BRUTE)
            assert np.array_equal(sh, rs.shadow_pass(planes, cam, spp))
        out, _, _ = o.shade(planes, cam, po.cfg_dict(spp=3, max_bounces=8, rng_mode=0), sh, 0, po.TRACE_BRUTE)
        assert np.array_equal(out, rs.hybrid_pass(planes, cam, sh))
