"""The oracle against the reference's own shader code.

tests/golden/ref_kat.json, ref_pass_small.npz and ref_pathtrace_small.npz
hold outputs of the reference's helpers.glsl / shadowRaygen.rgen / blur.comp /
hybridRaygen.rgen + hybridHit.rchit + miss.rmiss + shadow.rmiss and of its
path-traced raygen.rgen + closesthit.rchit, compiled as C++ from the
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


@pytest.mark.parametrize("mode", [po.TRACE_BRUTE, po.TRACE_BVH8])
def test_pathtrace_equals_reference(oracle_lib, mode):
    """raygen.rgen + closesthit.rchit + miss shaders: the B8G8R8A8 image after frames -1, 1, 2."""
    fx = dict(np.load(GOLD / "ref_pathtrace_small.npz"))
    wl = scenes.small_glass()
    o = po.OracleScene()
    o.set_scene(wl.scene)
    o.build_bvh()
    img = np.zeros((wl.height, wl.width, 4), np.uint8)
    for f in (0, 2, 3):
        img, _, st = o.pathtrace(fx[f"camera_f{f}"], wl.width, wl.height,
                                 po.cfg_dict(spp=2, max_bounces=8, rng_mode=0), img, mode)
        ref = fx[f"image_f{f}"]
        assert st["reflection_rays"] > 0 and st["shadow_rays"] > 0
        if mode == po.TRACE_BRUTE:
            assert np.array_equal(img, ref), f
        else:  # BVH8: the same hits except exact ties/edges
            assert np.mean(np.any(img != ref, -1)) <= 2e-3, f


def test_live_pathtrace_pin(oracle_lib):
    import sys
    sys.path.insert(0, str(Path(po.__file__).resolve().parent / "glsl_ref"))
    import pyref
    if not pyref.available():
        pytest.skip("reference checkout not present")
    wl = scenes.small(0, 40, 32)
    o = po.OracleScene()
    o.set_scene(wl.scene)
    rs = pyref.RefScene(wl.scene)
    a = np.zeros((wl.height, wl.width, 4), np.uint8)
    b = a.copy()
    for frame in (0.0, 5.0):
        cam = wl.camera(frame)
        a, _, _ = o.pathtrace(cam, wl.width, wl.height, po.cfg_dict(spp=3, max_bounces=8, rng_mode=0), a,
                              po.TRACE_BRUTE)
        b = rs.pathtrace_pass(cam, wl.width, wl.height, 3, b)
        assert np.array_equal(a, b)


def test_post_equals_reference(oracle_lib):
    """postFragment.frag: pow(max(rgb, 0.001), 1/2.2) on the 8-bit image."""
    fx = dict(np.load(GOLD / "ref_post_small.npz"))
    assert np.array_equal(po.post_resolve(fx["image"]), fx["post"])
    # the float input form equals the 8-bit one on the same values
    f = fx["image"][..., [2, 1, 0, 3]].astype(np.float32) / np.float32(255.0)
    assert np.array_equal(po.post_resolve(f), fx["post"])


@pytest.fixture(scope="module")
def tex_fx(oracle_lib):
    fx = dict(np.load(GOLD / "ref_textured_small.npz"))
    wl = scenes.small_textured(48, 40)
    o = po.OracleScene()
    o.set_scene(wl.scene)
    o.build_bvh()
    return fx, wl, o


def test_textured_gbuffer_input_is_the_oracle_producer(tex_fx):
    fx, wl, o = tex_fx
    planes = o.gbuffer(fx["camera"], wl.width, wl.height, po.TRACE_BRUTE)
    for i in range(6):
        assert np.array_equal(planes[i], fx[f"plane{i}"]), i
    # the textures show up: albedo varies within one material, emissive texels exist
    assert np.unique(planes[2][..., 0]).size > 8 and planes[5][..., :3].max() > 0


def test_textured_passes_equal_reference(tex_fx):
    """hybridHit.rchit / closesthit.rchit texture branches (hybridHit.rchit:63-65,
    closesthit.rchit:76-78) and the emissive term, on the reference's own shader code."""
    fx, wl, o = tex_fx
    planes = [np.ascontiguousarray(fx[f"plane{i}"]) for i in range(6)]
    sh, _ = o.shadow_pass(planes, fx["camera"], po.cfg_dict(spp=2, rng_mode=0), 0, po.TRACE_BRUTE)
    assert np.array_equal(sh, fx["shadow_spp2"])
    out, _, _ = o.shade(planes, fx["camera"], po.cfg_dict(spp=2, max_bounces=8, rng_mode=0), sh, 0, po.TRACE_BRUTE)
    assert np.array_equal(out, fx["hybrid_rgba"])
    img = np.zeros((wl.height, wl.width, 4), np.uint8)
    for f in (0, 2):
        img, _, _ = o.pathtrace(fx[f"pt_camera_f{f}"], wl.width, wl.height,
                                po.cfg_dict(spp=2, max_bounces=8, rng_mode=0), img, po.TRACE_BRUTE)
        assert np.array_equal(img, fx[f"pt_image_f{f}"]), f
