"""The FP64 gradient oracle on the CPU: its FP64 image equals the float
shading pass, and its forward-mode adjoint equals FP64 central finite
differences of the same function (visibility and light sides fixed)."""
import numpy as np
import pytest

from vulkanhybridraytracer_gb300 import diffrender, scenes


def _setup(oracle_lib, wl, spp=4):
    sc = oracle_lib.OracleScene()
    sc.set_scene(wl.scene)
    sc.build_bvh()
    cam = wl.camera(0.0)
    planes = sc.gbuffer(cam, wl.width, wl.height)
    cfg = oracle_lib.cfg_dict(spp=spp, max_bounces=wl.max_bounces, rng_mode=1)
    shadow, _ = sc.shadow_pass(planes, cam, cfg, 1)
    g = oracle_lib.GradOracle(sc, planes, cam, cfg, shadow, 1)
    _, _, _, _, mats, lights = wl.scene.pack()
    mp = diffrender.material_params(mats).astype(np.float64)
    lp = diffrender.light_params(lights).astype(np.float64)
    return sc, planes, cam, cfg, shadow, g, mp, lp


def _wl(which, w, h):
    if which == "diff":
        return scenes.diff(3, w, h)
    if which == "glass":
        return scenes.small_glass(w, h)
    return scenes.small_textured(w, h)


@pytest.mark.parametrize("which", ["diff", "glass", "textured"])
def test_fp64_forward_matches_float_pass(oracle_lib, which):
    wl = _wl(which, 40, 40)
    sc, planes, cam, cfg, shadow, g, mp, lp = _setup(oracle_lib, wl)
    img64 = g.forward(mp, lp)
    out_f, _, _ = sc.shade(planes, cam, cfg, shadow, 1)
    ref = out_f[..., :3].astype(np.float64)
    err = np.abs(img64 - ref)
    assert np.sqrt((err ** 2).mean()) <= 1e-5 * max(1.0, np.sqrt((ref ** 2).mean()))
    assert err.max() <= 1e-3 * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("which", ["diff", "glass", "textured"])
def test_fp64_adjoint_matches_central_differences(oracle_lib, which):
    wl = _wl(which, 32, 32)
    sc, planes, cam, cfg, shadow, g, mp, lp = _setup(oracle_lib, wl)
    rng = np.random.default_rng(7)
    w = rng.normal(size=(wl.height, wl.width, 3))
    gm, gl = g.adjoint(mp, lp, w)
    flat = np.concatenate([gm.ravel(), gl.ravel()])
    scale = np.abs(flat).max()
    assert scale > 0
    cand = np.flatnonzero(np.abs(flat) > 1e-3 * scale)
    pick = rng.choice(cand, size=min(24, len(cand)), replace=False)
    h = 1e-4
    nm = mp.size
    for j in pick:
        def f(delta):
            m2, l2 = mp.copy(), lp.copy()
            if j < nm:
                m2.ravel()[j] += delta
            else:
                l2.ravel()[j - nm] += delta
            return float((w * g.forward(m2, l2)).sum())
        fd = (f(h) - f(-h)) / (2 * h)
        assert abs(fd - flat[j]) <= 1e-5 * max(abs(fd), 1e-2 * scale), (int(j), fd, flat[j])
