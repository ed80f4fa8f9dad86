"""CPU tests of the oracle: golden RNG vectors, BRDF point values, BVH
correctness against brute force, and hand-derived cases of the reference
shaders' behaviour (each citing the shader lines it exercises)."""
import json
from pathlib import Path

import numpy as np
import pytest

import pyoracle as po
from vulkanhybridraytracer_gb300 import scenes
from vulkanhybridraytracer_gb300.scene import (DIRECTIONAL_LIGHT, POINT_LIGHT, Camera, Light, Material, Object,
                                               Scene)

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.fixture(scope="module")
def kat():
    return json.loads((GOLD / "rng_kat.json").read_text())


def test_tea_golden(oracle_lib, kat):
    W = kat["width"]
    for frame, seeds in kat["frames"].items():
        for e in seeds:
            assert po.tea((e["y"] * W + e["x"]) & 0xFFFFFFFF, int(frame) & 0xFFFFFFFF) == e["seed"]


def test_rnd_golden_and_grid(oracle_lib, kat):
    for s, d in kat["rnd"].items():
        st, v = po.rnd_seq(int(s), len(d["states"]))
        assert st.tolist() == d["states"]
        assert np.array_equal(v, np.array(d["values"], np.float32))
        # rnd() is exact: a 24-bit integer over 2^24 (random.glsl:30-33)
        assert np.all(v * (1 << 24) == np.floor(v * (1 << 24))) and np.all((v >= 0) & (v < 1))


def test_lcg_two_step_maps_restated(oracle_lib):
    """The shadow kernels start sample k of a pixel-light 2k LCG steps after its
    first state (two draws per sample, random.glsl:21-33) with the map
    x -> a_k x + c_k (mod 2^32) of 2k steps, read from a table for k < 64.  The
    table's recurrence, restated here, gives the states of the sequential
    generator for every k."""
    M = 1 << 32
    A, C = 1664525, 1013904223
    A2, C2 = (A * A) % M, ((A + 1) * C) % M  # two steps: x -> A (A x + C) + C
    a, c, maps = 1, 0, []
    for _ in range(64):
        maps.append((a, c))
        a, c = (A2 * a) % M, (A2 * c + C2) % M
    rng = np.random.default_rng(4)
    for seed in rng.integers(0, M, 8, dtype=np.uint64).tolist():
        st, _ = po.rnd_seq(int(seed), 2 * 63)
        for k in range(1, 64):
            ak, ck = maps[k]
            assert (ak * seed + ck) % M == int(st[2 * k - 1])
    assert maps[0] == (1, 0)


def test_sample_disk_by_value_seed(oracle_lib):
    """helpers.glsl:82-93 takes the seed by value: the same seed gives the same
    direction however many times it is called (all samples of a pixel agree)."""
    pos, L = np.array([1, 2, 3], np.float32), np.array([0.6, 0.8, 0], np.float32)
    a = po.sample_disk(0.5, pos, L, 12345)
    b = po.sample_disk(0.5, pos, L, 12345)
    assert np.array_equal(a, b)
    assert abs(np.linalg.norm(a) - 1) < 1e-6
    # the disk of radius r sits at unit distance: the angle to L is at most atan(r)
    ang = np.arccos(np.clip(a @ L / np.linalg.norm(L), -1, 1))
    assert ang <= np.arctan(0.5) + 1e-6
    # L == (0,1,0) takes the tangent special case (helpers.glsl:88-89) and stays finite
    up = po.sample_disk(0.5, pos, np.array([0, 1, 0], np.float32), 7)
    assert np.all(np.isfinite(up))


def test_brdf_point_values(oracle_lib):
    rng = np.random.default_rng(0)
    PI = np.float64(np.float32(3.14159265359))
    for _ in range(50):
        N = rng.normal(size=3); N /= np.linalg.norm(N)
        V = rng.normal(size=3); V /= np.linalg.norm(V)
        L = rng.normal(size=3); L /= np.linalg.norm(L)
        r = rng.uniform(0.05, 1)
        F0 = rng.uniform(0, 1, 3)
        c = rng.uniform(0, 1)
        got = po.brdf(N, V, L, r, F0, c)
        H = (V + L) / np.linalg.norm(V + L)
        a2 = (r * r) ** 2
        nh = max(N @ H, 0)
        D = a2 / (PI * (nh * nh * (a2 - 1) + 1) ** 2)
        k = (r + 1) ** 2 / 8
        g = lambda x: x / (x * (1 - k) + k)
        G = g(max(N @ V, 0)) * g(max(N @ L, 0))
        F = F0 + (1 - F0) * (1 - c) ** 5
        np.testing.assert_allclose(got, [D, G, *F], rtol=2e-4, atol=1e-6)


def _rays(rng, n, lo=-6, hi=6):
    org = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    org[:, 1] = rng.uniform(0.1, 4, n)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3], r[:, 3], r[:, 4:7], r[:, 7] = org, 0.001, d, 1000.0
    return r


@pytest.fixture(scope="module")
def small_orc(oracle_lib):
    wl = scenes.small(0, 64, 64)
    o = po.OracleScene()
    o.set_scene(wl.scene)
    info = o.build_bvh()
    return wl, o, info


@pytest.fixture(scope="module")
def lbvh_orc(oracle_lib):
    wl = scenes.small(0, 64, 64)
    o = po.OracleScene()
    o.set_scene(wl.scene)
    o.set_build_mode(po.HY_BUILD_LBVH)
    info = o.build_bvh()
    return wl, o, info


def test_bvh8_matches_brute_force(small_orc):
    wl, o, _ = small_orc
    rays = _rays(np.random.default_rng(2), 4000)
    hb, _ = o.trace(rays, False, po.TRACE_BRUTE)
    hv, cnt = o.trace(rays, False, po.TRACE_BVH8)
    assert np.array_equal(hb.view(np.uint32)[:, 1], hv.view(np.uint32)[:, 1])
    assert np.array_equal(hb.view(np.uint32), hv.view(np.uint32))
    ab, _ = o.trace(rays, True, po.TRACE_BRUTE)
    av, _ = o.trace(rays, True, po.TRACE_BVH8)
    assert np.array_equal(ab.view(np.uint32)[:, 1] != 0xFFFFFFFF, av.view(np.uint32)[:, 1] != 0xFFFFFFFF)
    assert cnt[:, 0].mean() < 40  # the 8-wide tree prunes: far fewer tests than 5122 triangles


def test_anyhit_orders_agree(oracle_lib):
    """Far-first and near-first any-hit traversal: the same occlusion for every
    ray (and brute force's), the same closest hits; the order only changes
    which nodes are visited.  Rays from the floor towards points above it,
    like shadow rays, meet their occluders sooner far first (on this scene's
    LBVH; the SAH structure's case is in test_sah.py)."""
    wl = scenes.small(0, 64, 64)
    o = po.OracleScene()
    o.set_scene(wl.scene)
    o.set_build_mode(po.HY_BUILD_LBVH)
    o.build_bvh()
    rng = np.random.default_rng(5)
    n = 4000
    rays = np.zeros((n, 8), np.float32)
    org = np.stack([rng.uniform(-6, 6, n), np.full(n, 0.01), rng.uniform(-6, 6, n)], 1)
    tgt = np.stack([rng.uniform(-6, 6, n), rng.uniform(4, 8, n), rng.uniform(-6, 6, n)], 1)
    d = tgt - org
    dist = np.linalg.norm(d, axis=1)
    rays[:, 0:3], rays[:, 4:7], rays[:, 3], rays[:, 7] = org, d / dist[:, None], 1e-3, dist
    ab, _ = o.trace(rays, True, po.TRACE_BRUTE)
    res = {}
    for order in (po.HY_ANYHIT_FAR_FIRST, po.HY_ANYHIT_NEAR_FIRST):
        o.set_anyhit_order(order)
        a, ca = o.trace(rays, True)
        c, _ = o.trace(rays, False)
        res[order] = (a.view(np.uint32)[:, 1] != 0xFFFFFFFF, c.view(np.uint32), ca[:, 0].sum())
    far, near = res[po.HY_ANYHIT_FAR_FIRST], res[po.HY_ANYHIT_NEAR_FIRST]
    assert np.array_equal(far[0], near[0])
    assert np.array_equal(far[0], ab.view(np.uint32)[:, 1] != 0xFFFFFFFF)
    assert far[0].any() and not far[0].all()
    assert np.array_equal(far[1], near[1])
    assert far[2] < near[2]
    o.set_anyhit_order(po.HY_ANYHIT_AUTO)
    a, _ = o.trace(rays, True)
    assert np.array_equal(a.view(np.uint32)[:, 1] != 0xFFFFFFFF, far[0])


def test_bvh_structure(lbvh_orc):
    wl, o, info = lbvh_orc
    n = info["num_tris"]
    morton, order, bvh2, bvh8, tris = o.download_bvh(info["num_bvh8_nodes"])
    assert np.all(np.diff(morton.astype(np.int64)) >= 0)
    assert sorted(order.tolist()) == list(range(n))
    # stable: equal codes keep triangle order
    eq = morton[1:] == morton[:-1]
    assert np.all(order[1:][eq] > order[:-1][eq])
    # every triangle appears exactly once in the packed array, with its world vertices
    ids = tris[:, 3].view(np.uint32)
    assert sorted(ids.tolist()) == list(range(n))
    world = o.world_tris()
    assert np.array_equal(tris[:, [0, 1, 2, 4, 5, 6, 8, 9, 10]], world[ids])
    # Karras ranges: the root covers [0, n-1]; children partition their parent
    assert bvh2[0, 2] == 0 and bvh2[0, 3] == n - 1
    for i in range(n - 1):
        l, r, f, la = bvh2[i, :4]
        lr = (l & 0x7FFFFFFF, l & 0x7FFFFFFF) if l & 0x80000000 else (bvh2[l, 2], bvh2[l, 3])
        rr = (r & 0x7FFFFFFF, r & 0x7FFFFFFF) if r & 0x80000000 else (bvh2[r, 2], bvh2[r, 3])
        assert lr[0] == f and rr[1] == la and lr[1] + 1 == rr[0]


def test_morton_restatement(lbvh_orc):
    """Morton codes recomputed in numpy float32 (one rounding per op) equal the oracle's."""
    wl, o, info = lbvh_orc
    w = o.world_tris().reshape(-1, 3, 3)
    lo, hi = w.min(1), w.max(1)
    c = ((lo + hi) * np.float32(0.5)).astype(np.float32)
    slo, shi = c.min(0), c.max(0)
    inv = (np.float32(1024.0) / (shi - slo)).astype(np.float32)
    q = np.clip(((c - slo).astype(np.float32) * inv).astype(np.float32), 0, 1023).astype(np.uint32)

    def expand(v):
        v = v & 0x3FF
        v = (v | (v << 16)) & 0x030000FF
        v = (v | (v << 8)) & 0x0300F00F
        v = (v | (v << 4)) & 0x030C30C3
        v = (v | (v << 2)) & 0x09249249
        return v
    code = (expand(q[:, 0]) << 2) | (expand(q[:, 1]) << 1) | expand(q[:, 2])
    morton, order, *_ = o.download_bvh(info["num_bvh8_nodes"])
    assert np.array_equal(np.sort(code, kind="stable"), morton)
    assert np.array_equal(np.argsort(code, kind="stable").astype(np.uint32), order)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 9, 33])
def test_tiny_scenes_exhaustive(oracle_lib, n):
    """1-33 triangles, including duplicates (equal Morton codes): BVH8 == brute force."""
    rng = np.random.default_rng(n)
    v = np.zeros((3 * n, 11), np.float32)
    base = rng.uniform(-1, 1, (n, 3))
    base[n // 2:] = base[0]  # duplicated positions
    for t in range(n):
        for k in range(3):
            v[3 * t + k, 0:3] = base[t] + rng.uniform(-0.5, 0.5, 3)
            v[3 * t + k, 4] = 1
    idx = np.arange(3 * n, dtype=np.uint32)
    prims = np.array([[0, 3 * n, 0, 0, 0, 0]], np.uint32)
    xf = np.eye(4, dtype=np.float32).reshape(1, 16)
    mats = Material().to_shader(0)[None]
    o = po.OracleScene()
    o.set_scene_arrays(v, idx, prims, xf, mats, np.zeros((0, 12), np.float32))
    o.build_bvh()
    rays = _rays(rng, 2000, -2, 2)
    rays[:, 1] = rng.uniform(-2, 2, len(rays))
    hb, _ = o.trace(rays, False, po.TRACE_BRUTE)
    hv, _ = o.trace(rays, False, po.TRACE_BVH8)
    assert np.array_equal(hb.view(np.uint32), hv.view(np.uint32))


# ---- hand-derived cases of the shaders --------------------------------------------------
def _plane_scene(mode=0, light=None, metallic=0.0, rough=0.5, ior=1.5, extra_quad=None):
    from vulkanhybridraytracer_gb300.scenes import quad, trs
    sc = Scene()
    sc.entities.append(Object(quad(20.0), 0, trs()))
    if extra_quad is not None:
        sc.entities.append(Object(quad(2.0), 1, trs(extra_quad)))
    sc.materials = [Material(mode, (0.5, 0.6, 0.7, 1), metallic, rough, ior), Material(0, (0.9, 0.9, 0.9, 1), 0, 1)]
    sc.lights = light or [Light(POINT_LIGHT, (1, 1, 1), (0, 5, 0), 20.0, 500.0, 0.1)]
    sc.camera = Camera((0, 3, 6), (0, 0, 0), 60)
    sc.env = [np.full((8, 16, 4), 200, np.uint8), np.full((8, 16, 4), 100, np.uint8)]
    return sc


def _run(sc, W=16, H=16, cfg=None, fmt=1):
    o = po.OracleScene()
    o.set_scene(sc)
    o.build_bvh()
    cam = sc.camera.rt_camera(W, H, 0)
    gb = o.gbuffer(cam, W, H)
    cfg = cfg or po.cfg_dict(spp=1, max_bounces=8, accum_frame=1, flags=2)
    hist = np.zeros((len(sc.lights), H, W), np.float32 if fmt else np.uint8)
    f, b8, sh, st = o.forward(gb, cam, cfg, hist, fmt)
    return o, gb, f, sh, st


def test_directional_light_never_traced(oracle_lib):
    """pos.w = -1: light_distance < -1 is false, so shadowRaygen.rgen:70-83 never
    traces and counts the sample as lit, even under an occluder."""
    sc = _plane_scene(light=[Light(DIRECTIONAL_LIGHT, (1, 1, 1), (0, 1, 0), 1, 500, 0.1)], extra_quad=(0, 1, 0))
    _, gb, f, sh, st = _run(sc)
    fg = gb[1][..., 3] > 0
    assert st["shadow_rays"] == 0
    assert np.all(sh[0][fg] == 1.0)


def test_point_light_occluded(oracle_lib):
    sc = _plane_scene(extra_quad=(0, 2.5, 0))
    o, gb, f, sh, st = _run(sc, 32, 32)
    assert st["shadow_rays"] > 0
    assert (sh[0] == 0).any() and (sh[0] == 1).any()


def test_glass_pixels_store_one(oracle_lib):
    """shadowRaygen.rgen:43-50: mode 4 stores 1 for every light, no rays."""
    sc = _plane_scene(mode=4, extra_quad=(0, 2.5, 0))
    sc.materials[1] = Material(4, (1, 1, 1, 1), 1, 0, 1.5)
    _, gb, f, sh, st = _run(sc)
    fg = gb[1][..., 3] > 0
    assert np.all(sh[0][fg] == 1.0) and st["shadow_rays"] == 0


def test_background_passthrough(oracle_lib):
    """hybridRaygen.rgen:182-183: background texels output albedo = pow(0, 2.2) = 0."""
    sc = _plane_scene()
    sc.camera = Camera((0, 3, 6), (0, 8, 6.5), 60)  # looking up at the sky
    _, gb, f, sh, st = _run(sc)
    bg = (gb[0][..., 3] == 0) & (gb[1][..., 3] == 0)
    assert bg.any()
    assert np.all(f[bg][:, :3] == 0) and np.all(f[bg][:, 3] == 1)


def test_mirror_bounce_direction(oracle_lib):
    """A mirror floor (mode 3) reflects the camera ray: the bounce is traced and
    its miss colour (sky) multiplies the direct term (hybridRaygen.rgen:151-170)."""
    sc = _plane_scene(mode=3, metallic=1.0, rough=0.1)
    o, gb, f, sh, st = _run(sc)
    assert st["reflection_rays"] > 0
    fg = gb[1][..., 3] > 0
    assert np.isfinite(f).all() and (f[fg][:, :3] > 0).any()


def test_hit_shadow_factor_one_or_two(oracle_lib):
    """hybridHit.rchit:291-331: the factor starts at 1 and the single shadow
    ray adds 1 when unoccluded, so direct light at a hit is doubled."""
    sc = _plane_scene(mode=3, metallic=1.0, rough=0.1, extra_quad=(0, 0.5, -2))
    o, gb, f, sh, st = _run(sc, 32, 32)
    assert st["hit_shadow_rays"] > 0


def test_blur_truncated_dispatch(oracle_lib):
    """blur.comp dispatch W/16 x H/16 (src/renderer.cpp:2672) leaves the last
    W%16 columns and H%16 rows untouched; the full-dispatch flag covers them."""
    W, H = 40, 24
    planes = [np.zeros((H, W, 4), np.float32) for _ in range(6)]
    planes[3] = np.full((H, W, 2), 0.5, np.float32)
    o = po.OracleScene()
    shadow = np.full((1, H, W), 200, np.uint8)
    hist = np.full((1, H, W), 10, np.uint8)
    o.accumulate(planes, po.cfg_dict(accum_frame=3), shadow, hist, 0)
    assert np.all(hist[0, :16, :32] != 10) and np.all(hist[0, 16:, :] == 10) and np.all(hist[0, :, 32:] == 10)
    hist2 = np.full((1, H, W), 10, np.uint8)
    o.accumulate(planes, po.cfg_dict(accum_frame=3, flags=1), shadow, hist2, 0)
    assert np.all(hist2 != 10)
    # running mean: mix(old, new, 1/(frame+1)) on the R8 values
    v = np.uint8(np.rint(np.clip((10 / 255) * (1 - 0.25) + (200 / 255) * 0.25, 0, 1) * 255))
    assert hist[0, 0, 0] == v


def test_blur_reset_clamp(oracle_lib):
    """frame <= 0: history clamped to the 3x3 min/max of the new image, then
    mix(old, new, 0.4) (blur.comp:49-80)."""
    W, H = 32, 16
    planes = [np.zeros((H, W, 4), np.float32) for _ in range(6)]
    planes[3] = np.full((H, W, 2), 0.5, np.float32)  # zero motion
    shadow = np.full((1, H, W), 100, np.uint8)
    hist = np.full((1, H, W), 250, np.uint8)
    po.OracleScene().accumulate(planes, po.cfg_dict(accum_frame=0), shadow, hist, 0)
    # interior: old clamped to 100, mix -> 100;  border: neighbours outside read 0 so min = 0, max = 100
    assert hist[0, 5, 5] == 100


def test_stale_attenuation_carry(oracle_lib):
    """hybridRaygen.rgen:86-99: attenuation is only updated when NdotL > 0, so a
    glass pixel (mode 4, which uses it regardless) carries the previous light's
    value into a light behind the surface."""
    lights = [Light(POINT_LIGHT, (1, 1, 1), (0, 5, 0), 20.0, 10.0, 0.1),
              Light(POINT_LIGHT, (1, 0, 0), (0, -5, 0), 20.0, 500.0, 0.1)]
    # no bounce: the refraction ray's colour would multiply the whole direct term
    cfg = po.cfg_dict(spp=1, max_bounces=0, accum_frame=1, flags=2)
    _, gb, f, sh, st = _run(_plane_scene(mode=4, light=lights, metallic=1.0), cfg=cfg)
    fg = gb[1][..., 3] > 0
    # light 2 is below the floor: NdotL = 0, its term uses light 1's attenuation
    P = gb[0][fg][:, :3].astype(np.float64)
    d2 = np.linalg.norm(np.array([0, -5, 0]) - P, axis=1)
    d1 = np.linalg.norm(np.array([0, 5, 0]) - P, axis=1)
    att1 = ((10 - d1) / 10).clip(0) ** 2
    alb = np.array([0.5, 0.6, 0.7]) ** 2.2
    I2 = 20.0 / d2 ** 2
    # the same render with light 2 black isolates light 2's term (ambient cancels)
    lights_b = [lights[0], Light(POINT_LIGHT, (0, 0, 0), (0, -5, 0), 20.0, 500.0, 0.1)]
    _, _, fb, _, _ = _run(_plane_scene(mode=4, light=lights_b, metallic=1.0), cfg=cfg)
    diff_r = (f[fg][:, 0] - fb[fg][:, 0]).astype(np.float64)
    assert (att1 > 0).any() and (att1 == 0).any()
    np.testing.assert_allclose(diff_r, I2 * att1 * alb[0], rtol=2e-3, atol=1e-6)


def _reflect(i, n):
    return i - 2.0 * np.dot(n, i) * n


def test_ggx_reflect_mirror_limit_and_precision(oracle_lib):
    """HY_FLAG_GGX_REFLECTION's direction: roughness 0 is the reference's mirror
    reflect(-V, N) (hybridRaygen.rgen:125); the FP32 and FP64 restatements
    agree; the direction never leaves below the surface."""
    rng = np.random.default_rng(4)
    for _ in range(300):
        n = rng.normal(size=3)
        n /= np.linalg.norm(n)
        v = rng.normal(size=3)
        v /= np.linalg.norm(v)
        if np.dot(v, n) < 0.05:
            v = v - 2 * np.dot(v, n) * n + 0.1 * n
            v /= np.linalg.norm(v)
        rough = rng.uniform(0, 0.3)
        u1, u2 = (rng.integers(0, 1 << 24, 2) / float(1 << 24)).tolist()   # rnd()'s 2^-24 grid
        d32 = po.ggx_reflect(n, v, rough, u1, u2)
        d64 = po.ggx_reflect(n, v, rough, u1, u2, double=True)
        assert np.dot(d32, n.astype(np.float32)) > 0
        if abs(np.dot(d64, n)) > 1e-3:   # away from the fallback switch
            assert np.abs(d32 - d64).max() <= 2e-5
        m = po.ggx_reflect(n, v, 0.0, u1, u2, double=True)
        np.testing.assert_allclose(m, _reflect(-v, n), atol=2e-6)


@pytest.mark.parametrize("rough", [0.1, 0.2])
def test_ggx_lobe_matches_reference_distribution(oracle_lib, rough):
    """The sampled microfacet normals follow D(H) (N.H) for the reference's
    DistributionGGX (helpers.glsl:33-45, alpha = roughness^2): moments of N.H over
    a stratified 200 x 200 grid of (u1, u2) equal the integrals of the same
    moments against D(H) (N.H) on the hemisphere (normal incidence, where the
    half vector of (V, direction) is the sampled H)."""
    n = np.array([0.0, 1.0, 0.0])
    grid = (np.arange(200) + 0.5) / 200
    hs = []
    for u1 in grid[::5]:
        for u2 in grid:
            d = po.ggx_reflect(n, n, rough, u1, u2, double=True).astype(np.float64)
            h = d + n
            hs.append(h / np.linalg.norm(h))
    c = np.array(hs)[:, 1]
    a2 = (rough * rough) ** 2
    th = np.linspace(0, np.pi / 2, 400001)
    ct = np.cos(th)
    D = a2 / (np.pi * (ct * ct * (a2 - 1) + 1) ** 2)          # DistributionGGX
    w = D * ct * np.sin(th) * 2 * np.pi                       # D(H) (N.H) dw over the azimuth
    assert abs(np.trapezoid(w, th) - 1.0) < 1e-3               # a probability density
    for k in (1, 2, 4):
        want = np.trapezoid(w * ct ** k, th)
        assert abs(np.mean(c ** k) - want) < 2e-3 * want, (k, np.mean(c ** k), want)
