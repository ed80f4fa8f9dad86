"""GPU parity of libhybridrt against the CPU oracle, through the C ABI.

Integer/index outputs (Morton codes, sort order, BVH arrays, packed
triangles, hit ids, traversal counts, R8 shadow/history images) must be
bit-exact.  Radiance follows the pass's stated tolerance: relative RMS
<= 1e-3 and per-pixel max |err| <= 1e-2 on pixels whose shadow decisions
agree; decisions may differ on at most 1e-4 of the shadow texels (a shadow
ray direction built from cosf/sinf can differ by an ulp between CUDA and
libm and graze an edge differently).  Texels whose decision flipped are not
exempt: the oracle also shades the frame from the GPU's own shadow history,
and the GPU image must match that within 1e-2 per pixel everywhere, so a
flip may change a pixel by exactly the flipped samples' share of their
light and no more.
"""
import numpy as np
import pytest

import pyoracle as po
from vulkanhybridraytracer_gb300 import _lib as L
from vulkanhybridraytracer_gb300 import scenes
from vulkanhybridraytracer_gb300.scene import Material

pytestmark = pytest.mark.gpu

RMS_TOL, MAX_TOL, FLIP_TOL = 1e-3, 1e-2, 1e-4


def _torch():
    import torch
    return torch


class Pair:
    """The same scene in the GPU context and in the oracle."""

    def __init__(self, wl, build=True, mode=None):
        from vulkanhybridraytracer_gb300.hybrid import HybridContext
        self.wl = wl
        self.ctx = HybridContext(0)
        self.ctx.set_scene(wl.scene)
        self.orc = po.OracleScene()
        self.orc.set_scene(wl.scene)
        if mode is not None:  # binary tree of the build: HY_BUILD_SAH (default) or HY_BUILD_LBVH
            self.ctx.set_build_mode(mode)
            self.orc.set_build_mode(mode)
        if build:
            self.gi = self.ctx.build_bvh()
            self.oi = self.orc.build_bvh()


def glass_workload(w=96, h=96):
    wl = scenes.small(0, w, h)
    for i in (2, 5, 9):
        wl.scene.materials[i] = Material(4, (0.9, 0.95, 1.0, 1), 1.0, 0.0, 1.5)
    for i in (3, 7):
        wl.scene.materials[i] = Material(3, (0.8, 0.8, 0.8, 1), 1.0, 0.05, 1.0)
    wl.scene.materials[0] = Material(3, (0.6, 0.6, 0.6, 1), 1.0, 0.1, 1.0)  # mirror floor
    wl.max_bounces = 8
    return wl


@pytest.fixture(scope="module")
def small(gpu_lib, oracle_lib):
    return Pair(scenes.small(0))


@pytest.fixture(scope="module")
def glass(gpu_lib, oracle_lib):
    return Pair(glass_workload())


def assert_bvh_equal(p: Pair):
    assert p.gi["num_bvh8_nodes"] == p.oi["num_bvh8_nodes"] and p.gi["depth"] == p.oi["depth"]
    g = p.ctx.download_bvh(p.gi["num_bvh8_nodes"])
    o = p.orc.download_bvh(p.oi["num_bvh8_nodes"])
    for name, a, b in zip(["morton", "order", "bvh2", "bvh8", "tris"], g, o):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), name


def test_bvh_bitexact_small(small):
    assert_bvh_equal(small)
    assert small.gi["scene_lo"] == small.oi["scene_lo"] and small.gi["scene_hi"] == small.oi["scene_hi"]


def test_bvh_bitexact_small_lbvh(gpu_lib, oracle_lib):
    p = Pair(scenes.small(0), mode=L.HY_BUILD_LBVH)
    assert_bvh_equal(p)
    morton, _, bvh2, _, _ = p.ctx.download_bvh(p.gi["num_bvh8_nodes"])
    assert np.all(np.diff(morton.astype(np.int64)) >= 0)  # Karras: sorted codes, root 0 over everything
    assert bvh2[0, 2] == 0 and bvh2[0, 3] == p.gi["num_tris"] - 1
    p.ctx.close()


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 17, 33, 1000, 5000, 9000])
def test_bvh_bitexact_tiny_and_degenerate(gpu_lib, oracle_lib, n, mode):
    """Few triangles, duplicated positions (equal Morton codes) and zero-area triangles."""
    from vulkanhybridraytracer_gb300.hybrid import HybridContext
    rng = np.random.default_rng(100 + n)
    v = np.zeros((3 * n, 11), np.float32)
    base = rng.uniform(-1, 1, (n, 3))
    base[n // 2:] = base[0]
    for t in range(n):
        for k in range(3):
            v[3 * t + k, 0:3] = base[t] + (rng.uniform(-0.5, 0.5, 3) if t % 5 else 0)  # every 5th is a point
            v[3 * t + k, 4] = 1
    idx = np.arange(3 * n, dtype=np.uint32)
    prims = np.array([[0, 3 * n, 0, 0, 0, 0]], np.uint32)
    xf = np.eye(4, dtype=np.float32).reshape(1, 16)
    mats = Material().to_shader(0)[None]
    lights = np.zeros((0, 12), np.float32)
    ctx = HybridContext(0)
    ctx.set_scene_arrays(v, idx, prims, xf, mats, lights)
    ctx.set_build_mode(mode)
    orc = po.OracleScene()
    orc.set_scene_arrays(v, idx, prims, xf, mats, lights)
    orc.set_build_mode(mode)
    p = Pair.__new__(Pair)
    p.ctx, p.orc, p.gi, p.oi = ctx, orc, ctx.build_bvh(), orc.build_bvh()
    assert_bvh_equal(p)
    rays = _rays(rng, 3000, -2, 2)
    torch = _torch()
    for any_hit in (False, True):
        hg, sg = ctx.trace(torch.from_numpy(rays).cuda(), any_hit, count=True)
        ho, co = orc.trace(rays, any_hit)
        assert np.array_equal(hg.cpu().numpy().view(np.uint32), ho.view(np.uint32))
        assert sg["nodes_visited"] == co[:, 0].sum() and sg["tris_tested"] == co[:, 1].sum()
    ctx.close()


@pytest.mark.parametrize("scale", [1e-6, 1.0, 1e6, 1e12])
def test_trace_bitexact_coordinate_scales(gpu_lib, oracle_lib, scale):
    """Scenes from micro to huge coordinates, with axis-aligned rays (a zero
    direction component: 1/d clamped to 1e20): the node test's plane distances
    (the node scale times 1/d, taken times 2^24 with the plane bytes as q * 2^-24)
    span the float range, and hits and counts still equal the oracle's."""
    from vulkanhybridraytracer_gb300.hybrid import HybridContext
    rng = np.random.default_rng(31)
    n = 2000
    v = np.zeros((3 * n, 11), np.float32)
    cen = rng.uniform(-1, 1, (n, 3))
    for t in range(n):
        for k in range(3):
            v[3 * t + k, 0:3] = (cen[t] + rng.uniform(-0.1, 0.1, 3)) * scale
            v[3 * t + k, 4] = 1
    idx = np.arange(3 * n, dtype=np.uint32)
    prims = np.array([[0, 3 * n, 0, 0, 0, 0]], np.uint32)
    xf = np.eye(4, dtype=np.float32).reshape(1, 16)
    mats = Material().to_shader(0)[None]
    lights = np.zeros((0, 12), np.float32)
    ctx = HybridContext(0)
    ctx.set_scene_arrays(v, idx, prims, xf, mats, lights)
    orc = po.OracleScene()
    orc.set_scene_arrays(v, idx, prims, xf, mats, lights)
    ctx.build_bvh()
    orc.build_bvh()
    m = 20000
    rays = np.zeros((m, 8), np.float32)
    d = rng.normal(size=(m, 3))
    d[::5, 0] = 0.0   # axis-parallel to the y-z plane
    d[::7, 1:] = 0.0  # along x
    d[::7, 0] = np.where(d[::7, 0] == 0, 1.0, d[::7, 0])
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 0:3] = rng.uniform(-1.5, 1.5, (m, 3)) * scale
    rays[:, 3] = 1e-3 * scale
    rays[:, 4:7] = d
    rays[:, 7] = 10.0 * scale
    torch = _torch()
    for any_hit in (False, True):
        hg, sg = ctx.trace(torch.from_numpy(rays).cuda(), any_hit, count=True)
        ho, co = orc.trace(rays, any_hit)
        assert np.array_equal(hg.cpu().numpy().view(np.uint32), ho.view(np.uint32))
        assert sg["nodes_visited"] == int(co[:, 0].sum()) and sg["tris_tested"] == int(co[:, 1].sum())
        assert sg["error_flags"] == 0
        assert (ho.view(np.uint32)[:, 1] != 0xFFFFFFFF).mean() > 0.05  # the rays do hit
    ctx.close()


def _rays(rng, n, lo=-6, hi=6):
    org = rng.uniform(lo, hi, (n, 3)).astype(np.float32)
    org[:, 1] = rng.uniform(0.1, 4, n)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3], r[:, 3], r[:, 4:7], r[:, 7] = org, 0.001, d, 1000.0
    return r


@pytest.mark.parametrize("any_hit", [False, True])
def test_trace_bitexact(small, any_hit):
    torch = _torch()
    rays = _rays(np.random.default_rng(7), 50000)
    rays[::7, 4:7] = [0, -1, 0]   # axis-aligned directions (zero components)
    rays[::11, 7] = 0.5           # short rays
    hg, sg = small.ctx.trace(torch.from_numpy(rays).cuda(), any_hit, count=True)
    ho, co = small.orc.trace(rays, any_hit)
    assert np.array_equal(hg.cpu().numpy().view(np.uint32), ho.view(np.uint32))
    assert sg["nodes_visited"] == int(co[:, 0].sum()) and sg["tris_tested"] == int(co[:, 1].sum())
    assert sg["error_flags"] == 0
    # against brute force (the reference's semantics without any BVH)
    hb, _ = small.orc.trace(rays, any_hit, po.TRACE_BRUTE)
    ig, ib = hg.cpu().numpy().view(np.uint32)[:, 1], hb.view(np.uint32)[:, 1]
    assert np.mean((ig != 0xFFFFFFFF) == (ib != 0xFFFFFFFF)) >= 0.9999
    if not any_hit:
        assert np.mean(ig == ib) >= 0.9999


def test_gbuffer_primary(small):
    torch = _torch()
    cam = small.wl.camera(0.0)
    W, H = small.wl.width, small.wl.height
    g = [p.cpu().numpy() for p in small.ctx.gbuffer(cam, W, H)]
    o = small.orc.gbuffer(cam, W, H)
    for i in (0, 2, 3, 4, 5):
        assert np.array_equal(g[i], o[i]), f"plane {i}"
    np.testing.assert_allclose(g[1], o[1], atol=2e-6)
    torch.cuda.synchronize()


def run_both(p: Pair, frame, spp, rng_mode, fmt, flags=0, max_bounces=None, hist0=None, planes=None,
             formats=None):
    from vulkanhybridraytracer_gb300.hybrid import GBUF_FP32_FORMATS, pass_config
    torch = _torch()
    wl = p.wl
    W, H = wl.width, wl.height
    mb = wl.max_bounces if max_bounces is None else max_bounces
    cam = wl.camera(float(frame))
    if planes is None:
        planes = p.orc.gbuffer(cam, W, H)
    formats = formats or GBUF_FP32_FORMATS
    nl = len(wl.scene.lights)
    dt = np.uint8 if fmt == L.HY_ACCUM_U8 else np.float32
    if hist0 is None:
        rng = np.random.default_rng(frame + 17)
        hist0 = (rng.integers(0, 256, (nl, H, W)).astype(np.uint8) if fmt == L.HY_ACCUM_U8
                 else rng.random((nl, H, W)).astype(np.float32))
    hist_g = torch.from_numpy(hist0.copy()).cuda()
    out_f = torch.zeros((H, W, 4), device="cuda")
    out_8 = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    dplanes = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in planes]
    st = p.ctx.forward(dplanes, cam, pass_config(spp, mb, rng_mode, frame, flags), hist_g, fmt, out_f=out_f,
                       out_8=out_8, formats=formats)
    hist_o = hist0.copy().astype(dt)
    ocfg = po.cfg_dict(spp, mb, rng_mode, frame, flags)
    of, o8, osh, ost = p.orc.forward(planes, cam, ocfg, hist_o, fmt, formats=formats)
    hg = hist_g.cpu().numpy()
    of_g = None
    if not flags & L.HY_FLAG_NO_ACCUM:
        # the oracle's shading of the GPU's own shadow history: what the GPU image must be
        # given the GPU's shadow decisions
        of_g = p.orc.shade(planes, cam, ocfg, np.ascontiguousarray(hg), fmt, formats=formats)[0]
    return (out_f.cpu().numpy(), out_8.cpu().numpy(), hg, st), (of, o8, hist_o, osh, ost, of_g)


def check_parity(g, o, fmt):
    out_f, out_8, hist_g, st = g
    of, o8, hist_o, osh, ost, of_g = o
    assert st["error_flags"] == 0
    flips = np.mean(hist_g != hist_o)
    assert flips <= FLIP_TOL, f"history differs on {flips:.2e} of texels"
    agree = np.all(hist_g == hist_o, axis=0)
    err = np.abs(out_f[..., :3].astype(np.float64) - of[..., :3])
    rms = np.sqrt((err ** 2).sum() / max((of[..., :3].astype(np.float64) ** 2).sum(), 1e-30))
    assert rms <= RMS_TOL, f"relative RMS {rms:.3e}"
    assert err[agree].max(initial=0) <= MAX_TOL, f"max |err| {err[agree].max():.3e}"
    if of_g is not None:
        # every pixel, flipped shadow decisions included, against the oracle shading the
        # GPU's history: a flip moves the pixel by its samples' share of the light only
        err_g = np.abs(out_f[..., :3].astype(np.float64) - of_g[..., :3])
        assert err_g.max(initial=0) <= MAX_TOL, f"max |err| vs shading of the GPU history {err_g.max():.3e}"
    assert np.all(out_f[..., 3] == 1)
    bad8 = np.abs(out_8.astype(int) - o8.astype(int)) > 1
    assert bad8[agree].mean() <= 1e-3
    for k in ("shadow_rays", "reflection_rays"):
        assert abs(st[k] - ost[k]) <= max(2, 1e-4 * ost[k]), (k, st[k], ost[k])


@pytest.mark.parametrize("frame", [0, 1, 5])
@pytest.mark.parametrize("rng_mode,spp", [(L.HY_RNG_REFERENCE, 1), (L.HY_RNG_REFERENCE, 8),
                                          (L.HY_RNG_DECORRELATED, 4)])
def test_forward_small(small, frame, rng_mode, spp):
    g, o = run_both(small, frame, spp, rng_mode, L.HY_ACCUM_U8)
    check_parity(g, o, L.HY_ACCUM_U8)


@pytest.mark.parametrize("flags", [0, L.HY_FLAG_NO_ACCUM, L.HY_FLAG_FULL_BLUR_DISPATCH])
@pytest.mark.parametrize("frame", [0, 3])
def test_forward_f32_history_and_flags(small, flags, frame):
    g, o = run_both(small, frame, 4, L.HY_RNG_DECORRELATED, L.HY_ACCUM_F32, flags)
    check_parity(g, o, L.HY_ACCUM_F32)


@pytest.mark.parametrize("frame", [0, 2])
def test_forward_glass_mirror_bounces(glass, frame):
    g, o = run_both(glass, frame, 2, L.HY_RNG_DECORRELATED, L.HY_ACCUM_U8)
    assert g[3]["reflection_rays"] > g[3]["hit_shadow_rays"] > 0
    check_parity(g, o, L.HY_ACCUM_U8)


@pytest.mark.parametrize("rng_mode,spp", [(L.HY_RNG_REFERENCE, 1), (L.HY_RNG_DECORRELATED, 4)])
def test_forward_ggx_reflection(small, rng_mode, spp):
    """HY_FLAG_GGX_REFLECTION: the mirror texels' reflection ray sampled from their GGX
    lobe with the texel's own RNG stream, against the oracle restating the same
    sampling; the flag changes the mirror texels and no others."""
    g, o = run_both(small, 2, spp, rng_mode, L.HY_ACCUM_U8, flags=L.HY_FLAG_GGX_REFLECTION)
    check_parity(g, o, L.HY_ACCUM_U8)
    g0, _ = run_both(small, 2, spp, rng_mode, L.HY_ACCUM_U8)
    wl = small.wl
    planes = small.orc.gbuffer(wl.camera(2.0), wl.width, wl.height)
    mats = np.array([m.shading_model for m in wl.scene.materials])
    mi = planes[0][..., 3].astype(np.int64)
    mirror = (mats[np.clip(mi, 0, len(mats) - 1)] == 3) & ~((planes[0][..., 3] == 0) & (planes[1][..., 3] == 0))
    changed = np.any(g[0] != g0[0], axis=-1)
    assert changed.any() and not changed[~mirror].any()
    assert g[3]["reflection_rays"] == g0[3]["reflection_rays"] > 0


@pytest.mark.parametrize("frame", [0, 2])
def test_forward_ggx_glass_mirror_bounces(glass, frame):
    """The GGX-sampled first bounce followed by the reference's 8-bounce glass/mirror chain."""
    g, o = run_both(glass, frame, 2, L.HY_RNG_DECORRELATED, L.HY_ACCUM_U8, flags=L.HY_FLAG_GGX_REFLECTION)
    check_parity(g, o, L.HY_ACCUM_U8)


def test_packed_reference_formats(small):
    """The reference's own attachment formats: RGBA16F, RGBA16F, RGBA8, RG16F, RGBA8, RGBA8."""
    cam = small.wl.camera(2.0)
    W, H = small.wl.width, small.wl.height
    f = small.orc.gbuffer(cam, W, H)
    p = [f[0].astype(np.float16), f[1].astype(np.float16),
         np.round(np.clip(f[2], 0, 1) * 255).astype(np.uint8), f[3].astype(np.float16),
         np.round(np.clip(f[4], 0, 1) * 255).astype(np.uint8), np.round(np.clip(f[5], 0, 1) * 255).astype(np.uint8)]
    fmts = (L.HY_FMT_RGBA16F, L.HY_FMT_RGBA16F, L.HY_FMT_RGBA8, L.HY_FMT_RG16F, L.HY_FMT_RGBA8, L.HY_FMT_RGBA8)
    g, o = run_both(small, 2, 1, L.HY_RNG_REFERENCE, L.HY_ACCUM_U8, planes=p, formats=fmts)
    check_parity(g, o, L.HY_ACCUM_U8)


def test_stagewise_matches_fused(small):
    """shadow -> accumulate -> shade called one by one equals hy_hybrid_forward's fused kernel."""
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    torch = _torch()
    wl = small.wl
    W, H, nl = wl.width, wl.height, len(wl.scene.lights)
    cam = wl.camera(4.0)
    planes = [torch.from_numpy(x).cuda() for x in small.orc.gbuffer(cam, W, H)]
    h0 = torch.from_numpy(np.random.default_rng(1).integers(0, 256, (nl, H, W)).astype(np.uint8)).cuda()
    cfg = pass_config(4, 1, L.HY_RNG_DECORRELATED, 4, 0)
    ha, hb = h0.clone(), h0.clone()
    fa, fb = torch.zeros((H, W, 4), device="cuda"), torch.zeros((H, W, 4), device="cuda")
    shadow = torch.zeros((nl, H, W), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()   # torch's stream vs the context's own stream
    small.ctx.forward(planes, cam, cfg, ha, L.HY_ACCUM_U8, out_f=fa)
    small.ctx.shadow_pass(planes, cam, cfg, shadow, L.HY_ACCUM_U8)
    small.ctx.accumulate_pass(planes, cfg, shadow, hb, L.HY_ACCUM_U8)
    small.ctx.shade_pass(planes, cam, cfg, hb, L.HY_ACCUM_U8, out_f=fb)
    assert torch.equal(ha, hb)
    assert torch.equal(fa, fb)


def test_accumulate_reprojection(small):
    """blur.comp reset branch with non-zero motion: reads the pre-pass history at
    (x + r.x W, y + r.x H), clamps to the 3x3 range, mixes 0.4; bit-exact."""
    torch = _torch()
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    W, H, nl = 72, 40, 2
    rng = np.random.default_rng(3)
    planes = [np.zeros((H, W, 4), np.float32) for _ in range(6)]
    planes[3] = (0.5 + rng.integers(-3, 4, (H, W, 2)) / (2.0 * W)).astype(np.float32)
    shadow = rng.integers(0, 256, (nl, H, W)).astype(np.uint8)
    hist = rng.integers(0, 256, (nl, H, W)).astype(np.uint8)
    for frame in (0, -1, 6):
        hg = torch.from_numpy(hist.copy()).cuda()
        small.ctx.accumulate_pass([torch.from_numpy(x).cuda() for x in planes], pass_config(accum_frame=frame),
                                  torch.from_numpy(shadow).cuda(), hg, L.HY_ACCUM_U8)
        ho = hist.copy()
        small.orc.accumulate(planes, po.cfg_dict(accum_frame=frame), shadow, ho, 0)
        assert np.array_equal(hg.cpu().numpy(), ho), frame


def test_host_buffers_equal_device(small):
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    torch = _torch()
    wl = small.wl
    W, H, nl = wl.width, wl.height, len(wl.scene.lights)
    cam = wl.camera(3.0)
    pn = small.orc.gbuffer(cam, W, H)
    cfg = pass_config(2, 1, L.HY_RNG_DECORRELATED, 3, 0)
    h1 = torch.zeros((nl, H, W), dtype=torch.uint8, device="cuda")
    h2 = h1.clone()
    o1 = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()   # torch's stream vs the context's own stream
    small.ctx.forward([torch.from_numpy(x).cuda() for x in pn], cam, cfg, h1, L.HY_ACCUM_U8, out_8=o1)
    o2 = np.zeros((H, W, 4), np.uint8)
    st = small.ctx.forward_host(pn, cam, cfg, h2, L.HY_ACCUM_U8, out_8=o2)
    assert np.array_equal(o1.cpu().numpy(), o2) and torch.equal(h1, h2)
    assert st["shadow_rays"] > 0


def test_host_buffers_back_to_back(small):
    """Host-buffer calls one after another, each on another G-buffer: frames 0
    (raw images + blur) and 1-3 (fused running mean) equal the device-buffer
    calls.  hy_hybrid_forward_host always waits for its own result (it copies
    the image back), so these calls run in sequence; the next test covers a
    host-buffer call queued behind work still running on the stream."""
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    torch = _torch()
    wl = small.wl
    W, H, nl = wl.width, wl.height, len(wl.scene.lights)
    frames = [0, 1, 2, 3]
    gbs = [small.orc.gbuffer(wl.camera(float(5 + f)), W, H) for f in frames]
    h_dev = torch.zeros((nl, H, W), dtype=torch.uint8, device="cuda")
    h_host = h_dev.clone()
    want = []
    torch.cuda.synchronize()
    for f, pn in zip(frames, gbs):
        o = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
        small.ctx.forward([torch.from_numpy(x).cuda() for x in pn], wl.camera(float(5 + f)),
                          pass_config(4, 1, L.HY_RNG_DECORRELATED, f, 0), h_dev, L.HY_ACCUM_U8, out_8=o)
        want.append(o.cpu().numpy())
    got = [np.zeros((H, W, 4), np.uint8) for _ in frames]
    for f, pn, o in zip(frames, gbs, got):
        small.ctx.forward_host(pn, wl.camera(float(5 + f)),
                               pass_config(4, 1, L.HY_RNG_DECORRELATED, f, L.HY_FLAG_NO_STATUS_SYNC), h_host,
                               L.HY_ACCUM_U8, out_8=o, stats=False)
    small.ctx.synchronize()
    for f, a, b in zip(frames, want, got):
        assert np.array_equal(a, b), f
    assert torch.equal(h_dev, h_host)


def test_host_buffers_behind_pending_work(small):
    """A host-buffer call queued behind device-buffer calls that are still
    running (HY_FLAG_NO_STATUS_SYNC, no host sync in between): its planes 2-5
    go up on a side stream that must start only after the earlier passes, and
    the shared history must see every frame in order.  Alternating device and
    host calls give the same images and history as device calls alone."""
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    torch = _torch()
    wl = small.wl
    W, H, nl = wl.width, wl.height, len(wl.scene.lights)
    frames = [0, 1, 2, 3, 4, 5]
    gbs = [small.orc.gbuffer(wl.camera(float(9 + f)), W, H) for f in frames]
    h_ref = torch.zeros((nl, H, W), dtype=torch.uint8, device="cuda")
    h_mix = h_ref.clone()
    dplanes = [[torch.from_numpy(x).cuda() for x in pn] for pn in gbs]
    outs_ref = [torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda") for _ in frames]
    outs_dev = [torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda") for _ in frames]
    torch.cuda.synchronize()   # torch's stream vs the context's own stream
    want = []
    for f, dp, o in zip(frames, dplanes, outs_ref):
        small.ctx.forward(dp, wl.camera(float(9 + f)), pass_config(4, 1, L.HY_RNG_DECORRELATED, f, 0), h_ref,
                          L.HY_ACCUM_U8, out_8=o)
        want.append(o.cpu().numpy())
    got = []
    for f, pn, dp, od in zip(frames, gbs, dplanes, outs_dev):
        if f % 2 == 0:   # queued, not waited for
            small.ctx.forward(dp, wl.camera(float(9 + f)),
                              pass_config(4, 1, L.HY_RNG_DECORRELATED, f, L.HY_FLAG_NO_STATUS_SYNC), h_mix,
                              L.HY_ACCUM_U8, out_8=od, stats=False)
            got.append(od)
        else:            # host buffers, right behind the pending call
            oh = np.zeros((H, W, 4), np.uint8)
            small.ctx.forward_host(pn, wl.camera(float(9 + f)),
                                   pass_config(4, 1, L.HY_RNG_DECORRELATED, f, 0), h_mix, L.HY_ACCUM_U8, out_8=oh)
            got.append(oh)
    small.ctx.synchronize()
    for f, a, b in zip(frames, want, got):
        b = b.cpu().numpy() if hasattr(b, "cpu") else b
        assert np.array_equal(a, b), f
    assert torch.equal(h_ref, h_mix)


def test_deterministic(small):
    a = run_both(small, 3, 4, L.HY_RNG_DECORRELATED, L.HY_ACCUM_U8)[0]
    b = run_both(small, 3, 4, L.HY_RNG_DECORRELATED, L.HY_ACCUM_U8)[0]
    for x, y in zip(a[:3], b[:3]):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("visits", [1, 8, 16])
def test_stream_counts_equal_per_lane_walk(small, visits):
    """The tile streams split every ray's walk into scheduling rounds and hand
    the samples to whichever lanes are free, but each ray makes the same node
    visits and triangle tests: images and node/triangle counts equal one lane
    per pixel's."""
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    torch = _torch()
    wl = small.wl
    W, H, nl = wl.width, wl.height, len(wl.scene.lights)
    cam = wl.camera(6.0)
    planes = [torch.from_numpy(x).cuda() for x in small.orc.gbuffer(cam, W, H)]
    a = torch.zeros((nl, H, W), dtype=torch.uint8, device="cuda")
    b = torch.zeros_like(a)
    torch.cuda.synchronize()
    fl = L.HY_FLAG_COUNT_TRAVERSAL
    sa = small.ctx.shadow_pass(planes, cam, pass_config(8, 1, L.HY_RNG_DECORRELATED, 6, fl, visits_per_round=visits),
                               a)
    sb = small.ctx.shadow_pass(planes, cam, pass_config(8, 1, L.HY_RNG_DECORRELATED, 6, fl | L.HY_FLAG_PIXEL_PARALLEL),
                               b)
    assert torch.equal(a, b)
    for k in ("shadow_rays", "nodes_visited", "tris_tested"):
        assert sa[k] == sb[k] > 0, k


def test_counts_match_oracle_pass(small):
    """With HY_FLAG_COUNT_TRAVERSAL the pass's node/triangle counts equal the
    oracle's BVH8 traversal of the same frame (REFERENCE RNG, exact rays)."""
    g, o = run_both(small, 1, 1, L.HY_RNG_REFERENCE, L.HY_ACCUM_U8, flags=L.HY_FLAG_COUNT_TRAVERSAL)
    st, ost = g[3], o[4]
    assert abs(st["nodes_visited"] - ost["nodes_visited"]) <= 1e-3 * ost["nodes_visited"]
    assert abs(st["tris_tested"] - ost["tris_tested"]) <= 1e-3 * ost["tris_tested"]


@pytest.mark.parametrize("order", [L.HY_ANYHIT_FAR_FIRST, L.HY_ANYHIT_NEAR_FIRST])
def test_anyhit_order(gpu_lib, oracle_lib, order):
    """Both any-hit child orders: hits and traversal counts bit-exact with the
    oracle walking in the same order; the occlusion of every ray, the pass's
    shadow history and its image equal across the orders; closest-hit
    queries do not depend on the order."""
    torch = _torch()
    p = Pair(scenes.small(0))
    assert p.ctx.anyhit_order() == L.HY_ANYHIT_FAR_FIRST  # AUTO: the structure fits in L2
    rays = _rays(np.random.default_rng(11), 40000)
    base = {}
    for o in (L.HY_ANYHIT_FAR_FIRST, order):
        p.ctx.set_anyhit_order(o)
        p.orc.set_anyhit_order(o)
        assert p.ctx.anyhit_order() == o
        for any_hit in (True, False):
            hg, sg = p.ctx.trace(torch.from_numpy(rays).cuda(), any_hit, count=True)
            ho, co = p.orc.trace(rays, any_hit)
            hg = hg.cpu().numpy().view(np.uint32)
            assert np.array_equal(hg, ho.view(np.uint32))
            assert sg["nodes_visited"] == int(co[:, 0].sum()) and sg["tris_tested"] == int(co[:, 1].sum())
            base.setdefault(any_hit, hg)
            if any_hit:
                assert np.array_equal(hg[:, 1] != L.HY_NO_HIT, base[True][:, 1] != L.HY_NO_HIT)
            else:
                assert np.array_equal(hg, base[False])
        g, o_ = run_both(p, 1, 4, L.HY_RNG_DECORRELATED, L.HY_ACCUM_U8, flags=L.HY_FLAG_COUNT_TRAVERSAL)
        check_parity(g, o_, L.HY_ACCUM_U8)
        base.setdefault("pass", g)
        assert np.array_equal(g[2], base["pass"][2]) and np.array_equal(g[1], base["pass"][1])
    with pytest.raises(L.HyError):
        p.ctx.set_anyhit_order(3)
    p.ctx.set_anyhit_order(L.HY_ANYHIT_AUTO)
    assert p.ctx.anyhit_order() == L.HY_ANYHIT_FAR_FIRST
    p.ctx.close()


def test_error_paths(gpu_lib, oracle_lib):
    from vulkanhybridraytracer_gb300.hybrid import HybridContext, pass_config
    torch = _torch()
    wl = scenes.small(0, 32, 32)
    ctx = HybridContext(0)
    planes = [torch.zeros((32, 32, 4 if i != 3 else 2), device="cuda") for i in range(6)]
    hist = torch.zeros((2, 32, 32), dtype=torch.uint8, device="cuda")
    cam = wl.camera(0.0)
    with pytest.raises(L.HyError) as e:
        ctx.forward(planes, cam, pass_config(1), hist)
    assert e.value.code == L.HY_ERR_NOT_READY
    ctx.set_scene(wl.scene)
    with pytest.raises(L.HyError) as e:
        ctx.forward(planes, cam, pass_config(1), hist)
    assert e.value.code == L.HY_ERR_NOT_READY   # no BVH yet
    ctx.build_bvh()
    with pytest.raises(L.HyError) as e:
        ctx.forward(planes, cam, pass_config(0), hist)
    assert e.value.code == L.HY_ERR_INVALID_ARG  # spp 0
    with pytest.raises(L.HyError) as e:
        ctx.forward(planes, cam, pass_config(1), torch.zeros((3, 32, 32), dtype=torch.uint8, device="cuda"))
    assert e.value.code == L.HY_ERR_INVALID_ARG  # history for more lights than the scene has
    # forced allocation failure surfaces as HY_ERR_OOM and leaves the context usable
    assert ctx.lib.hy_debug_fail_alloc_after(ctx.h, 1) == 0
    with pytest.raises(L.HyError) as e:
        ctx.forward(planes, cam, pass_config(1, accum_frame=0), hist)   # reset frame allocates scratch
    assert e.value.code == L.HY_ERR_OOM
    ctx.forward(planes, cam, pass_config(1, accum_frame=0), hist)
    # non-finite geometry is rejected at upload
    verts, idx, prims, xf, mats, lights = wl.scene.pack()
    bad = verts.copy()
    bad[0, 0] = np.nan
    with pytest.raises(L.HyError) as e:
        ctx.set_scene_arrays(bad, idx, prims, xf, mats, lights)
    assert e.value.code == L.HY_ERR_NAN_INPUT
    badp = prims.copy()
    badp[0, 3] = 99   # material id past the material table
    ctx.set_scene_arrays(verts, idx, badp, xf, mats, lights)
    ctx.build_bvh()
    with pytest.raises(L.HyError) as e:
        ctx.forward(planes, cam, pass_config(1), hist)
    assert e.value.code == L.HY_ERR_INVALID_ARG
    ctx.close()


def test_traversal_limits_run_out(gpu_lib, oracle_lib):
    """Failure detection without a GPU fault: with the per-ray node-visit budget
    or the stack cap lowered at run time, every kind of walk stops at the
    counter test and the call reports HY_ERR_TIMEOUT / HY_ERR_STACK_OVERFLOW;
    with the limits restored the same context traces and renders exactly as
    the oracle again."""
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    torch = _torch()
    p = Pair(glass_workload(48, 48))
    lib, h = p.ctx.lib, p.ctx.h
    rays = torch.from_numpy(_rays(np.random.default_rng(5), 20000)).cuda()
    W, H, nl = p.wl.width, p.wl.height, len(p.wl.scene.lights)
    cam = p.wl.camera(1.0)
    planes = [torch.from_numpy(x).cuda() for x in p.orc.gbuffer(cam, W, H)]
    hist = torch.zeros((nl, H, W), dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    cases = [((2, 0), L.HY_ERR_TIMEOUT), ((0, 1), L.HY_ERR_STACK_OVERFLOW)]
    for (visits, depth), code in cases:
        assert lib.hy_debug_set_traversal_limits(h, visits, depth) == L.HY_OK
        for any_hit in (False, True):
            with pytest.raises(L.HyError) as e:
                p.ctx.trace(rays, any_hit)
            assert e.value.code == code, (visits, depth, any_hit)
        for frame, flags in ((0, 0), (3, 0), (3, L.HY_FLAG_PIXEL_PARALLEL)):
            with pytest.raises(L.HyError) as e:
                p.ctx.forward(planes, cam, pass_config(4, 8, L.HY_RNG_DECORRELATED, frame, flags), hist)
            assert e.value.code == code, (visits, depth, frame, flags)
    assert lib.hy_debug_set_traversal_limits(h, 0, 65) == L.HY_ERR_INVALID_ARG
    assert lib.hy_debug_set_traversal_limits(h, 0, 0) == L.HY_OK
    hg, sg = p.ctx.trace(rays, False, count=True)
    ho, co = p.orc.trace(rays.cpu().numpy(), False)
    assert np.array_equal(hg.cpu().numpy().view(np.uint32), ho.view(np.uint32)) and sg["error_flags"] == 0
    g, o = run_both(p, 2, 2, L.HY_RNG_DECORRELATED, L.HY_ACCUM_U8)
    check_parity(g, o, L.HY_ACCUM_U8)
    assert lib.hy_error_string(L.HY_ERR_BAD_INDEX).decode().startswith("acceleration structure index")
    p.ctx.close()


def test_device_memory_cap(gpu_lib):
    from vulkanhybridraytracer_gb300.hybrid import HybridContext
    wl = scenes.small(0, 32, 32)
    ctx = HybridContext(0, max_device_bytes=1 << 16)
    with pytest.raises(L.HyError) as e:
        ctx.set_scene(wl.scene)
        ctx.build_bvh()
    assert e.value.code == L.HY_ERR_OOM
    ctx.close()


# ---- full size: the 1080p / 1.5M-triangle workload -------------------------------------------
@pytest.fixture(scope="module")
def hd(gpu_lib, oracle_lib):
    return Pair(scenes.hd(1))


def test_hd_bvh_bitexact(hd):
    assert hd.gi["num_tris"] == 1505282
    assert_bvh_equal(hd)


def test_hd_bvh_bitexact_lbvh(gpu_lib, oracle_lib):
    p = Pair(scenes.hd(1), mode=L.HY_BUILD_LBVH)
    assert_bvh_equal(p)
    p.ctx.close()


@pytest.mark.parametrize("flags", [0, L.HY_FLAG_GGX_REFLECTION])
def test_hd_forward_parity(hd, flags):
    """Whole 1920x1080 frame, 4 lights x 16 decorrelated samples, against the oracle;
    with perfect mirror reflections (the reference's) and with the configuration's
    GGX-sampled reflection ray for roughness < 0.3 texels."""
    g, o = run_both(hd, 3, 16, L.HY_RNG_DECORRELATED, L.HY_ACCUM_U8, flags=flags)
    check_parity(g, o, L.HY_ACCUM_U8)
    assert g[3]["reflection_rays"] > 0


@pytest.mark.parametrize("spp", [2, 3, 16, 40])
def test_group_kernel_equals_pixel_kernel(small, spp):
    """The sample-parallel shadow kernels (lane groups, and the per-warp ray pool;
    LCG jump-ahead per sample) write the same shadow images as the
    one-lane-per-pixel kernel, bit for bit."""
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    torch = _torch()
    wl = small.wl
    W, H, nl = wl.width, wl.height, len(wl.scene.lights)
    cam = wl.camera(5.0)
    planes = [torch.from_numpy(x).cuda() for x in small.orc.gbuffer(cam, W, H)]
    a = torch.zeros((nl, H, W), dtype=torch.uint8, device="cuda")
    b = torch.zeros_like(a)
    c = torch.zeros_like(a)
    torch.cuda.synchronize()
    sa = small.ctx.shadow_pass(planes, cam, pass_config(spp, 1, L.HY_RNG_DECORRELATED, 5, 0), a)
    sb = small.ctx.shadow_pass(planes, cam, pass_config(spp, 1, L.HY_RNG_DECORRELATED, 5, L.HY_FLAG_PIXEL_PARALLEL), b)
    sc = small.ctx.shadow_pass(planes, cam, pass_config(spp, 1, L.HY_RNG_DECORRELATED, 5, L.HY_FLAG_RAY_POOL), c)
    e = torch.zeros_like(a)
    torch.cuda.synchronize()
    se = small.ctx.shadow_pass(planes, cam, pass_config(spp, 1, L.HY_RNG_DECORRELATED, 5, L.HY_FLAG_LANE_GROUPS), e)
    assert torch.equal(a, b) and torch.equal(a, c) and torch.equal(a, e)
    assert sa["shadow_rays"] == sb["shadow_rays"] == sc["shadow_rays"] == se["shadow_rays"] > 0
    # the same schedules with one node visit per round, the tile streams at each register cap
    # and with the shared-memory short stack
    for flags, minb, visits, depth in ((L.HY_FLAG_LANE_GROUPS, 0, 1, 0), (0, 5, 1, 0), (0, 6, 3, 0), (0, 8, 16, 0),
                                       (0, 0, 0, 8)):
        f = torch.zeros_like(a)
        torch.cuda.synchronize()
        small.ctx.shadow_pass(planes, cam, pass_config(spp, 1, L.HY_RNG_DECORRELATED, 5, flags, min_blocks=minb,
                                                       visits_per_round=visits, stack_depth=depth), f)
        assert torch.equal(a, f), (flags, minb, visits, depth)
    # smaller lane groups (several samples per lane in turn): the same images
    for G in (2, 4, 8):
        d = torch.zeros_like(a)
        torch.cuda.synchronize()
        small.ctx.shadow_pass(planes, cam, pass_config(spp, 1, L.HY_RNG_DECORRELATED, 5, 0, group_lanes=G), d)
        assert torch.equal(a, d), G


@pytest.mark.parametrize("frame", [0, 3])
def test_tile_stream_forward_equals_groups(small, frame):
    """The light-major tile schedule (the default), raw images and the fused
    running-mean variant alike, gives the same history and image as the lane
    groups (HY_FLAG_LANE_GROUPS), bit for bit."""
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    torch = _torch()
    wl = small.wl
    W, H, nl = wl.width, wl.height, len(wl.scene.lights)
    cam = wl.camera(float(frame))
    planes = [torch.from_numpy(x).cuda() for x in small.orc.gbuffer(cam, W, H)]
    h0 = torch.randint(0, 256, (nl, H, W), dtype=torch.uint8, generator=torch.Generator().manual_seed(frame)).cuda()
    outs = []
    for flags in (L.HY_FLAG_LANE_GROUPS, 0):
        h = h0.clone()
        o = torch.zeros((H, W, 4), dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        st = small.ctx.forward(planes, cam, pass_config(8, 2, L.HY_RNG_DECORRELATED, frame, flags), h, out_8=o)
        outs.append((h, o, st))
    (ha, oa, sa), (hb, ob, sb) = outs
    assert torch.equal(ha, hb) and torch.equal(oa, ob)
    assert sa["shadow_rays"] == sb["shadow_rays"] > 0 and sb["error_flags"] == 0


@pytest.mark.parametrize("rng_mode,spp", [(L.HY_RNG_REFERENCE, 1), (L.HY_RNG_REFERENCE, 8),
                                          (L.HY_RNG_DECORRELATED, 1)])
def test_tile_stream_one_ray_per_pixel_light(small, rng_mode, spp):
    """REFERENCE RNG (all samples one ray) and spp = 1 also go through the tile
    streams by default: the same images as one lane per pixel."""
    from vulkanhybridraytracer_gb300.hybrid import pass_config
    torch = _torch()
    wl = small.wl
    W, H, nl = wl.width, wl.height, len(wl.scene.lights)
    cam = wl.camera(2.0)
    planes = [torch.from_numpy(x).cuda() for x in small.orc.gbuffer(cam, W, H)]
    a = torch.zeros((nl, H, W), dtype=torch.uint8, device="cuda")
    b = torch.zeros_like(a)
    torch.cuda.synchronize()
    sa = small.ctx.shadow_pass(planes, cam, pass_config(spp, 1, rng_mode, 2, 0), a)
    sb = small.ctx.shadow_pass(planes, cam, pass_config(spp, 1, rng_mode, 2, L.HY_FLAG_PIXEL_PARALLEL), b)
    assert torch.equal(a, b)
    assert sa["shadow_rays"] == sb["shadow_rays"] > 0


@pytest.mark.parametrize("rng_mode,spp", [(L.HY_RNG_REFERENCE, 4), (L.HY_RNG_DECORRELATED, 1)])
@pytest.mark.parametrize("w,h", [(96, 64), (37, 23)])
def test_one_ray_streams_many_lights(gpu_lib, oracle_lib, rng_mode, spp, w, h):
    """One ray per pixel-light over 40 lights, some directional, out of range
    or below the horizon: the tile streams' raw shadow images and fused
    running mean equal one lane per pixel bit for bit, and the raw images
    match the oracle."""
    from vulkanhybridraytracer_gb300.hybrid import HybridContext, pass_config
    from vulkanhybridraytracer_gb300.scene import Light
    torch = _torch()
    rng = np.random.default_rng(23)
    wl = scenes.small(0, w, h)
    lights = []
    for i in range(40):
        if i % 13 == 5:
            lights.append(Light(scenes.DIRECTIONAL_LIGHT, (1, 1, 1), (0.3, 1.0, 0.2), 1.0, 500.0, 0.1))
        else:
            pos = (rng.uniform(-8, 8), rng.uniform(-1, 9), rng.uniform(-8, 8))
            lights.append(Light(scenes.POINT_LIGHT, (1, 1, 1), pos, float(rng.uniform(5, 30)),
                                float(rng.choice([3.0, 500.0])), float(rng.uniform(0.05, 0.6))))
    wl.scene.lights = lights
    ctx = HybridContext(0)
    orc = po.OracleScene()
    try:
        ctx.set_scene(wl.scene)
        ctx.build_bvh()
        orc.set_scene(wl.scene)
        orc.build_bvh()
        cam = wl.camera(3.0)
        planes_np = orc.gbuffer(cam, w, h)
        planes = [torch.from_numpy(x).cuda() for x in planes_np]
        nl = len(lights)
        a = torch.zeros((nl, h, w), dtype=torch.uint8, device="cuda")
        b = torch.zeros_like(a)
        sa = ctx.shadow_pass(planes, cam, pass_config(spp, 1, rng_mode, 3, 0), a)
        sb = ctx.shadow_pass(planes, cam, pass_config(spp, 1, rng_mode, 3, L.HY_FLAG_PIXEL_PARALLEL), b)
        assert torch.equal(a, b)
        assert sa["shadow_rays"] == sb["shadow_rays"] > 0 and sa["error_flags"] == 0
        osh, _ = orc.shadow_pass(planes_np, cam, po.cfg_dict(spp, 1, rng_mode, 3), L.HY_ACCUM_U8)
        assert np.mean(a.cpu().numpy() != osh) <= FLIP_TOL
        h0 = torch.randint(0, 256, (nl, h, w), dtype=torch.uint8, generator=torch.Generator().manual_seed(3)).cuda()
        outs = []
        for flags in (0, L.HY_FLAG_PIXEL_PARALLEL):
            hh = h0.clone()
            o = torch.zeros((h, w, 4), dtype=torch.uint8, device="cuda")
            ctx.forward(planes, cam, pass_config(spp, 1, rng_mode, 3, flags), hh, out_8=o)
            outs.append((hh, o))
        assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][1], outs[1][1])
    finally:
        ctx.close()


@pytest.mark.parametrize("w,h,spp", [(37, 23, 5), (8, 4, 64), (1, 1, 3), (130, 3, 2)])
def test_tile_stream_ragged_frames(gpu_lib, oracle_lib, w, h, spp):
    """Frames whose sides are not multiples of the 8x4 tile (lanes without a pixel
    still take items), one tile, one pixel: the tile streams write the same
    images as one lane per pixel."""
    from vulkanhybridraytracer_gb300.hybrid import HybridContext, pass_config
    torch = _torch()
    wl = scenes.small(0, w, h)
    ctx = HybridContext(0)
    try:
        ctx.set_scene(wl.scene)
        ctx.build_bvh()
        cam = wl.camera(4.0)
        planes = ctx.gbuffer(cam, w, h)
        nl = len(wl.scene.lights)
        a = torch.zeros((nl, h, w), dtype=torch.uint8, device="cuda")
        b = torch.zeros_like(a)
        torch.cuda.synchronize()
        sa = ctx.shadow_pass(planes, cam, pass_config(spp, 1, L.HY_RNG_DECORRELATED, 4, 0), a)
        sb = ctx.shadow_pass(planes, cam, pass_config(spp, 1, L.HY_RNG_DECORRELATED, 4, L.HY_FLAG_PIXEL_PARALLEL), b)
        assert torch.equal(a, b)
        assert sa["shadow_rays"] == sb["shadow_rays"] and sa["error_flags"] == 0
    finally:
        ctx.close()
