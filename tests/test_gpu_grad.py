"""hy_hybrid_backward against the FP64 CPU adjoint and FP64 central finite
differences (h = 1e-4), on the differentiable workload's scene (64
icospheres, 64 materials, 8 point lights, 16 shadow samples) at a reduced
resolution, plus glass/mirror chains.  Tolerance: gradient relative error
<= 1e-3."""
import numpy as np
import pytest

from vulkanhybridraytracer_gb300 import _lib as L
from vulkanhybridraytracer_gb300 import diffrender, scenes

pytestmark = pytest.mark.gpu

REL_TOL = 1e-3


def _case(oracle_lib, wl, spp=16, sigma=0.05, seed=0):
    import torch
    r = diffrender.DiffRenderer(wl.scene, wl.camera(0.0), wl.width, wl.height, spp=spp,
                                max_bounces=wl.max_bounces)
    mp0, lp0 = r.params0
    rng = np.random.default_rng(seed)
    mp_t = np.clip(mp0 + rng.normal(0, sigma, mp0.shape), 0.0, 1.0).astype(np.float32)
    lp_t = (lp0 + rng.normal(0, sigma, lp0.shape)).astype(np.float32)
    target, _ = r.render(mp_t, lp_t)
    target = target.clone()
    img, state = r.render(mp0, lp0)
    grad = 2.0 * (img - target)
    grad[..., 3] = 0.0
    gm, gl, st = r.backward(state, grad)
    torch.cuda.synchronize()
    planes, shadow = state
    planes_np = [p.cpu().numpy() for p in planes]
    shadow_np = shadow.cpu().numpy()
    sc = oracle_lib.OracleScene()
    sc.set_scene(wl.scene)
    sc.build_bvh()
    cfg = oracle_lib.cfg_dict(spp=spp, max_bounces=wl.max_bounces, rng_mode=1)
    go = oracle_lib.GradOracle(sc, planes_np, wl.camera(0.0), cfg, shadow_np, 1)
    out = dict(r=r, mp0=mp0.astype(np.float64), lp0=lp0.astype(np.float64), img=img.cpu().numpy(),
               target=target.cpu().numpy(), w=grad[..., :3].cpu().numpy().astype(np.float64),
               gm=gm.cpu().numpy().astype(np.float64), gl=gl.cpu().numpy().astype(np.float64), go=go, st=st)
    return out


def _rel(a, b, floor):
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


@pytest.fixture(scope="module")
def diff_case(gpu_lib, oracle_lib):
    c = _case(oracle_lib, scenes.diff(3, 160, 128))
    yield c
    c["r"].close()


def test_fp64_image_matches_gpu_image(diff_case):
    c = diff_case
    img64 = c["go"].forward(c["mp0"], c["lp0"])
    ref = c["img"][..., :3]
    err = np.abs(img64 - ref)
    assert np.sqrt((err ** 2).mean()) / np.sqrt((ref ** 2).mean()) <= 1e-3
    assert err.max() <= 1e-2 * max(1.0, np.abs(ref).max())


def test_backward_matches_fp64_adjoint(diff_case):
    c = diff_case
    gm64, gl64 = c["go"].adjoint(c["mp0"], c["lp0"], c["w"])
    g64 = np.concatenate([gm64.ravel(), gl64.ravel()])
    g = np.concatenate([c["gm"].ravel(), c["gl"].ravel()])
    scale = np.abs(g64).max()
    assert scale > 0
    rel = _rel(g, g64, 1e-2 * scale)
    worst = int(np.argmax(rel))
    assert rel.max() <= REL_TOL, (worst, g[worst], g64[worst])
    # parameters the image does not depend on get none; those it clearly does, some
    assert np.all(np.abs(g[g64 == 0]) <= 1e-6 * scale)
    assert np.all(g[np.abs(g64) > 1e-4 * scale] != 0)


def test_backward_matches_central_differences(diff_case):
    c = diff_case
    go, target = c["go"], c["target"][..., :3].astype(np.float64)
    gm64, gl64 = go.adjoint(c["mp0"], c["lp0"], c["w"])
    g64 = np.concatenate([gm64.ravel(), gl64.ravel()])
    g = np.concatenate([c["gm"].ravel(), c["gl"].ravel()])
    scale = np.abs(g64).max()
    rng = np.random.default_rng(1)
    cand = np.flatnonzero(np.abs(g64) > 1e-2 * scale)
    pick = rng.choice(cand, size=min(32, len(cand)), replace=False)
    nm = c["mp0"].size
    h = 1e-4

    def loss(j, delta):
        m2, l2 = c["mp0"].copy(), c["lp0"].copy()
        if j < nm:
            m2.ravel()[j] += delta
        else:
            l2.ravel()[j - nm] += delta
        return float(((go.forward(m2, l2) - target) ** 2).sum())

    fd = np.array([(loss(j, h) - loss(j, -h)) / (2 * h) for j in pick])
    rel = _rel(g[pick], fd, 1e-2 * scale)
    assert rel.max() <= REL_TOL, list(zip(pick.tolist(), g[pick].tolist(), fd.tolist()))


def test_autograd_harness_matches_direct_call(diff_case):
    import torch
    c = diff_case
    r = c["r"]
    from grad_harness import render_fn
    fn = render_fn()
    mp = torch.tensor(c["mp0"], dtype=torch.float32, requires_grad=True)
    lp = torch.tensor(c["lp0"], dtype=torch.float32, requires_grad=True)
    target = torch.tensor(c["target"][..., :3], device=r.dev)
    img = fn.apply(mp, lp, r)
    loss = ((img - target) ** 2).sum()
    loss.backward()
    scale = max(np.abs(c["gm"]).max(), np.abs(c["gl"]).max())
    assert np.abs(mp.grad.numpy() - c["gm"]).max() <= 1e-4 * scale
    assert np.abs(lp.grad.numpy() - c["gl"]).max() <= 1e-4 * scale


def test_backward_glass_and_mirror_chains(gpu_lib, oracle_lib):
    wl = scenes.small_glass(64, 64)
    c = _case(oracle_lib, wl, spp=4)
    try:
        gm64, gl64 = c["go"].adjoint(c["mp0"], c["lp0"], c["w"])
        g64 = np.concatenate([gm64.ravel(), gl64.ravel()])
        g = np.concatenate([c["gm"].ravel(), c["gl"].ravel()])
        scale = np.abs(g64).max()
        rel = _rel(g, g64, 1e-2 * scale)
        assert rel.max() <= REL_TOL, (int(np.argmax(rel)), g[np.argmax(rel)], g64[np.argmax(rel)])
        assert c["st"]["reflection_rays"] > 0
    finally:
        c["r"].close()


def test_backward_zero_upstream_gives_zero(gpu_lib):
    import torch
    wl = scenes.diff(3, 40, 24)
    r = diffrender.DiffRenderer(wl.scene, wl.camera(0.0), wl.width, wl.height, spp=2)
    try:
        img, state = r.render(*r.params0)
        gm, gl, _ = r.backward(state, torch.zeros_like(img))
        torch.cuda.synchronize()
        assert float(gm.abs().max()) == 0.0 and float(gl.abs().max()) == 0.0
    finally:
        r.close()


def test_backward_argument_errors(gpu_lib):
    import torch
    wl = scenes.diff(3, 32, 16)
    r = diffrender.DiffRenderer(wl.scene, wl.camera(0.0), wl.width, wl.height, spp=1)
    try:
        img, (planes, shadow) = r.render(*r.params0)
        g = torch.zeros_like(img)
        from vulkanhybridraytracer_gb300.hybrid import pass_config
        deep = pass_config(spp=1, max_bounces=L.HY_GRAD_MAX_BOUNCES + 1, rng_mode=1)
        with pytest.raises(L.HyError) as e:
            r.ctx.backward(planes, r.cam, deep, shadow, g, r.fmt)
        assert e.value.code == L.HY_ERR_UNSUPPORTED
        with pytest.raises(L.HyError) as e:
            r.ctx.backward(planes, r.cam, r.cfg, shadow, g.view(-1)[1:], r.fmt)  # misaligned upstream pointer
        assert e.value.code == L.HY_ERR_INVALID_ARG
    finally:
        r.close()
