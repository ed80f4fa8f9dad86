"""hy_accumulate_pass_noalloc against hy_accumulate_pass.

The allocation-free entry point serves callers that may not allocate device
memory (an engine whose allocator owns every device allocation, a frame loop
that cannot take cudaFree's device-wide wait).  Its reset-frame history
snapshot lives in a fixed array inside the library instead of context
scratch; this test checks, through the C ABI, that two calls in a row give
exactly what the context-based entry point gives, and that a history larger
than the fixed array is refused.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _planes(torch, W, H, rng):
    planes = [torch.zeros((H, W, 4), device="cuda") for _ in range(6)]
    motion = (0.5 + rng.integers(-3, 4, (H, W, 2)) / (2.0 * W)).astype(np.float32)
    planes[3] = torch.from_numpy(motion).cuda()
    return planes


def test_noalloc_accumulate_matches_context_pass(gpu_lib):
    import torch
    from vulkanhybridraytracer_gb300 import _lib as L
    from vulkanhybridraytracer_gb300 import scenes
    from vulkanhybridraytracer_gb300.hybrid import HybridContext, gbuffer_struct, pass_config

    lib = L.load()
    ctx = HybridContext(0)
    ctx.set_scene(scenes.small(0, 16, 16).scene)
    W, H, nl = 200, 120, 3
    rng = np.random.default_rng(11)
    planes = _planes(torch, W, H, rng)
    gb = gbuffer_struct(planes, W, H)
    hist0 = torch.from_numpy(rng.integers(0, 256, (nl, H, W)).astype(np.uint8)).cuda()
    h_ref, h_new = hist0.clone(), hist0.clone()
    stream = torch.cuda.current_stream().cuda_stream
    # two calls in a row: the reset branch (uses the fixed scratch), then a second
    # reset call that must not see the first call's leftovers, then a running mean
    for frame in (0, -1, 4):
        shadow = torch.from_numpy(rng.integers(0, 256, (nl, H, W)).astype(np.uint8)).cuda()
        cfg = pass_config(accum_frame=frame)
        torch.cuda.synchronize()   # the context runs on its own stream
        ctx.accumulate_pass(planes, cfg, shadow, h_ref, L.HY_ACCUM_U8)
        acc = L.HyAccum(L.HY_ACCUM_U8, nl, h_new.data_ptr())
        rc = lib.hy_accumulate_pass_noalloc(C.byref(gb), C.byref(cfg), C.c_void_p(shadow.data_ptr()), C.byref(acc),
                                            C.c_void_p(stream))
        assert rc == L.HY_OK
        torch.cuda.synchronize()
        assert torch.equal(h_ref, h_new), frame
    # float history too
    hf_ref = torch.rand((nl, H, W), device="cuda")
    hf_new = hf_ref.clone()
    shadow_f = torch.rand((nl, H, W), device="cuda")
    cfg = pass_config(accum_frame=0)
    torch.cuda.synchronize()
    ctx.accumulate_pass(planes, cfg, shadow_f, hf_ref, L.HY_ACCUM_F32)
    acc = L.HyAccum(L.HY_ACCUM_F32, nl, hf_new.data_ptr())
    assert lib.hy_accumulate_pass_noalloc(C.byref(gb), C.byref(cfg), C.c_void_p(shadow_f.data_ptr()), C.byref(acc),
                                          C.c_void_p(stream)) == L.HY_OK
    torch.cuda.synchronize()
    assert torch.equal(hf_ref, hf_new)
    ctx.close()


def test_noalloc_rejects_history_beyond_scratch(gpu_lib):
    import torch
    from vulkanhybridraytracer_gb300 import _lib as L
    from vulkanhybridraytracer_gb300.hybrid import gbuffer_struct, pass_config

    lib = L.load()
    W, H = 1024, 1024
    nl = L.HY_NOALLOC_SCRATCH_BYTES // (W * H) + 1   # one light too many for the u8 history
    planes = _planes(torch, W, H, np.random.default_rng(0))
    gb = gbuffer_struct(planes, W, H)
    hist = torch.zeros((nl, H, W), dtype=torch.uint8, device="cuda")
    shadow = torch.zeros_like(hist)
    acc = L.HyAccum(L.HY_ACCUM_U8, nl, hist.data_ptr())
    cfg = pass_config(accum_frame=0)
    rc = lib.hy_accumulate_pass_noalloc(C.byref(gb), C.byref(cfg), C.c_void_p(shadow.data_ptr()), C.byref(acc),
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == L.HY_ERR_TOO_LARGE
    assert "scratch" in lib.hy_error_string(rc).decode()
    # the running-mean branch needs no scratch and accepts the same size
    cfg = pass_config(accum_frame=2)
    assert lib.hy_accumulate_pass_noalloc(C.byref(gb), C.byref(cfg), C.c_void_p(shadow.data_ptr()), C.byref(acc),
                                          C.c_void_p(torch.cuda.current_stream().cuda_stream)) == L.HY_OK
    torch.cuda.synchronize()
