"""Gradient-check harness: the hybrid pass's forward/backward pair
(hy_shade_pass / hy_hybrid_backward through DiffRenderer) wrapped in a
``torch.autograd.Function``.  Test code only; the product exposes the pair
through the C ABI.
"""
from __future__ import annotations


def _autograd_function():
    import torch

    class HybridRenderFn(torch.autograd.Function):
        """image[..., :3] = shade(materials, lights); backward = hy_hybrid_backward."""

        @staticmethod
        def forward(ctx, mat_p, light_p, renderer):
            img, state = renderer.render(mat_p.detach().cpu().numpy(), light_p.detach().cpu().numpy())
            ctx.renderer = renderer
            ctx.state = state
            ctx.shapes = (mat_p.shape, light_p.shape, mat_p.device, light_p.device, mat_p.dtype)
            return img[..., :3]

        @staticmethod
        def backward(ctx, grad):
            r = ctx.renderer
            g4 = torch.zeros((r.H, r.W, 4), dtype=torch.float32, device=r.dev)
            g4[..., :3] = grad
            gm, gl, _ = r.backward(ctx.state, g4)
            ms, ls, md, ld, dt = ctx.shapes
            return gm.reshape(ms).to(md, dt), gl.reshape(ls).to(ld, dt), None

    return HybridRenderFn


def render_fn():
    """The torch.autograd.Function of the gradient-check harness:
    ``render_fn().apply(mat_params, light_params, renderer)``."""
    return _autograd_function()
