"""Differentiable form of the hybrid pass: the host side of the
forward/backward pair.

The product interface is the C ABI pair hy_shade_pass (forward, after
hy_gbuffer_primary and hy_shadow_pass) and hy_hybrid_backward (its adjoint,
visibility held fixed).  This module names the parameters the gradient
covers and renders an image from a parameter vector; it has no autograd
code (the ``torch.autograd.Function`` of the gradient check lives with the
tests, tests/grad_harness.py).

Parameters (float32):
  materials (num_mats, 5): HyMaterial diffuse[0..2], roughness (smr[2]),
      metallic (smr[1]) -- the values Material::materialToShader writes
      (src/material.cpp:19-26);
  lights (num_lights, 4): uboLight pos.xyz and intensity color.w
      (src/vk_engine.cpp:146-164).
"""
from __future__ import annotations

import numpy as np

from . import _lib as L
from .hybrid import HybridContext, pass_config

MATERIAL_FIELDS = (0, 1, 2, 10, 9)   # floats of a HyMaterial row
LIGHT_FIELDS = (0, 1, 2, 7)          # floats of a HyLight row


def material_params(mats: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(mats, np.float32)[:, MATERIAL_FIELDS])


def with_material_params(mats: np.ndarray, params: np.ndarray) -> np.ndarray:
    out = np.array(mats, np.float32, copy=True)
    out[:, MATERIAL_FIELDS] = np.asarray(params, np.float32)
    return out


def light_params(lights: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(lights, np.float32)[:, LIGHT_FIELDS])


def with_light_params(lights: np.ndarray, params: np.ndarray) -> np.ndarray:
    out = np.array(lights, np.float32, copy=True)
    out[:, LIGHT_FIELDS] = np.asarray(params, np.float32)
    return out


class DiffRenderer:
    """A scene whose materials and lights are variables.

    ``render(mat_p, light_p)`` uploads the parameters, makes the G-buffer
    (hy_gbuffer_primary), the per-light shadow images (hy_shadow_pass,
    F32 so a pixel's visibility is its exact unoccluded-sample fraction) and
    the shaded image (hy_shade_pass); ``backward`` runs hy_hybrid_backward on
    what that render produced.  The context runs on torch's current stream so
    tensors move between the two without extra synchronisation."""

    def __init__(self, scene, cam36, width: int, height: int, spp: int = 16, max_bounces: int = 1,
                 rng_mode: int = L.HY_RNG_DECORRELATED, device: int = 0):
        import torch
        self.torch = torch
        self.dev = torch.device("cuda", device)
        stream = torch.cuda.current_stream(self.dev).cuda_stream
        self.ctx = HybridContext(device, stream=stream)
        self.ctx.set_scene(scene)
        self.ctx.build_bvh()
        verts, idx, prims, xf, mats, lights = scene.pack()
        self.mats_rows, self.light_rows = mats, lights
        self.cam = np.ascontiguousarray(cam36, np.float32)
        self.W, self.H = width, height
        self.cfg = pass_config(spp=spp, max_bounces=max_bounces, rng_mode=rng_mode)
        self.fmt = L.HY_ACCUM_F32

    @property
    def params0(self):
        return material_params(self.mats_rows), light_params(self.light_rows)

    def set_params(self, mat_p, light_p):
        self.ctx.set_materials(with_material_params(self.mats_rows, mat_p))
        self.ctx.set_lights(with_light_params(self.light_rows, light_p))

    def render(self, mat_p, light_p):
        """Returns (image (H, W, 4) float32 device tensor, state for backward)."""
        torch = self.torch
        self.set_params(mat_p, light_p)
        planes = self.ctx.gbuffer(self.cam, self.W, self.H)
        shadow = torch.zeros((self.ctx.num_lights, self.H, self.W), dtype=torch.float32, device=self.dev)
        self.ctx.shadow_pass(planes, self.cam, self.cfg, shadow, self.fmt)
        img = torch.empty((self.H, self.W, 4), dtype=torch.float32, device=self.dev)
        self.ctx.shade_pass(planes, self.cam, self.cfg, shadow, self.fmt, out_f=img)
        return img, (planes, shadow)

    def backward(self, state, grad_img):
        planes, shadow = state
        g = grad_img.contiguous()
        gm, gl, st = self.ctx.backward(planes, self.cam, self.cfg, shadow, g, self.fmt)
        return gm, gl, st

    def close(self):
        self.ctx.close()
