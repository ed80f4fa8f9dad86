"""Python host API over the C ABI (include/hybridrt.h).

``HybridContext`` is the counterpart of the hybrid part of VkPinut's
``Renderer``: it takes a ``Scene`` (what Renderer::load_data_to_gpu and
create_hybrid_descriptors upload, src/renderer.cpp:1477-1530, 3015-3048),
builds the acceleration structure (create_bottom/top_acceleration_structure,
src/renderer.cpp:1643-1688) and runs the pass that rasterize_hybrid submits
(src/renderer.cpp:559-580).  Device buffers are torch CUDA tensors, used as
plain memory; every computation runs in libhybridrt's CUDA kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from .scene import Scene


def _ptr(t) -> int:
    """Address of a packed tensor / array (the C ABI takes row-major planes without strides)."""
    if hasattr(t, "data_ptr"):
        if not t.is_contiguous():
            raise ValueError("the C ABI takes packed (contiguous) tensors")
        return t.data_ptr()
    if not t.flags["C_CONTIGUOUS"]:
        raise ValueError("the C ABI takes packed (C-contiguous) arrays")
    return t.ctypes.data


def _np_ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)


def camera_struct(cam36) -> L.HyCamera:
    cam = np.ascontiguousarray(cam36, np.float32)
    c = L.HyCamera()
    C.memmove(C.byref(c), cam.ctypes.data, 144)
    return c


def pass_config(spp=1, max_bounces=8, rng_mode=L.HY_RNG_REFERENCE, accum_frame=0, flags=0, block_size=0,
                queue_chunk=0, stack_depth=0, min_blocks=0, group_lanes=0, visits_per_round=0) -> L.HyPassConfig:
    return L.HyPassConfig(spp, max_bounces, rng_mode, accum_frame, flags, block_size, queue_chunk, stack_depth,
                          group_lanes, min_blocks, visits_per_round)


GBUF_FP32_FORMATS = (L.HY_FMT_RGBA32F, L.HY_FMT_RGBA32F, L.HY_FMT_RGBA32F, L.HY_FMT_RG32F, L.HY_FMT_RGBA32F,
                     L.HY_FMT_RGBA32F)


def gbuffer_struct(planes, width, height, formats=GBUF_FP32_FORMATS) -> L.HyGBuffer:
    g = L.HyGBuffer()
    g.width, g.height = width, height
    for i in range(6):
        g.plane[i] = _ptr(planes[i])
        g.format[i] = formats[i]
    return g


class HybridContext:
    """One device context: scene, BVH, and the hybrid pass."""

    def __init__(self, device: int = 0, stream: int | None = None, max_device_bytes: int = 0):
        self.lib = L.load()
        self.device = device
        info = L.HyCreateInfo(device, 0, stream, max_device_bytes)
        h = C.c_void_p()
        L.check(self.lib.hy_create(C.byref(h), C.byref(info)), "hy_create")
        self.h = h
        self.num_lights = 0
        self.num_mats = 0
        self.num_tris = 0

    def close(self):
        if getattr(self, "h", None):
            self.lib.hy_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- scene ----
    def set_scene_arrays(self, verts, idx, prims, xf, mats, lights, env=None):
        self._keep = (verts, idx, prims, xf, mats, lights)
        L.check(self.lib.hy_scene_set_geometry(self.h, _np_ptr(verts), len(verts), _np_ptr(idx), len(idx),
                                               _np_ptr(prims), len(prims), _np_ptr(xf), len(xf)), "geometry")
        L.check(self.lib.hy_scene_set_materials(self.h, _np_ptr(mats), len(mats)), "materials")
        L.check(self.lib.hy_scene_set_lights(self.h, _np_ptr(lights) if len(lights) else None, len(lights)),
                "lights")
        for slot, e in enumerate(env or []):
            e = np.ascontiguousarray(e, np.uint8)
            L.check(self.lib.hy_scene_set_env(self.h, slot, _np_ptr(e), e.shape[1], e.shape[0]), "env")
        self.num_lights = len(lights)
        self.num_mats = len(mats)
        self.num_tris = int(sum(int(p[1]) // 3 for p in prims))

    def set_scene(self, scene: Scene):
        verts, idx, prims, xf, mats, lights = scene.pack()
        self.set_scene_arrays(verts, idx, prims, xf, mats, lights, scene.env)
        if scene.textures:
            self.set_textures(scene.textures)

    def set_textures(self, textures):
        """Material textures (Texture::_textures): (H, W, 4) uint8 RGBA8 images, indexed by the
        materials' texture ids."""
        texs = [np.ascontiguousarray(t, np.uint8) for t in textures]
        self._tex = texs
        n = len(texs)
        ptrs = (C.c_void_p * max(n, 1))(*[t.ctypes.data for t in texs])
        w = (C.c_uint32 * max(n, 1))(*[t.shape[1] for t in texs])
        h = (C.c_uint32 * max(n, 1))(*[t.shape[0] for t in texs])
        L.check(self.lib.hy_scene_set_textures(self.h, ptrs, w, h, n), "textures")

    def set_lights(self, lights: np.ndarray):
        lights = np.ascontiguousarray(lights, np.float32)
        L.check(self.lib.hy_scene_set_lights(self.h, _np_ptr(lights), len(lights)), "lights")
        self.num_lights = len(lights)

    def set_materials(self, mats: np.ndarray):
        mats = np.ascontiguousarray(mats, np.float32)
        L.check(self.lib.hy_scene_set_materials(self.h, _np_ptr(mats), len(mats)), "materials")
        self.num_mats = len(mats)

    def build_bvh(self, instanced: bool = False) -> dict:
        """One BVH8 over the world-space triangles, or (instanced) one BLAS per
        distinct mesh under a TLAS over the primitives."""
        st = L.HyBvhStats()
        fn = self.lib.hy_bvh_build_instanced if instanced else self.lib.hy_bvh_build
        L.check(fn(self.h, C.byref(st)), "bvh_build")
        return {"num_tris": st.num_tris, "num_bvh2_nodes": st.num_bvh2_nodes, "num_bvh8_nodes": st.num_bvh8_nodes,
                "depth": st.depth, "build_ms": st.build_ms, "scene_lo": list(st.scene_lo),
                "scene_hi": list(st.scene_hi)}

    def bvh_layout(self) -> dict:
        lay = L.HyBvhLayout()
        L.check(self.lib.hy_bvh_layout(self.h, C.byref(lay)), "bvh_layout")
        return {k: int(getattr(lay, k)) for k, _ in L.HyBvhLayout._fields_}

    def set_build_mode(self, mode: int):
        """hy_scene_set_build_mode: HY_BUILD_SAH (default) or HY_BUILD_LBVH, from the next build."""
        L.check(self.lib.hy_scene_set_build_mode(self.h, mode), "set_build_mode")

    def set_anyhit_order(self, order: int):
        """hy_scene_set_anyhit_order: HY_ANYHIT_AUTO (default), FAR_FIRST or NEAR_FIRST."""
        L.check(self.lib.hy_scene_set_anyhit_order(self.h, order), "set_anyhit_order")

    def anyhit_order(self) -> int:
        """The order passes use now: HY_ANYHIT_FAR_FIRST or HY_ANYHIT_NEAR_FIRST."""
        v = C.c_uint32()
        L.check(self.lib.hy_scene_anyhit_order(self.h, C.byref(v)), "anyhit_order")
        return int(v.value)

    def download_bvh_instanced(self):
        """(layout, nodes [num_nodes, 20] u32, records [num_records, 12] f32,
        instances [num_instances, 16] f32, instance boxes [num_instances, 6] f32)"""
        lay = self.bvh_layout()
        nodes = np.zeros((lay["num_nodes"], 20), np.uint32)
        recs = np.zeros((lay["num_records"], 12), np.float32)
        inst = np.zeros((lay["num_instances"], 16), np.float32)
        boxes = np.zeros((lay["num_instances"], 6), np.float32)
        L.check(self.lib.hy_bvh_download(self.h, None, None, None, _np_ptr(nodes), _np_ptr(recs)), "bvh_download")
        L.check(self.lib.hy_bvh_download_instances(self.h, _np_ptr(inst), _np_ptr(boxes)), "bvh_download_instances")
        return lay, nodes, recs, inst, boxes

    def refit_bvh(self, transforms: np.ndarray):
        """New column-major transforms, same topology (the per-frame TLAS update)."""
        xf = np.ascontiguousarray(transforms, np.float32).reshape(-1, 16)
        L.check(self.lib.hy_bvh_refit(self.h, _np_ptr(xf), len(xf)), "bvh_refit")

    def download_bvh(self, n_bvh8: int):
        n = self.num_tris
        morton = np.zeros(n, np.uint32)
        order = np.zeros(n, np.uint32)
        bvh2 = np.zeros((max(n - 1, 0), 10), np.uint32)
        bvh8 = np.zeros((n_bvh8, 20), np.uint32)
        tris = np.zeros((n, 12), np.float32)
        L.check(self.lib.hy_bvh_download(self.h, _np_ptr(morton), _np_ptr(order), _np_ptr(bvh2), _np_ptr(bvh8),
                                         _np_ptr(tris)), "bvh_download")
        return morton, order, bvh2, bvh8, tris

    # ---- queries ----
    def trace(self, rays, any_hit: bool, count: bool = False):
        """rays: CUDA float32 tensor (n, 8); returns (hits int32/float32 view (n, 4) tensor, stats)."""
        import torch
        n = rays.shape[0]
        hits = torch.empty((n, 4), dtype=torch.float32, device=rays.device)
        st = L.HyStats()
        L.check(self.lib.hy_trace_rays(self.h, C.c_void_p(_ptr(rays)), n, int(any_hit),
                                       C.c_void_p(_ptr(hits)), C.byref(st) if count else None), "trace")
        return hits, st.as_dict()

    def gbuffer(self, cam36, width: int, height: int):
        import torch
        dev = torch.device("cuda", self.device)
        planes = [torch.empty((height, width, 4 if i != 3 else 2), dtype=torch.float32, device=dev)
                  for i in range(6)]
        arr = (C.c_void_p * 6)(*[_ptr(p) for p in planes])
        cam = camera_struct(cam36)
        L.check(self.lib.hy_gbuffer_primary(self.h, C.byref(cam), width, height, arr), "gbuffer")
        return planes

    # ---- the pass ----
    def new_history(self, width, height, fmt=L.HY_ACCUM_U8, fill=0):
        import torch
        dt = torch.uint8 if fmt == L.HY_ACCUM_U8 else torch.float32
        return torch.full((self.num_lights, height, width), fill, dtype=dt, device=torch.device("cuda", self.device))

    @staticmethod
    def _accum(hist, fmt):
        return L.HyAccum(fmt, hist.shape[0], _ptr(hist))

    def forward(self, planes, cam36, cfg: L.HyPassConfig, hist, fmt=L.HY_ACCUM_U8, out_f=None, out_8=None,
                formats=GBUF_FP32_FORMATS, stats: bool = True):
        """hy_hybrid_forward.  stats=False with HY_FLAG_NO_STATUS_SYNC in cfg returns without a host sync."""
        h, w = planes[0].shape[0], planes[0].shape[1]
        gb = gbuffer_struct(planes, w, h, formats)
        cam = camera_struct(cam36)
        acc = self._accum(hist, fmt)
        st = L.HyStats()
        L.check(self.lib.hy_hybrid_forward(self.h, C.byref(gb), C.byref(cam), C.byref(cfg), C.byref(acc),
                                           C.c_void_p(_ptr(out_f)) if out_f is not None else None,
                                           C.c_void_p(_ptr(out_8)) if out_8 is not None else None,
                                           C.byref(st) if stats else None), "hybrid_forward")
        return st.as_dict()

    def forward_host(self, planes_np, cam36, cfg, hist, fmt=L.HY_ACCUM_U8, out_f=None, out_8=None,
                     formats=GBUF_FP32_FORMATS, stats=True):
        """Host planes / outputs (numpy or pinned CPU tensors); history stays on the device."""
        h, w = planes_np[0].shape[0], planes_np[0].shape[1]
        gb = gbuffer_struct(planes_np, w, h, formats)
        cam = camera_struct(cam36)
        acc = self._accum(hist, fmt)
        st = L.HyStats()
        L.check(self.lib.hy_hybrid_forward_host(self.h, C.byref(gb), C.byref(cam), C.byref(cfg), C.byref(acc),
                                                C.c_void_p(_ptr(out_f)) if out_f is not None else None,
                                                C.c_void_p(_ptr(out_8)) if out_8 is not None else None,
                                                C.byref(st) if stats else None), "hybrid_forward_host")
        return st.as_dict()

    def shadow_pass(self, planes, cam36, cfg, shadow, fmt=L.HY_ACCUM_U8, formats=GBUF_FP32_FORMATS):
        h, w = planes[0].shape[0], planes[0].shape[1]
        gb = gbuffer_struct(planes, w, h, formats)
        cam = camera_struct(cam36)
        st = L.HyStats()
        L.check(self.lib.hy_shadow_pass(self.h, C.byref(gb), C.byref(cam), C.byref(cfg), fmt,
                                        C.c_void_p(_ptr(shadow)), C.byref(st)), "shadow_pass")
        return st.as_dict()

    def accumulate_pass(self, planes, cfg, shadow, hist, fmt=L.HY_ACCUM_U8, formats=GBUF_FP32_FORMATS):
        h, w = planes[0].shape[0], planes[0].shape[1]
        gb = gbuffer_struct(planes, w, h, formats)
        acc = self._accum(hist, fmt)
        L.check(self.lib.hy_accumulate_pass(self.h, C.byref(gb), C.byref(cfg), C.c_void_p(_ptr(shadow)),
                                            C.byref(acc)), "accumulate_pass")

    def shade_pass(self, planes, cam36, cfg, hist, fmt=L.HY_ACCUM_U8, out_f=None, out_8=None,
                   formats=GBUF_FP32_FORMATS):
        h, w = planes[0].shape[0], planes[0].shape[1]
        gb = gbuffer_struct(planes, w, h, formats)
        cam = camera_struct(cam36)
        acc = self._accum(hist, fmt)
        st = L.HyStats()
        L.check(self.lib.hy_shade_pass(self.h, C.byref(gb), C.byref(cam), C.byref(cfg), C.byref(acc),
                                       C.c_void_p(_ptr(out_f)) if out_f is not None else None,
                                       C.c_void_p(_ptr(out_8)) if out_8 is not None else None,
                                       C.byref(st)), "shade_pass")
        return st.as_dict()

    def pathtrace(self, cam36, width: int, height: int, cfg, image=None, out_f=None, stats: bool = True):
        """hy_pathtrace_pass: the reference's path-traced mode into the BGRA8 image `image`
        (device (H, W, 4) uint8, accumulated in place; allocated when None) and the frame's
        colour into out_f (device (H, W, 4) float32, optional).  Returns (image, stats)."""
        import torch
        if image is None:
            image = torch.zeros((height, width, 4), dtype=torch.uint8, device=torch.device("cuda", self.device))
            torch.cuda.synchronize(self.device)  # the fill runs on torch's stream
        cam = camera_struct(cam36)
        st = L.HyStats()
        L.check(self.lib.hy_pathtrace_pass(self.h, C.byref(cam), width, height, C.byref(cfg),
                                           C.c_void_p(_ptr(image)),
                                           C.c_void_p(_ptr(out_f)) if out_f is not None else None,
                                           C.byref(st) if stats else None), "pathtrace_pass")
        return image, st.as_dict()

    def post(self, image, out=None):
        """hy_post_resolve: gamma 1/2.2 of the pass's BGRA8 image (uint8 (H, W, 4)) or float image
        (float32 (H, W, 4)) into a BGRA8 image."""
        import torch
        h, w = image.shape[0], image.shape[1]
        if out is None:
            out = torch.empty((h, w, 4), dtype=torch.uint8, device=image.device)
        is8 = image.dtype == torch.uint8
        if not is8 and image.dtype != torch.float32:
            raise TypeError("post expects a uint8 BGRA8 or float32 RGBA image")
        if not image.is_contiguous():  # the kernel reads packed (H, W, 4) texels
            image = image.contiguous()
            torch.cuda.synchronize(image.device)  # the copy ran on torch's stream
        if not out.is_contiguous():
            raise ValueError("post writes a packed (H, W, 4) image")
        L.check(self.lib.hy_post_resolve(self.h, w, h, C.c_void_p(_ptr(image)) if is8 else None,
                                         None if is8 else C.c_void_p(_ptr(image)),
                                         C.c_void_p(_ptr(out))), "post_resolve")
        return out

    def backward(self, planes, cam36, cfg, hist, grad_img, fmt=L.HY_ACCUM_U8, grad_mats=None, grad_lights=None,
                 formats=GBUF_FP32_FORMATS, stats: bool = True):
        """hy_hybrid_backward: dLoss/dImage (device (H, W, 4) float32) -> gradients with respect to the
        materials (num_mats, 5: diffuse rgb, roughness, metallic) and lights (num_lights, 4: position,
        intensity), visibility held fixed.  Returns (grad_mats, grad_lights, stats)."""
        import torch
        h, w = planes[0].shape[0], planes[0].shape[1]
        dev = grad_img.device
        if grad_mats is None:
            grad_mats = torch.empty((self.num_mats, L.HY_GRAD_MATERIAL_PARAMS), dtype=torch.float32, device=dev)
        if grad_lights is None:
            grad_lights = torch.empty((max(self.num_lights, 1), L.HY_GRAD_LIGHT_PARAMS), dtype=torch.float32,
                                      device=dev)
        gb = gbuffer_struct(planes, w, h, formats)
        cam = camera_struct(cam36)
        acc = self._accum(hist, fmt)
        st = L.HyStats()
        L.check(self.lib.hy_hybrid_backward(self.h, C.byref(gb), C.byref(cam), C.byref(cfg), C.byref(acc),
                                            C.c_void_p(_ptr(grad_img)), C.c_void_p(_ptr(grad_mats)),
                                            C.c_void_p(_ptr(grad_lights)), C.byref(st) if stats else None),
                "hybrid_backward")
        return grad_mats, grad_lights[: self.num_lights], st.as_dict()

    def _views(self, scenes, views):
        arr = (C.c_void_p * len(scenes))(*[s.h.value for s in scenes])
        vs = (L.HyView * len(views))()
        keep = []
        for i, v in enumerate(views):
            planes = v["planes"]
            h, w = planes[0].shape[0], planes[0].shape[1]
            vs[i].scene = v["scene"]
            vs[i].gbuffer = gbuffer_struct(planes, w, h, v.get("formats", GBUF_FP32_FORMATS))
            vs[i].camera = camera_struct(v["camera"])
            vs[i].config = v["config"]
            vs[i].accum = self._accum(v["hist"], v.get("fmt", L.HY_ACCUM_U8))
            vs[i].out_rgba32f = _ptr(v["out_f"]) if v.get("out_f") is not None else None
            vs[i].out_bgra8 = _ptr(v["out_8"]) if v.get("out_8") is not None else None
            keep.append(planes)
        return arr, vs, keep

    def batch_forward(self, scenes, views, graph: bool = True, tuning: L.HyPassConfig | None = None,
                      sync: bool = True):
        """One batch of views over scene contexts (hy_batch_forward).

        views: list of dicts with keys scene, planes, camera (36 floats), config
        (HyPassConfig), hist, fmt and optionally out_f / out_8 (device tensors).
        """
        arr, vs, keep = self._views(scenes, views)
        flags = (0 if graph else L.HY_BATCH_NO_GRAPH) | (0 if sync else L.HY_BATCH_NO_STATUS_SYNC)
        st = L.HyStats()
        L.check(self.lib.hy_batch_forward(self.h, arr, len(scenes), vs, len(views), flags,
                                          C.byref(tuning) if tuning is not None else None,
                                          C.byref(st) if sync else None), "batch_forward")
        return st.as_dict()

    def batch_autotune(self, scenes, views, reps: int = 2):
        """hy_batch_autotune: the fastest launch shape of the batch, (HyPassConfig, ms).
        Runs the batch many times (its histories and outputs are overwritten)."""
        arr, vs, keep = self._views(scenes, views)
        tuning = L.HyPassConfig()
        ms = C.c_float()
        L.check(self.lib.hy_batch_autotune(self.h, arr, len(scenes), vs, len(views), reps, C.byref(tuning),
                                           C.byref(ms)), "batch_autotune")
        return tuning, ms.value

    def synchronize(self):
        L.check(self.lib.hy_synchronize(self.h), "synchronize")

    # ---- per-kernel timing ----
    def profile(self, enable: bool = True):
        L.check(self.lib.hy_profile_enable(self.h, int(enable)), "profile_enable")

    def profile_read(self) -> dict:
        """{kernel: {"launches": n, "total_ms": t, "avg_ms": t / n}} since the last read / enable."""
        buf = (L.HyKernelTime * 16)()
        n = C.c_uint32()
        L.check(self.lib.hy_profile_read(self.h, buf, 16, C.byref(n)), "profile_read")
        out = {}
        for i in range(min(n.value, 16)):
            k = buf[i]
            out[k.kernel.decode()] = {"launches": k.launches, "total_ms": k.total_ms,
                                      "avg_ms": k.total_ms / max(k.launches, 1)}
        return out
