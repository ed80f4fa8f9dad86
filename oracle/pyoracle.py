"""ORACLE — test infrastructure only.

ctypes front end of liboracle.so, the CPU restatement of the hybrid pass.
Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline use it, as
the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"

P = C.c_void_p
U32 = C.c_uint32
_lib = None


def build() -> Path:
    r = subprocess.run(["make", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not LIB.exists():
        build()
    lib = C.CDLL(str(LIB))
    sig = {
        "orc_scene_create": (P, []),
        "orc_scene_destroy": (None, [P]),
        "orc_set_threads": (None, [C.c_int]),
        "orc_get_threads": (C.c_int, []),
        "orc_scene_set_geometry": (C.c_int, [P, P, U32, P, U32, P, U32, P, U32]),
        "orc_scene_set_materials": (C.c_int, [P, P, U32]),
        "orc_scene_set_lights": (C.c_int, [P, P, U32]),
        "orc_scene_set_env": (C.c_int, [P, C.c_int, P, U32, U32]),
        "orc_scene_set_textures": (C.c_int, [P, P, P, P, U32]),
        "orc_num_tris": (U32, [P]),
        "orc_world_tris": (None, [P, P]),
        "orc_bvh_build": (C.c_int, [P, P, P]),
        "orc_bvh_download": (None, [P, P, P, P, P, P]),
        "orc_bvh_refit": (C.c_int, [P, P, U32]),
        "orc_bvh_build_instanced": (C.c_int, [P, P]),
        "orc_scene_set_anyhit_order": (C.c_int, [P, U32]),
        "orc_scene_set_build_mode": (C.c_int, [P, U32]),
        "orc_bvh_download_instanced": (None, [P, P, P, P, P, P]),
        "orc_trace": (None, [P, P, U32, C.c_int, C.c_int, P, P]),
        "orc_tea": (U32, [U32, U32]),
        "orc_rnd_seq": (None, [U32, U32, P, P]),
        "orc_sample_disk": (None, [P, P, P, U32, P]),
        "orc_brdf": (None, [P, P, P, C.c_float, P, C.c_float, P]),
        "orc_ggx_reflect": (None, [P, P, C.c_float, C.c_float, C.c_float, C.c_int, P]),
        "orc_gbuffer_primary": (C.c_int, [P, P, U32, U32, P, C.c_int]),
        "orc_shadow_pass": (C.c_int, [P, P, P, P, U32, P, C.c_int, P]),
        "orc_accumulate": (C.c_int, [P, P, P, P, P]),
        "orc_shade": (C.c_int, [P, P, P, P, P, P, P, C.c_int, P]),
        "orc_pathtrace": (C.c_int, [P, P, U32, U32, P, P, P, C.c_int, P]),
        "orc_post_resolve": (None, [U32, P, P, P]),
        "orc_grad_record": (P, [P, P, P, P, P, C.c_int]),
        "orc_grad_free": (None, [P]),
        "orc_grad_forward": (C.c_int, [P, P, P, P, P]),
        "orc_grad_adjoint": (C.c_int, [P, P, P, P, P, P, P]),
    }
    for k, (r, a) in sig.items():
        f = getattr(lib, k)
        f.restype = r
        f.argtypes = a
    _lib = lib
    return lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"], "arrays must be C-contiguous"
    return C.c_void_p(a.ctypes.data)


# mirrors of the C structs (same layout as include/hybridrt.h)
class _GBuf(C.Structure):
    _fields_ = [("width", U32), ("height", U32), ("plane", C.c_void_p * 6), ("format", U32 * 6)]


class _Cfg(C.Structure):
    _fields_ = [("shadow_spp", U32), ("max_bounces", U32), ("rng_mode", U32), ("accum_frame", C.c_int32),
                ("flags", U32), ("block_size", U32), ("queue_chunk", U32), ("stack_depth", U32), ("group_lanes", U32),
                ("min_blocks", U32), ("visits_per_round", U32)]


class _Accum(C.Structure):
    _fields_ = [("format", U32), ("num_lights", U32), ("history", C.c_void_p)]


class _Stats(C.Structure):
    _fields_ = [("shadow_rays", C.c_uint64), ("reflection_rays", C.c_uint64), ("hit_shadow_rays", C.c_uint64),
                ("nodes_visited", C.c_uint64), ("tris_tested", C.c_uint64), ("error_flags", U32), ("_pad", U32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if not k.startswith("_")}


FP32_FORMATS = (0, 0, 0, 1, 0, 0)
TRACE_BRUTE, TRACE_BVH8 = 0, 1
HY_ANYHIT_AUTO, HY_ANYHIT_FAR_FIRST, HY_ANYHIT_NEAR_FIRST = 0, 1, 2  # any-hit child orders
HY_BUILD_SAH, HY_BUILD_LBVH = 0, 1  # binary tree under the 8-wide nodes


def set_threads(n: int):
    load().orc_set_threads(n)


def threads() -> int:
    return load().orc_get_threads()


def tea(a: int, b: int) -> int:
    return int(load().orc_tea(a, b))


def rnd_seq(seed: int, n: int):
    st = np.zeros(n, np.uint32)
    v = np.zeros(n, np.float32)
    load().orc_rnd_seq(seed, n, _p(st), _p(v))
    return st, v


def sample_disk(radius: float, pos, L, seed: int) -> np.ndarray:
    r = np.array([radius], np.float32)
    p = np.ascontiguousarray(pos, np.float32)
    l = np.ascontiguousarray(L, np.float32)
    out = np.zeros(3, np.float32)
    load().orc_sample_disk(_p(r), _p(p), _p(l), seed, _p(out))
    return out


def brdf(N, V, L, roughness, F0, cos_theta):
    out = np.zeros(5, np.float32)
    a = [np.ascontiguousarray(x, np.float32) for x in (N, V, L, F0)]
    load().orc_brdf(_p(a[0]), _p(a[1]), _p(a[2]), float(roughness), _p(a[3]), float(cos_theta), _p(out))
    return out


def ggx_reflect(N, V, roughness, u1, u2, double=False) -> np.ndarray:
    """The GGX-sampled reflection direction (HY_FLAG_GGX_REFLECTION) for one texel."""
    n = np.ascontiguousarray(N, np.float32)
    v = np.ascontiguousarray(V, np.float32)
    out = np.zeros(3, np.float32)
    load().orc_ggx_reflect(_p(n), _p(v), float(roughness), float(u1), float(u2), int(double), _p(out))
    return out


class OracleScene:
    def __init__(self):
        self.lib = load()
        self.h = self.lib.orc_scene_create()
        self.num_lights = 0

    def __del__(self):
        try:
            if self.h:
                self.lib.orc_scene_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def set_scene_arrays(self, verts, idx, prims, xf, mats, lights, env=None):
        self._keep = (verts, idx, prims, xf, mats, lights)
        self.lib.orc_scene_set_geometry(self.h, _p(verts), len(verts), _p(idx), len(idx), _p(prims), len(prims),
                                        _p(xf), len(xf))
        self.lib.orc_scene_set_materials(self.h, _p(mats), len(mats))
        self.lib.orc_scene_set_lights(self.h, _p(lights) if len(lights) else None, len(lights))
        for slot, e in enumerate(env or []):
            e = np.ascontiguousarray(e, np.uint8)
            self.lib.orc_scene_set_env(self.h, slot, _p(e), e.shape[1], e.shape[0])
        self.num_lights = len(lights)

    def set_scene(self, scene):
        self.set_scene_arrays(*scene.pack(), scene.env)
        if getattr(scene, "textures", None):
            self.set_textures(scene.textures)

    def set_textures(self, textures):
        """textures: list of (H, W, 4) uint8 RGBA8 images, indexed by the materials' texture ids."""
        texs = [np.ascontiguousarray(t, np.uint8) for t in textures]
        self._tex = texs
        n = len(texs)
        ptrs = (C.c_void_p * max(n, 1))(*[t.ctypes.data for t in texs])
        w = np.array([t.shape[1] for t in texs] or [0], np.uint32)
        h = np.array([t.shape[0] for t in texs] or [0], np.uint32)
        self.lib.orc_scene_set_textures(self.h, ptrs, _p(w), _p(h), n)

    def set_lights(self, lights):
        lights = np.ascontiguousarray(lights, np.float32)
        self._lights = lights
        self.lib.orc_scene_set_lights(self.h, _p(lights), len(lights))
        self.num_lights = len(lights)

    def set_materials(self, mats):
        mats = np.ascontiguousarray(mats, np.float32)
        self._mats = mats
        self.lib.orc_scene_set_materials(self.h, _p(mats), len(mats))

    @property
    def num_tris(self) -> int:
        return int(self.lib.orc_num_tris(self.h))

    def world_tris(self) -> np.ndarray:
        out = np.zeros((self.num_tris, 9), np.float32)
        self.lib.orc_world_tris(self.h, _p(out))
        return out

    def build_bvh(self):
        info = np.zeros(4, np.uint32)
        b = np.zeros(6, np.float32)
        rc = self.lib.orc_bvh_build(self.h, _p(info), _p(b))
        if rc != 0:
            raise RuntimeError("oracle bvh build failed")
        return {"num_tris": int(info[0]), "num_bvh2_nodes": int(info[1]), "num_bvh8_nodes": int(info[2]),
                "depth": int(info[3]), "scene_lo": b[:3].tolist(), "scene_hi": b[3:].tolist()}

    LAYOUT_FIELDS = ("two_level", "num_nodes", "num_records", "num_instances", "num_blas", "tlas_region",
                     "tlas_nodes", "depth")

    def set_build_mode(self, mode: int):
        """Binary tree of the next build: HY_BUILD_SAH (default) or HY_BUILD_LBVH."""
        if self.lib.orc_scene_set_build_mode(self.h, mode) != 0:
            raise ValueError(f"bad build mode {mode}")

    def set_anyhit_order(self, order: int):
        """Child order of any-hit traversal (HY_ANYHIT_AUTO / FAR_FIRST / NEAR_FIRST)."""
        if self.lib.orc_scene_set_anyhit_order(self.h, order) != 0:
            raise ValueError(f"bad any-hit order {order}")

    def build_bvh_instanced(self):
        """Two-level structure: one BLAS per distinct mesh, a TLAS over the instances."""
        lay = np.zeros(8, np.uint32)
        if self.lib.orc_bvh_build_instanced(self.h, _p(lay)) != 0:
            raise RuntimeError("oracle two-level build failed")
        return dict(zip(self.LAYOUT_FIELDS, (int(v) for v in lay)))

    def download_bvh_instanced(self):
        """(layout, nodes [num_nodes, 20] u32, records [num_records, 12] f32,
        instances [num_instances, 16] f32, instance boxes [num_instances, 6] f32)"""
        lay = np.zeros(8, np.uint32)
        self.lib.orc_bvh_download_instanced(self.h, _p(lay), None, None, None, None)
        L = dict(zip(self.LAYOUT_FIELDS, (int(v) for v in lay)))
        nodes = np.zeros((L["num_nodes"], 20), np.uint32)
        recs = np.zeros((L["num_records"], 12), np.float32)
        inst = np.zeros((L["num_instances"], 16), np.float32)
        boxes = np.zeros((L["num_instances"], 6), np.float32)
        self.lib.orc_bvh_download_instanced(self.h, None, _p(nodes), _p(recs), _p(inst), _p(boxes))
        return L, nodes, recs, inst, boxes

    def refit_bvh(self, xf: np.ndarray):
        xf = np.ascontiguousarray(xf, np.float32)
        self._xf = xf
        if self.lib.orc_bvh_refit(self.h, _p(xf), len(xf)) != 0:
            raise RuntimeError("oracle refit needs a built BVH and the same transform count")

    def download_bvh(self, n_bvh8: int):
        n = self.num_tris
        morton = np.zeros(n, np.uint32)
        order = np.zeros(n, np.uint32)
        bvh2 = np.zeros((max(n - 1, 0), 10), np.uint32)
        bvh8 = np.zeros((n_bvh8, 20), np.uint32)
        tris = np.zeros((n, 12), np.float32)
        self.lib.orc_bvh_download(self.h, _p(morton), _p(order), _p(bvh2), _p(bvh8), _p(tris))
        return morton, order, bvh2, bvh8, tris

    def trace(self, rays: np.ndarray, any_hit: bool, mode: int = TRACE_BVH8):
        rays = np.ascontiguousarray(rays, np.float32)
        n = len(rays)
        hits = np.zeros((n, 4), np.float32)
        cnt = np.zeros((n, 2), np.uint32)
        self.lib.orc_trace(self.h, _p(rays), n, int(any_hit), mode, _p(hits), _p(cnt))
        return hits, cnt

    def gbuffer(self, cam36, width, height, mode=TRACE_BVH8):
        planes = [np.zeros((height, width, 4 if i != 3 else 2), np.float32) for i in range(6)]
        arr = (C.c_void_p * 6)(*[p.ctypes.data for p in planes])
        cam = np.ascontiguousarray(cam36, np.float32)
        self.lib.orc_gbuffer_primary(self.h, _p(cam), width, height, arr, mode)
        return planes

    @staticmethod
    def _gb(planes, formats=FP32_FORMATS):
        g = _GBuf()
        g.width, g.height = planes[0].shape[1], planes[0].shape[0]
        for i in range(6):
            g.plane[i] = planes[i].ctypes.data
            g.format[i] = formats[i]
        return g

    def shadow_pass(self, planes, cam36, cfg: dict, fmt: int, mode=TRACE_BVH8, formats=FP32_FORMATS):
        H, W = planes[0].shape[:2]
        dt = np.uint8 if fmt == 0 else np.float32
        out = np.zeros((self.num_lights, H, W), dt)
        st = _Stats()
        cam = np.ascontiguousarray(cam36, np.float32)
        self.lib.orc_shadow_pass(self.h, C.byref(self._gb(planes, formats)), _p(cam), C.byref(_Cfg(**cfg)), fmt,
                                 _p(out), mode, C.byref(st))
        return out, st.as_dict()

    def accumulate(self, planes, cfg: dict, shadow: np.ndarray, hist: np.ndarray, fmt: int, formats=FP32_FORMATS):
        acc = _Accum(fmt, hist.shape[0], hist.ctypes.data)
        self.lib.orc_accumulate(self.h, C.byref(self._gb(planes, formats)), C.byref(_Cfg(**cfg)), _p(shadow),
                                C.byref(acc))

    def shade(self, planes, cam36, cfg: dict, hist: np.ndarray, fmt: int, mode=TRACE_BVH8, formats=FP32_FORMATS):
        H, W = planes[0].shape[:2]
        out_f = np.zeros((H, W, 4), np.float32)
        out_8 = np.zeros((H, W, 4), np.uint8)
        acc = _Accum(fmt, hist.shape[0], hist.ctypes.data)
        st = _Stats()
        cam = np.ascontiguousarray(cam36, np.float32)
        self.lib.orc_shade(self.h, C.byref(self._gb(planes, formats)), _p(cam), C.byref(_Cfg(**cfg)), C.byref(acc),
                           _p(out_f), _p(out_8), mode, C.byref(st))
        return out_f, out_8, st.as_dict()

    def pathtrace(self, cam36, width: int, height: int, cfg: dict, image: np.ndarray | None = None,
                  mode=TRACE_BVH8):
        """Path-traced mode: returns (accumulated BGRA8 image (updated in place when given), the
        frame's RGBA32F colour before accumulation, stats)."""
        if image is None:
            image = np.zeros((height, width, 4), np.uint8)
        out_f = np.zeros((height, width, 4), np.float32)
        st = _Stats()
        cam = np.ascontiguousarray(cam36, np.float32)
        self.lib.orc_pathtrace(self.h, _p(cam), width, height, C.byref(_Cfg(**cfg)), _p(image), _p(out_f), mode,
                               C.byref(st))
        return image, out_f, st.as_dict()

    def forward(self, planes, cam36, cfg: dict, hist: np.ndarray, fmt: int, mode=TRACE_BVH8,
                formats=FP32_FORMATS):
        """shadow -> accumulate -> shade, the order of Renderer::rasterize_hybrid."""
        flags = cfg.get("flags", 0)
        shadow, st1 = self.shadow_pass(planes, cam36, cfg, fmt, mode, formats)
        if flags & 0x2:  # HY_FLAG_NO_ACCUM: shade from the raw images
            src = shadow
        else:
            self.accumulate(planes, cfg, shadow, hist, fmt, formats)
            src = hist
        out_f, out_8, st2 = self.shade(planes, cam36, cfg, src, fmt, mode, formats)
        st = {k: st1[k] + st2[k] for k in st1 if k != "error_flags"}
        st["error_flags"] = st1["error_flags"] | st2["error_flags"]
        return out_f, out_8, shadow, st


def post_resolve(image: np.ndarray) -> np.ndarray:
    """postFragment.frag on a BGRA8 (uint8) or RGBA32F (float32) (H, W, 4) image -> BGRA8."""
    img = np.ascontiguousarray(image)
    out = np.zeros(img.shape[:2] + (4,), np.uint8)
    n = img.shape[0] * img.shape[1]
    if img.dtype == np.uint8:
        load().orc_post_resolve(n, _p(img), None, _p(out))
    else:
        img = np.ascontiguousarray(img, np.float32)
        load().orc_post_resolve(n, None, _p(img), _p(out))
    return out


class GradOracle:
    """FP64 shading as a function of the scene parameters, visibility fixed.

    Records (in float, like the shading pass) the G-buffer geometry, bounce
    hits, bounce-hit shadow outcomes and light sides of every pixel from the
    scene as it is now, then evaluates the image in FP64 (`forward`) and the
    gradient of sum(w * image) (`adjoint`) for any parameter vector:
    mats (num_mats, 5) = diffuse rgb, roughness, metallic;
    lights (num_lights, 4) = position xyz, intensity."""

    def __init__(self, scene: "OracleScene", planes, cam36, cfg: dict, hist: np.ndarray, fmt: int,
                 mode=TRACE_BVH8, formats=FP32_FORMATS):
        self.scene = scene
        self.lib = scene.lib
        H, W = planes[0].shape[:2]
        self.shape = (H, W)
        self._hist = np.ascontiguousarray(hist)
        acc = _Accum(fmt, self._hist.shape[0], self._hist.ctypes.data)
        cam = np.ascontiguousarray(cam36, np.float32)
        self.h = self.lib.orc_grad_record(scene.h, C.byref(scene._gb(planes, formats)), _p(cam),
                                          C.byref(_Cfg(**cfg)), C.byref(acc), mode)
        if not self.h:
            raise ValueError("the record needs history planes for every scene light (<= 64)")

    def __del__(self):
        try:
            if self.h:
                self.lib.orc_grad_free(self.h)
                self.h = None
        except Exception:
            pass

    def forward(self, mats: np.ndarray, lights: np.ndarray) -> np.ndarray:
        m = np.ascontiguousarray(mats, np.float64)
        l = np.ascontiguousarray(lights, np.float64)
        out = np.zeros(self.shape + (3,), np.float64)
        self.lib.orc_grad_forward(self.scene.h, self.h, _p(m), _p(l), _p(out))
        return out

    def adjoint(self, mats: np.ndarray, lights: np.ndarray, w: np.ndarray):
        m = np.ascontiguousarray(mats, np.float64)
        l = np.ascontiguousarray(lights, np.float64)
        w = np.ascontiguousarray(w, np.float64)
        assert w.shape == self.shape + (3,)
        gm = np.zeros_like(m)
        gl = np.zeros_like(l)
        self.lib.orc_grad_adjoint(self.scene.h, self.h, _p(m), _p(l), _p(w), _p(gm), _p(gl))
        return gm, gl


def cfg_dict(spp=1, max_bounces=8, rng_mode=0, accum_frame=0, flags=0):
    return dict(shadow_spp=spp, max_bounces=max_bounces, rng_mode=rng_mode, accum_frame=accum_frame, flags=flags,
                block_size=0, queue_chunk=0, stack_depth=0, group_lanes=0, min_blocks=0)
