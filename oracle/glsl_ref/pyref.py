"""ORACLE PIN — test infrastructure only.

ctypes front end of oracle/_ref/libglslref.so: the reference's own shader
sources compiled as C++ (see translate.py, harness.cpp).  Built only where
the reference checkout exists (make -C oracle/glsl_ref); used to pin the
oracle and to generate tests/golden fixtures.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE.parent / "_ref" / "libglslref.so"


def _reference_dir() -> Path | None:
    """The reference checkout: HY_REFERENCE_DIR, else the recipe's (Makefile) default."""
    env = os.environ.get("HY_REFERENCE_DIR")
    if env:
        return Path(env)
    r = subprocess.run(["make", "-s", "-C", str(HERE), "print-ref"], capture_output=True, text=True)
    out = r.stdout.strip()
    return Path(out) if r.returncode == 0 and out else None


REF_DIR = _reference_dir()
P = C.c_void_p
U32 = C.c_uint32
_lib = None


def available() -> bool:
    return LIB.exists() or (REF_DIR is not None and (REF_DIR / "data" / "shaders" / "hybridRaygen.rgen").exists())


def build() -> Path:
    r = subprocess.run(["make", "-C", str(HERE), f"REF={REF_DIR}"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference shader build failed:\n" + r.stdout + r.stderr)
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    if REF_DIR is not None and (REF_DIR / "data" / "shaders").exists():
        build()
    if not LIB.exists():
        raise RuntimeError("oracle/_ref/libglslref.so is not built (needs the reference checkout)")
    lib = C.CDLL(str(LIB))
    sig = {
        "ref_scene_create": (P, []),
        "ref_scene_destroy": (None, [P]),
        "ref_scene_set": (C.c_int, [P, P, U32, P, U32, P, U32, P, U32, P, U32, P, U32]),
        "ref_scene_set_env": (C.c_int, [P, C.c_int, P, U32, U32]),
        "ref_scene_set_texture": (C.c_int, [P, P, U32, U32]),
        "ref_tea": (U32, [U32, U32]),
        "ref_rnd_seq": (None, [U32, U32, P, P]),
        "ref_sample_disk": (None, [C.c_float, P, P, U32, P]),
        "ref_brdf": (None, [P, P, P, C.c_float, P, C.c_float, P]),
        "ref_shadow_pass": (C.c_int, [P, U32, U32, P, P, C.c_int, P]),
        "ref_blur": (C.c_int, [U32, U32, C.c_int, P, P, P]),
        "ref_hybrid_pass": (C.c_int, [P, U32, U32, P, P, P, P]),
        "ref_pathtrace_pass": (C.c_int, [P, U32, U32, P, C.c_int, P]),
        "ref_post": (C.c_int, [U32, U32, P, P]),
    }
    for k, (r, a) in sig.items():
        f = getattr(lib, k)
        f.restype = r
        f.argtypes = a
    _lib = lib
    return lib


def _p(a):
    assert a.flags["C_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)


def tea(a, b):
    return int(load().ref_tea(a, b))


def rnd_seq(seed, n):
    st = np.zeros(n, np.uint32)
    v = np.zeros(n, np.float32)
    load().ref_rnd_seq(seed, n, _p(st), _p(v))
    return st, v


def sample_disk(radius, pos, L, seed):
    out = np.zeros(3, np.float32)
    p, l = np.ascontiguousarray(pos, np.float32), np.ascontiguousarray(L, np.float32)
    load().ref_sample_disk(float(radius), _p(p), _p(l), seed, _p(out))
    return out


def brdf(N, V, L, roughness, F0, cos_theta):
    out = np.zeros(5, np.float32)
    a = [np.ascontiguousarray(x, np.float32) for x in (N, V, L, F0)]
    load().ref_brdf(_p(a[0]), _p(a[1]), _p(a[2]), float(roughness), _p(a[3]), float(cos_theta), _p(out))
    return out


class RefScene:
    """The reference shaders driven by the CPU pipeline harness (brute-force traversal)."""

    def __init__(self, scene=None, arrays=None, env=None):
        self.lib = load()
        self.h = self.lib.ref_scene_create()
        if scene is not None:
            arrays, env = scene.pack(), scene.env
        verts, idx, prims, xf, mats, lights = arrays
        self._keep = arrays
        self.num_lights = len(lights)
        self.lib.ref_scene_set(self.h, _p(verts), len(verts), _p(idx), len(idx), _p(prims), len(prims), _p(xf),
                               len(xf), _p(mats), len(mats), _p(lights) if len(lights) else None, len(lights))
        for slot, e in enumerate(env or []):
            e = np.ascontiguousarray(e, np.uint8)
            self.lib.ref_scene_set_env(self.h, slot, _p(e), e.shape[1], e.shape[0])
        for t in (getattr(scene, "textures", None) or []) if scene is not None else []:
            t = np.ascontiguousarray(t, np.uint8)
            self.lib.ref_scene_set_texture(self.h, _p(t), t.shape[1], t.shape[0])

    def __del__(self):
        try:
            self.lib.ref_scene_destroy(self.h)
        except Exception:
            pass

    @staticmethod
    def _planes(planes):
        planes = [np.ascontiguousarray(p, np.float32) for p in planes]
        return planes, (C.c_void_p * 6)(*[p.ctypes.data for p in planes])

    def shadow_pass(self, planes, cam36, samples):
        H, W = planes[0].shape[:2]
        keep, arr = self._planes(planes)
        out = np.zeros((self.num_lights, H, W), np.uint8)
        cam = np.ascontiguousarray(cam36, np.float32)
        rc = self.lib.ref_shadow_pass(self.h, W, H, arr, _p(cam), samples, _p(out))
        if rc != 0:
            raise RuntimeError("shadowRaygen binds at most 3 shadow images")
        return out

    def hybrid_pass(self, planes, cam36, shadow_u8):
        H, W = planes[0].shape[:2]
        keep, arr = self._planes(planes)
        out = np.zeros((H, W, 4), np.float32)
        cam = np.ascontiguousarray(cam36, np.float32)
        sh = np.ascontiguousarray(shadow_u8, np.uint8)
        self.lib.ref_hybrid_pass(self.h, W, H, arr, _p(cam), _p(sh), _p(out))
        return out

    def pathtrace_pass(self, cam36, width, height, samples, image_bgra8=None):
        """raygen.rgen + closesthit.rchit + miss shaders; accumulates into the B8G8R8A8 image
        (in place when given)."""
        if image_bgra8 is None:
            image_bgra8 = np.zeros((height, width, 4), np.uint8)
        cam = np.ascontiguousarray(cam36, np.float32)
        self.lib.ref_pathtrace_pass(self.h, width, height, _p(cam), samples, _p(image_bgra8))
        return image_bgra8


def post(image_bgra8):
    """postFragment.frag over a B8G8R8A8 image -> B8G8R8A8."""
    img = np.ascontiguousarray(image_bgra8, np.uint8)
    out = np.zeros_like(img)
    load().ref_post(img.shape[1], img.shape[0], _p(img), _p(out))
    return out


def blur(frame, motion_rg, shadow3_u8, hist3_u8):
    """blur.comp on 3 images (NLIGHTS = 3); updates hist3_u8 in place."""
    H, W = motion_rg.shape[:2]
    m = np.ascontiguousarray(motion_rg, np.float32)
    load().ref_blur(W, H, frame, _p(m), _p(shadow3_u8), _p(hist3_u8))
    return hist3_u8
