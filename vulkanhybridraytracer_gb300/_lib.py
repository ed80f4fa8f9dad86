"""ctypes view of include/hybridrt.h and the loader of libhybridrt.so.

The library is built in-tree (``build.py``).  Loading fails loudly when it is
missing: there is no CPU fallback for the pass.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libhybridrt.so"

# ---- error codes / enums (hybridrt.h) ------------------------------------------
HY_OK = 0
HY_ERR_INVALID_ARG = -1
HY_ERR_OOM = -2
HY_ERR_CUDA = -3
HY_ERR_TIMEOUT = -4
HY_ERR_STACK_OVERFLOW = -5
HY_ERR_QUEUE_OVERFLOW = -6
HY_ERR_NAN_INPUT = -7
HY_ERR_NOT_READY = -8
HY_ERR_UNSUPPORTED = -9
HY_ERR_TOO_LARGE = -10
HY_ERR_BAD_INDEX = -11
HY_NOALLOC_SCRATCH_BYTES = 16 << 20
HY_GRAD_MATERIAL_PARAMS = 5
HY_GRAD_LIGHT_PARAMS = 4
HY_GRAD_MAX_BOUNCES = 8
HY_GRAD_MAX_LIGHTS = 64

HY_FMT_RGBA32F, HY_FMT_RG32F, HY_FMT_RGBA16F, HY_FMT_RG16F, HY_FMT_RGBA8 = range(5)
HY_ACCUM_U8, HY_ACCUM_F32 = 0, 1
HY_RNG_REFERENCE, HY_RNG_DECORRELATED = 0, 1
HY_FLAG_FULL_BLUR_DISPATCH = 0x1
HY_FLAG_NO_ACCUM = 0x2
HY_FLAG_COUNT_TRAVERSAL = 0x4
HY_FLAG_NO_STATUS_SYNC = 0x8
HY_FLAG_PIXEL_PARALLEL = 0x10
HY_FLAG_RAY_POOL = 0x20
HY_FLAG_LANE_GROUPS = 0x40
HY_FLAG_GGX_REFLECTION = 0x80
HY_ANYHIT_AUTO, HY_ANYHIT_FAR_FIRST, HY_ANYHIT_NEAR_FIRST = 0, 1, 2
HY_BUILD_SAH, HY_BUILD_LBVH = 0, 1
HY_NO_HIT = 0xFFFFFFFF

HY_STATUS_STACK_OVERFLOW = 0x1
HY_STATUS_TIMEOUT = 0x2
HY_STATUS_BAD_INDEX = 0x10


class HyCreateInfo(C.Structure):
    _fields_ = [("device", C.c_int32), ("flags", C.c_uint32), ("stream", C.c_void_p),
                ("max_device_bytes", C.c_uint64)]


class HyLight(C.Structure):
    _fields_ = [("pos", C.c_float * 4), ("color", C.c_float * 4), ("radius", C.c_float), ("_pad", C.c_float * 3)]


class HyMaterial(C.Structure):
    _fields_ = [("diffuse", C.c_float * 4), ("textures", C.c_float * 4), ("smr", C.c_float * 4)]


class HyVertex(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("normal", C.c_float * 3), ("color", C.c_float * 3), ("uv", C.c_float * 2)]


class HyPrimitive(C.Structure):
    _fields_ = [("first_index", C.c_uint32), ("index_count", C.c_uint32), ("vertex_offset", C.c_uint32),
                ("material_id", C.c_uint32), ("transform_id", C.c_uint32), ("instance_id", C.c_uint32)]


class HyCamera(C.Structure):
    _fields_ = [("inv_view", C.c_float * 16), ("inv_proj", C.c_float * 16), ("frame", C.c_float * 4)]


class HyGBuffer(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("plane", C.c_void_p * 6), ("format", C.c_uint32 * 6)]


class HyAccum(C.Structure):
    _fields_ = [("format", C.c_uint32), ("num_lights", C.c_uint32), ("history", C.c_void_p)]


class HyPassConfig(C.Structure):
    _fields_ = [("shadow_spp", C.c_uint32), ("max_bounces", C.c_uint32), ("rng_mode", C.c_uint32),
                ("accum_frame", C.c_int32), ("flags", C.c_uint32), ("block_size", C.c_uint32),
                ("queue_chunk", C.c_uint32), ("stack_depth", C.c_uint32), ("group_lanes", C.c_uint32),
                ("min_blocks", C.c_uint32), ("visits_per_round", C.c_uint32)]


class HyStats(C.Structure):
    _fields_ = [("shadow_rays", C.c_uint64), ("reflection_rays", C.c_uint64), ("hit_shadow_rays", C.c_uint64),
                ("nodes_visited", C.c_uint64), ("tris_tested", C.c_uint64), ("error_flags", C.c_uint32),
                ("_pad", C.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if not k.startswith("_")}


class HyKernelTime(C.Structure):
    _fields_ = [("kernel", C.c_char * 40), ("launches", C.c_uint32), ("total_ms", C.c_float)]


class HyView(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("_pad", C.c_uint32), ("gbuffer", HyGBuffer), ("camera", HyCamera),
                ("config", HyPassConfig), ("accum", HyAccum), ("out_rgba32f", C.c_void_p),
                ("out_bgra8", C.c_void_p)]


HY_BATCH_NO_GRAPH = 0x1
HY_BATCH_NO_STATUS_SYNC = 0x2


class HyBvhStats(C.Structure):
    _fields_ = [("num_tris", C.c_uint32), ("num_bvh2_nodes", C.c_uint32), ("num_bvh8_nodes", C.c_uint32),
                ("depth", C.c_uint32), ("build_ms", C.c_float), ("scene_lo", C.c_float * 3),
                ("scene_hi", C.c_float * 3)]


class HyBvhLayout(C.Structure):
    _fields_ = [("two_level", C.c_uint32), ("num_nodes", C.c_uint32), ("num_records", C.c_uint32),
                ("num_instances", C.c_uint32), ("num_blas", C.c_uint32), ("tlas_region", C.c_uint32),
                ("tlas_nodes", C.c_uint32), ("depth", C.c_uint32)]


assert C.sizeof(HyLight) == 48 and C.sizeof(HyMaterial) == 48 and C.sizeof(HyVertex) == 44
assert C.sizeof(HyCamera) == 144

P = C.c_void_p
U32 = C.c_uint32
I32 = C.c_int

# name -> (restype, argtypes); the exported surface of hybridrt.h
PROTOTYPES = {
    "hy_create": (I32, [C.POINTER(P), C.POINTER(HyCreateInfo)]),
    "hy_destroy": (None, [P]),
    "hy_error_string": (C.c_char_p, [I32]),
    "hy_get_abi_version": (I32, []),
    "hy_synchronize": (I32, [P]),
    "hy_profile_enable": (I32, [P, I32]),
    "hy_profile_read": (I32, [P, C.POINTER(HyKernelTime), C.c_uint32, C.POINTER(C.c_uint32)]),
    "hy_debug_fail_alloc_after": (I32, [P, U32]),
    "hy_debug_set_traversal_limits": (I32, [P, U32, U32]),
    "hy_scene_set_geometry": (I32, [P, P, U32, P, U32, P, U32, P, U32]),
    "hy_scene_set_materials": (I32, [P, P, U32]),
    "hy_scene_set_lights": (I32, [P, P, U32]),
    "hy_scene_set_env": (I32, [P, I32, P, U32, U32]),
    "hy_bvh_build": (I32, [P, C.POINTER(HyBvhStats)]),
    "hy_bvh_refit": (I32, [P, P, U32]),
    "hy_bvh_download": (I32, [P, P, P, P, P, P]),
    "hy_bvh_build_instanced": (I32, [P, C.POINTER(HyBvhStats)]),
    "hy_bvh_layout": (I32, [P, C.POINTER(HyBvhLayout)]),
    "hy_bvh_download_instances": (I32, [P, P, P]),
    "hy_scene_set_build_mode": (I32, [P, C.c_uint32]),
    "hy_scene_set_anyhit_order": (I32, [P, C.c_uint32]),
    "hy_scene_anyhit_order": (I32, [P, C.POINTER(C.c_uint32)]),
    "hy_trace_rays": (I32, [P, P, U32, I32, P, C.POINTER(HyStats)]),
    "hy_gbuffer_primary": (I32, [P, C.POINTER(HyCamera), U32, U32, C.POINTER(C.c_void_p)]),
    "hy_shadow_pass": (I32, [P, C.POINTER(HyGBuffer), C.POINTER(HyCamera), C.POINTER(HyPassConfig), U32, P,
                             C.POINTER(HyStats)]),
    "hy_accumulate_pass": (I32, [P, C.POINTER(HyGBuffer), C.POINTER(HyPassConfig), P, C.POINTER(HyAccum)]),
    "hy_shade_pass": (I32, [P, C.POINTER(HyGBuffer), C.POINTER(HyCamera), C.POINTER(HyPassConfig),
                            C.POINTER(HyAccum), P, P, C.POINTER(HyStats)]),
    "hy_hybrid_forward": (I32, [P, C.POINTER(HyGBuffer), C.POINTER(HyCamera), C.POINTER(HyPassConfig),
                                C.POINTER(HyAccum), P, P, C.POINTER(HyStats)]),
    "hy_hybrid_forward_host": (I32, [P, C.POINTER(HyGBuffer), C.POINTER(HyCamera), C.POINTER(HyPassConfig),
                                     C.POINTER(HyAccum), P, P, C.POINTER(HyStats)]),
    "hy_scene_set_textures": (I32, [P, C.POINTER(C.c_void_p), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32),
                                    C.c_uint32]),
    "hy_post_resolve": (I32, [P, C.c_uint32, C.c_uint32, P, P, P]),
    "hy_hybrid_backward": (I32, [P, C.POINTER(HyGBuffer), C.POINTER(HyCamera), C.POINTER(HyPassConfig),
                                 C.POINTER(HyAccum), P, P, P, C.POINTER(HyStats)]),
    "hy_pathtrace_pass": (I32, [P, C.POINTER(HyCamera), C.c_uint32, C.c_uint32, C.POINTER(HyPassConfig), P, P,
                                C.POINTER(HyStats)]),
    "hy_accumulate_pass_noalloc": (I32, [C.POINTER(HyGBuffer), C.POINTER(HyPassConfig), P, C.POINTER(HyAccum), P]),
    "hy_batch_forward": (I32, [P, C.POINTER(P), U32, C.POINTER(HyView), U32, U32, C.POINTER(HyPassConfig),
                               C.POINTER(HyStats)]),
    "hy_batch_autotune": (I32, [P, C.POINTER(P), U32, C.POINTER(HyView), U32, U32, C.POINTER(HyPassConfig),
                                C.POINTER(C.c_float)]),
}

_lib = None


class HyError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        msg = error_string(code) if _lib is not None else str(code)
        super().__init__(f"{what}: {msg} ({code})" if what else f"{msg} ({code})")
        self.code = code


def error_string(code: int) -> str:
    return load().hy_error_string(code).decode()


def load(path: Path | str | None = None):
    """Load libhybridrt.so (raises if it has not been built)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with vulkanhybridraytracer_gb300.build.build_cuda()")
    lib = C.CDLL(str(p))
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(code: int, what: str = "") -> None:
    if code != HY_OK:
        raise HyError(code, what)
