"""Generates the golden vectors in this directory.

rng_kat.json      TEA seeds, LCG states and rnd() values of random.glsl:3-33,
                  from an independent pure-Python restatement (mod 2^32
                  integer arithmetic, exact float division by 2^24),
                  cross-checked against the reference's own random.glsl.
ref_kat.json      sampleDisk directions and GGX / Smith / Fresnel values
                  computed by the reference's own helpers.glsl.
ref_pass_small.npz
                  the reference's own shadowRaygen.rgen, blur.comp and
                  hybridRaygen.rgen + hybridHit.rchit + miss.rmiss +
                  shadow.rmiss run on the 48x48 small_glass workload (glass,
                  mirrors, 8 bounces), with its inputs (G-buffer, camera).
ref_pathtrace_small.npz
                  the reference's own path-traced pipeline (raygen.rgen +
                  closesthit.rchit + miss.rmiss + shadow.rmiss) on the same
                  workload: the B8G8R8A8 image after frames -1, 1 and 2.
ref_textured_small.npz
                  the reference's own shadowRaygen / hybrid shaders and
                  path-traced shaders on the textured 48x40 workload, with
                  its G-buffer input.
ref_post_small.npz
                  the reference's postFragment.frag (gamma 1/2.2) over a
                  random B8G8R8A8 image.

"The reference's own" = the reference checkout's shader sources rewritten
into C++ and compiled by oracle/glsl_ref (Makefile, translate.py,
harness.cpp) into oracle/_ref/libglslref.so; that build needs the reference
checkout, so this script runs where it exists.  The fixtures let every other
machine check the oracle and the GPU path against the reference's output.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
M32 = 0xFFFFFFFF
for p in (ROOT, ROOT / "oracle", ROOT / "oracle" / "glsl_ref"):
    sys.path.insert(0, str(p))


def tea(v0: int, v1: int) -> int:
    s0 = 0
    for _ in range(16):
        s0 = (s0 + 0x9E3779B9) & M32
        v0 = (v0 + ((((v1 << 4) + 0xA341316C) & M32) ^ ((v1 + s0) & M32) ^ (((v1 >> 5) + 0xC8013EA4) & M32))) & M32
        v1 = (v1 + ((((v0 << 4) + 0xAD90777D) & M32) ^ ((v0 + s0) & M32) ^ (((v0 >> 5) + 0x7E95761E) & M32))) & M32
    return v0


def lcg(state: int) -> int:
    return (1664525 * state + 1013904223) & M32


def rng_kat(ref=None):
    W = 1700  # the reference window width (src/vk_engine.cpp:27)
    kat = {"width": W, "frames": {}, "rnd": {}}
    for frame in (0, 1, 7, -1):
        fu = frame & M32
        seeds = []
        for y in (0, 1, 899):
            for x in (0, 1, 2, 3, 1699):
                seeds.append({"x": x, "y": y, "seed": tea((y * W + x) & M32, fu)})
        kat["frames"][str(frame)] = seeds
    for s in (0, 1, 0xDEADBEEF, tea(0, 0)):
        st, vals, states = s, [], []
        for _ in range(8):
            st = lcg(st)
            states.append(st)
            vals.append((st & 0xFFFFFF) / float(1 << 24))
        kat["rnd"][str(s)] = {"states": states, "values": vals}
    if ref is not None:
        for frame, seeds in kat["frames"].items():
            for e in seeds:
                assert ref.tea((e["y"] * W + e["x"]) & M32, int(frame) & M32) == e["seed"]
        for s, d in kat["rnd"].items():
            st, v = ref.rnd_seq(int(s), 8)
            assert st.tolist() == d["states"] and np.array_equal(v, np.float32(d["values"]))
        kat["checked_against"] = "reference random.glsl compiled as C++ (oracle/_ref/libglslref.so)"
    return kat


def ref_kat(ref):
    rng = np.random.default_rng(20261203)
    disk, brdf = [], []
    for i in range(64):
        pos = rng.normal(size=3).astype(np.float32)
        L = rng.normal(size=3).astype(np.float32)
        L /= np.linalg.norm(L)
        if i == 0:
            L = np.array([0, 1, 0], np.float32)  # the tangent special case
        radius, seed = float(np.float32(rng.uniform(0.05, 1.0))), int(rng.integers(0, 2**32))
        d = ref.sample_disk(radius, pos, L, seed)
        disk.append({"radius": radius, "pos": pos.tolist(), "L": L.tolist(), "seed": seed, "dir": d.tolist()})
    for i in range(64):
        N, V, L = [(lambda x: (x / np.linalg.norm(x)).astype(np.float32))(rng.normal(size=3)) for _ in range(3)]
        r, c = float(np.float32(rng.uniform(0.05, 1))), float(np.float32(rng.uniform(0, 1)))
        F0 = rng.uniform(0, 1, 3).astype(np.float32)
        out = ref.brdf(N, V, L, r, F0, c)
        brdf.append({"N": N.tolist(), "V": V.tolist(), "L": L.tolist(), "roughness": r, "F0": F0.tolist(),
                     "cos": c, "D_G_F": out.tolist()})
    return {"source": "reference helpers.glsl compiled as C++ (oracle/_ref/libglslref.so)", "sampleDisk": disk,
            "brdf": brdf}


def ref_pass(ref):
    """Reference shaders on the small_glass workload (brute-force traversal of the harness)."""
    import pyoracle as po
    from vulkanhybridraytracer_gb300 import scenes

    wl = scenes.small_glass()
    cam = wl.camera(3.0)
    orc = po.OracleScene()
    orc.set_scene(wl.scene)
    planes = orc.gbuffer(cam, wl.width, wl.height, po.TRACE_BRUTE)  # G-buffer input (the raster pass's job)
    rs = ref.RefScene(wl.scene)
    shadow1 = rs.shadow_pass(planes, cam, 1)
    shadow4 = rs.shadow_pass(planes, cam, 4)
    # blur.comp: reset frame then a running-mean frame, on 3 images of 120x72 (not multiples of 16)
    bh, bw = 72, 120
    g = np.random.default_rng(7)
    motion = np.full((bh, bw, 2), 0.5, np.float32)
    blur_in = g.integers(0, 256, (3, bh, bw)).astype(np.uint8)
    blur_hist0 = g.integers(0, 256, (3, bh, bw)).astype(np.uint8)
    blur_f0 = ref.blur(0, motion, blur_in.copy(), blur_hist0.copy())
    blur_f3 = ref.blur(3, motion, blur_in.copy(), blur_f0.copy())
    hybrid = rs.hybrid_pass(planes, cam, shadow4)
    return dict(camera=cam, **{f"plane{i}": planes[i] for i in range(6)}, shadow_spp1=shadow1, shadow_spp4=shadow4,
                hybrid_rgba=hybrid, blur_motion=motion, blur_in=blur_in, blur_hist0=blur_hist0,
                blur_after_frame0=blur_f0, blur_after_frame3=blur_f3)


def ref_pathtrace(ref):
    """The reference's path-traced pipeline (raygen.rgen + closesthit.rchit + miss shaders) on
    the 48x48 small_glass workload, 2 shadow samples: frame -1 stores, frames 1 and 2 mix
    into the B8G8R8A8 image."""
    from vulkanhybridraytracer_gb300 import scenes

    wl = scenes.small_glass()
    rs = ref.RefScene(wl.scene)
    img = np.zeros((wl.height, wl.width, 4), np.uint8)
    out = {}
    for frame in (-1, 1, 2):
        cam = wl.camera(float(frame))
        img = rs.pathtrace_pass(cam, wl.width, wl.height, 2, img)
        out[f"camera_f{frame + 1}"] = cam
        out[f"image_f{frame + 1}"] = img.copy()
    return out


def ref_textured(ref):
    """The reference's hybrid and path-traced shaders on the 48x40 small_textured workload
    (checker / noise / emissive RGBA8 textures, NEAREST + REPEAT), with its G-buffer input."""
    import pyoracle as po
    from vulkanhybridraytracer_gb300 import scenes

    wl = scenes.small_textured(48, 40)
    cam = wl.camera(2.0)
    orc = po.OracleScene()
    orc.set_scene(wl.scene)
    planes = orc.gbuffer(cam, wl.width, wl.height, po.TRACE_BRUTE)
    rs = ref.RefScene(wl.scene)
    shadow = rs.shadow_pass(planes, cam, 2)
    hybrid = rs.hybrid_pass(planes, cam, shadow)
    img = np.zeros((wl.height, wl.width, 4), np.uint8)
    out = dict(camera=cam, **{f"plane{i}": planes[i] for i in range(6)}, shadow_spp2=shadow, hybrid_rgba=hybrid)
    for frame in (-1, 1):
        c = wl.camera(float(frame))
        img = rs.pathtrace_pass(c, wl.width, wl.height, 2, img)
        out[f"pt_camera_f{frame + 1}"] = c
        out[f"pt_image_f{frame + 1}"] = img.copy()
    return out


def make():
    ref = None
    try:
        import pyref

        if pyref.available():
            pyref.load()
            ref = pyref
    except Exception as e:  # the reference checkout is not on every machine
        print("reference shaders unavailable:", e)
    (HERE / "rng_kat.json").write_text(json.dumps(rng_kat(ref), indent=1) + "\n")
    if ref is None:
        print("wrote rng_kat.json (not cross-checked); ref_kat.json / ref_pass_small.npz need the reference")
        return
    (HERE / "ref_kat.json").write_text(json.dumps(ref_kat(ref)) + "\n")
    np.savez_compressed(HERE / "ref_pass_small.npz", **ref_pass(ref))
    np.savez_compressed(HERE / "ref_pathtrace_small.npz", **ref_pathtrace(ref))
    np.savez_compressed(HERE / "ref_textured_small.npz", **ref_textured(ref))
    g = np.random.default_rng(11)
    post_in = g.integers(0, 256, (24, 40, 4)).astype(np.uint8)
    post_in[0, :8, :3] = 0  # below the 0.001 floor
    np.savez_compressed(HERE / "ref_post_small.npz", image=post_in, post=ref.post(post_in))
    print("wrote rng_kat.json, ref_kat.json, ref_pass_small.npz, ref_pathtrace_small.npz, ref_textured_small.npz, "
          "ref_post_small.npz from the reference's shader code")


if __name__ == "__main__":
    make()
