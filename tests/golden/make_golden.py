"""Generates the golden vectors in this directory.

rng_kat.json — TEA seeds, LCG states and rnd() values of random.glsl:3-33,
computed here by an independent pure-Python restatement (mod 2^32 integer
arithmetic, exact float division by 2^24) and, when the reference's own
random.glsl/helpers.glsl have been compiled as C++ into oracle/_ref
(oracle/glsl_ref/Makefile, needs /root/reference), cross-checked against
that build before anything is written.

Run:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import json
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
M32 = 0xFFFFFFFF


def tea(v0: int, v1: int) -> int:
    s0 = 0
    for _ in range(16):
        s0 = (s0 + 0x9E3779B9) & M32
        v0 = (v0 + ((((v1 << 4) + 0xA341316C) & M32) ^ ((v1 + s0) & M32) ^ (((v1 >> 5) + 0xC8013EA4) & M32))) & M32
        v1 = (v1 + ((((v0 << 4) + 0xAD90777D) & M32) ^ ((v0 + s0) & M32) ^ (((v0 >> 5) + 0x7E95761E) & M32))) & M32
    return v0


def lcg(state: int) -> int:
    return (1664525 * state + 1013904223) & M32


def make():
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
    ref = ROOT / "oracle" / "_ref" / "libglslref.so"
    if ref.exists():
        lib = ctypes.CDLL(str(ref))
        lib.ref_tea.restype = ctypes.c_uint32
        lib.ref_tea.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
        for frame, seeds in kat["frames"].items():
            for e in seeds:
                got = lib.ref_tea((e["y"] * W + e["x"]) & M32, int(frame) & M32)
                assert got == e["seed"], (frame, e, got)
        kat["checked_against"] = "reference random.glsl compiled as C++ (oracle/_ref/libglslref.so)"
    (HERE / "rng_kat.json").write_text(json.dumps(kat, indent=1) + "\n")
    return kat


if __name__ == "__main__":
    k = make()
    print("wrote rng_kat.json", k.get("checked_against", "(not cross-checked: oracle/_ref not built)"))
