"""Build of the native parts: libhybridrt.so (CUDA, sm_103a) and the oracle.

The CUDA translation units are compiled in parallel with one -gencode for
sm_103a and linked into an in-tree shared library next to this file.  The
oracle (test infrastructure) is built with make in ``oracle/``.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libhybridrt.so"
ORACLE_DIR = ROOT / "oracle"
ORACLE_LIB = ORACLE_DIR / "liboracle.so"

SOURCES = ["hy_api.cu", "hy_bvh.cu", "hy_sah.cu", "hy_pass.cu", "hy_grad.cu", "hy_pt.cu", "hy_noalloc.cu",
           "hy_batch_64.cu", "hy_batch_128.cu", "hy_batch_256.cu", "hy_stream_raw.cu", "hy_stream_accum.cu",
           "hy_stream_two.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = [
    "-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-Xptxas", "-O3",
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build_cuda(force: bool = False, verbose: bool = False, extra_flags=()) -> Path:
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "hybridrt.h"]
    objs = []
    jobs = []
    for src in SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers]):
            cmd = [nvcc, *ARCH, *NVFLAGS, *extra_flags, "-c", str(s), "-o", str(o)]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lcudart"]
        run(cmd)
    return LIB


def build_oracle(force: bool = False) -> Path:
    args = ["make", "-C", str(ORACLE_DIR)]
    if force:
        args.insert(1, "-B")
    r = subprocess.run(args, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return ORACLE_LIB


def reference_dir() -> Path | None:
    """The reference checkout: HY_REFERENCE_DIR, else the default of the recipe
    that reads it (oracle/glsl_ref/Makefile)."""
    env = os.environ.get("HY_REFERENCE_DIR")
    if env:
        return Path(env)
    r = subprocess.run(["make", "-s", "-C", str(ORACLE_DIR / "glsl_ref"), "print-ref"], capture_output=True,
                       text=True)
    out = r.stdout.strip()
    return Path(out) if r.returncode == 0 and out else None


def build_reference_pin(force: bool = False):
    """The reference's own shaders compiled as C++ into oracle/_ref (test
    infrastructure); only where the reference checkout exists."""
    ref = reference_dir()
    if ref is None or not (ref / "data" / "shaders").exists():
        return None
    args = ["make", "-C", str(ORACLE_DIR / "glsl_ref"), f"REF={ref}"]
    if force:
        args.insert(1, "-B")
    r = subprocess.run(args, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference shader build failed:\n" + r.stdout + r.stderr)
    return ORACLE_DIR / "_ref" / "libglslref.so"


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=3) as ex:
        f1 = ex.submit(build_cuda, force)
        f2 = ex.submit(build_oracle, force)
        f3 = ex.submit(build_reference_pin, force)
        f1.result()
        f2.result()
        f3.result()


if __name__ == "__main__":
    import sys

    build_all(force="-f" in sys.argv)
    print(LIB)
