"""The C++ host side (include/hybridrt.hpp): it compiles and links against
libhybridrt with the reference's scene/renderer vocabulary (CPU), and on a
GPU tests/cpp/adapter_smoke.cpp renders frames bit-identical to direct C ABI
calls, restarts accumulation on a camera move, refits and reports errors."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
CUDA = Path("/usr/local/cuda")


def _compile(out: Path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    from vulkanhybridraytracer_gb300 import build

    lib = build.build_cuda()
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}",
           f"-I{CUDA / 'include'}", str(ROOT / "tests" / "cpp" / "adapter_smoke.cpp"), f"-L{lib.parent}", "-lhybridrt",
           f"-L{CUDA / 'lib64'}", "-lcudart", f"-Wl,-rpath,{lib.parent}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def test_cpp_adapter_compiles(tmp_path):
    assert _compile(tmp_path / "adapter_smoke").exists()


@pytest.mark.gpu
def test_cpp_adapter_runs(gpu_lib, tmp_path):
    exe = _compile(tmp_path / "adapter_smoke")
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "adapter OK" in r.stdout
