import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
for p in (ROOT, ROOT / "oracle"):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libhybridrt.so")


@pytest.fixture(scope="session")
def oracle_lib():
    import pyoracle

    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def gpu_lib():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from vulkanhybridraytracer_gb300 import _lib, build

    build.build_cuda()
    return _lib.load()
