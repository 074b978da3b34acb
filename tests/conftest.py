import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")


@pytest.fixture(scope="session")
def lib():
    from cpp_volume_rendering_gb300 import abi, build
    build.build()
    return abi.load()


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build_lib()
    return oracle


def _gpu_available() -> bool:
    try:
        import ctypes
        cudart = None
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                cudart = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if cudart is None:
            return os.path.exists("/dev/nvidia0")
        n = ctypes.c_int(0)
        return cudart.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def ctx(lib):
    """A cvr context on GPU 0 (gpu tests only)."""
    if not _gpu_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    from cpp_volume_rendering_gb300 import scene
    c = scene.Context(0)
    yield c
    c.close()
