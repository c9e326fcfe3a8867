"""pytest configuration: the `gpu` marker and shared helpers."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the device path through the C ABI")


def gpu_available() -> bool:
    try:
        import ctypes
        rt = ctypes.CDLL("libcudart.so")
    except OSError:
        try:
            import glob
            cands = glob.glob("/usr/local/cuda/lib64/libcudart.so*")
            rt = ctypes.CDLL(cands[0]) if cands else None
        except OSError:
            rt = None
    if rt is None:
        return False
    import ctypes
    n = ctypes.c_int(0)
    return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0


@pytest.fixture(scope="session")
def require_gpu():
    if not gpu_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    return True
