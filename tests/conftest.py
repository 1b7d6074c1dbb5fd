import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__ as ge  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsunnygb300.so")


@pytest.fixture(scope="session")
def sg():
    return ge.package()


@pytest.fixture(scope="session")
def orc():
    mod = ge.oracle()
    mod.load()
    return mod


def _gpu_available():
    import ctypes
    for name in ("libcudart.so.13", "libcudart.so", "/usr/local/cuda/lib64/libcudart.so.13"):
        try:
            lib = ctypes.CDLL(name)
        except OSError:
            continue
        n = ctypes.c_int(0)
        return lib.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    return False


@pytest.fixture(scope="session")
def gpu(sg):
    if not _gpu_available():
        pytest.skip("no CUDA device")
    sg.load_library()
    return True
