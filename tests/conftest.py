import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the sm_103a library")


def _has_gpu() -> bool:
    try:
        import ctypes

        rt = None
        for name in ("libcudart.so", "libcudart.so.13", "libcudart.so.12"):
            try:
                rt = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if rt is None:
            import torch

            return torch.cuda.is_available()
        n = ctypes.c_int(0)
        return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    """The CUDA library, built in-tree; a GPU test fails (not skips) without a GPU."""
    if not _has_gpu():
        pytest.fail("this test needs a CUDA device")
    from swe_fvm_gb300 import _lib

    return _lib.load()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle

    return oracle.lib()
