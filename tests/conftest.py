import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libfwi_gb300.so")


def _have_gpu():
    try:
        import ctypes
        lib = ctypes.CDLL(os.path.join(ROOT, "fwi_gb300", "_lib", "libfwi_gb300.so"))
    except OSError:
        return None  # library missing: the GPU tests must fail, not skip
    return lib.fwi_init(0) == 0


def pytest_collection_modifyitems(config, items):
    if not any(item.get_closest_marker("gpu") for item in items):
        return
    have = _have_gpu()
    if have is False:
        skip = pytest.mark.skip(reason="no CUDA device visible")
        for item in items:
            if item.get_closest_marker("gpu"):
                item.add_marker(skip)


@pytest.fixture(scope="session")
def golden():
    import numpy as np

    def load(name):
        return np.load(os.path.join(GOLDEN, name + ".npz"))
    return load
