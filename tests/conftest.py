import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


def pytest_collection_modifyitems(config, items):
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(autouse=True)
def _chunked_at_every_size(request):
    """GPU tests take the chunked mixed kernels at every call size (the
    library takes them from ~3e7 samples per call on), so that their small
    cases exercise them; a test of the per-sample tier raises the threshold
    itself (it is restored after every test)."""
    if request.node.get_closest_marker("gpu") is None or not HAS_GPU:
        yield
        return
    from so3g_gb300 import set_chunked_min_samples
    old = set_chunked_min_samples(0)
    yield
    set_chunked_min_samples(old)


@pytest.fixture(scope="session")
def orc():
    from oracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def gpulib():
    """Builds (if needed) and loads the CUDA library."""
    import so3g_gb300.build as b
    b.build()
    from so3g_gb300 import _abi
    return _abi.lib()


def bits_equal(a, b):
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    if a.dtype == np.float64:
        return np.array_equal(a.view(np.int64), b.view(np.int64))
    if a.dtype == np.float32:
        return np.array_equal(a.view(np.int32), b.view(np.int32))
    return np.array_equal(a, b)
