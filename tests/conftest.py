import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300); runs the libht3d parity tests")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.load()
    return oracle


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(os.path.join(ROOT, "tests", "golden", "dimless_small.npz")))


@pytest.fixture(scope="session")
def gpu_stream():
    """One CUDA stream for the GPU tests: the library context runs on it and
    every GPU test issues its torch work (allocations, fills, copies) on it,
    so the library's kernels are ordered after the inputs they read."""
    import torch
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    return torch.cuda.Stream()


@pytest.fixture(scope="session")
def ctx(gpu_stream):
    from hydrothermal3d_gb300 import Context
    c = Context(device=0, stream=gpu_stream.cuda_stream)
    yield c
    c.close()


@pytest.fixture(autouse=True)
def _torch_on_gpu_stream(request):
    if request.node.get_closest_marker("gpu") is None:
        yield
        return
    import torch
    with torch.cuda.stream(request.getfixturevalue("gpu_stream")):
        yield


def rel_err(a, b, mask=None):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if mask is not None:
        a, b = a[mask], b[mask]
    scale = max(np.max(np.abs(b)), 1e-300)
    return float(np.max(np.abs(a - b)) / scale)


def no_edges_mask(shape):
    """Mask of a ghosted array without its edge and corner ghosts."""
    m = np.zeros(shape, dtype=int)
    for ax, n in enumerate(shape):
        idx = [slice(None)] * 3
        sl = np.zeros(n, dtype=int)
        sl[0] = sl[-1] = 1
        m += sl.reshape([-1 if a == ax else 1 for a in range(3)])
    return m <= 1
