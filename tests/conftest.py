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
def ctx():
    import torch
    from hydrothermal3d_gb300 import Context
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    c = Context(device=0)
    yield c
    c.close()


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
