"""Writes tests/golden/breakpoint_h5_3x2x1.h5: the library's Breakpoint%05d.h5
image (ht3d_h5_breakpoint_image, host-only) of a small seeded state, kept as a
known-byte fixture of the format.

    python tests/golden/make_h5_fixture.py
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
NX, NY, NZ = 3, 2, 1
PATH = os.path.join(HERE, "breakpoint_h5_3x2x1.h5")


def state():
    rng = np.random.default_rng(17)
    shape = (NX + 2, NY + 2, NZ + 2)
    T = np.asfortranarray(rng.uniform(0.0, 1.0, shape))
    P = np.asfortranarray(rng.uniform(-1.0, 1.0, shape))
    return T, P, 0.125, 3.0e-3


def write(path):
    from hydrothermal3d_gb300 import _lib
    lib = _lib.load()
    T, P, t, dt = state()
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    return lib.ht3d_h5_breakpoint_image(path.encode(), p(T), p(P), t, dt, NX, NY, NZ)


if __name__ == "__main__":
    assert write(PATH) == 0
    print(PATH, os.path.getsize(PATH))
