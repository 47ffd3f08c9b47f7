"""CPU FP64 oracle of the HydroThermal3D hot path -- TEST INFRASTRUCTURE ONLY.

Python access to ``oracle/ht3d_oracle.cpp`` (see that file's header for what
it restates and how it is pinned).  Only tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline / reference arm use it, always as the checker or the
timed CPU baseline, never as a product code path.

Arrays are numpy float64 arrays in Fortran (column-major) order with the
reference's shapes; functions mutate their output arguments in place.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


def load():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(_build.build())
    return _lib


def _p(a):
    if a is None:
        return None
    if not isinstance(a, np.ndarray) or a.dtype != np.float64:
        raise ValueError("oracle arrays must be float64 numpy arrays")
    if a.ndim > 1 and not a.flags.f_contiguous:
        raise ValueError("oracle arrays must be Fortran-ordered")
    return a.ctypes.data_as(ctypes.c_void_p)


def _conv(x):
    if isinstance(x, np.ndarray):
        return _p(x)
    if x is None:
        return ctypes.c_void_p(0)
    if isinstance(x, bool):
        return ctypes.c_int(int(x))
    if isinstance(x, (int, np.integer)):
        return ctypes.c_longlong(int(x))
    if isinstance(x, (float, np.floating)):
        return ctypes.c_double(float(x))
    return x  # ctypes objects / byref


def call(name, *args):
    """Call ``orc_<name>`` with numpy arrays / python scalars.

    Integer scalars are passed as 64-bit (the oracle's dims and n are i64);
    use ``ctypes.c_int`` explicitly for int parameters.
    """
    fn = getattr(load(), "orc_" + name)
    return fn(*[_conv(a) for a in args])


def set_threads(n):
    load().orc_set_num_threads(ctypes.c_int(int(n)))


def num_threads():
    return int(load().orc_num_threads())


def reduce(op, a):
    f = {"sum": "orc_sum", "sum_abs": "orc_sum_abs", "max": "orc_max", "min": "orc_min", "max_abs": "orc_max_abs"}[op]
    fn = getattr(load(), f)
    fn.restype = ctypes.c_double
    return fn(_p(a), ctypes.c_longlong(a.size))


def law(which, a, b=0.0):
    fn = load().orc_law
    fn.restype = ctypes.c_double
    return fn(ctypes.c_int(which), ctypes.c_double(a), ctypes.c_double(b))


def nusselt(qy, Lx, Lz):
    """Nu of the (nx, ny+1, nz) y-flux (orc_Nusselt)."""
    fn = load().orc_Nusselt
    fn.restype = ctypes.c_double
    nx, ny1, nz = qy.shape
    return fn(_p(qy), ctypes.c_double(Lx), ctypes.c_double(Lz), ctypes.c_longlong(nx), ctypes.c_longlong(ny1 - 1),
              ctypes.c_longlong(nz))


def zeros(*shape):
    return np.zeros(shape, order="F")


def int6(*v):
    return (ctypes.c_int * 6)(*v)


def dbl6(*v):
    return (ctypes.c_double * 6)(*[float(x) for x in v])


def dyrel_solve_dimless(X, R, kx, ky, kz, cX, dx, dy, dz, bc_type6, bc_val6, params, F, F0, n_iter_fixed=0):
    """Returns (status, DyrelStats)."""
    from hydrothermal3d_gb300.abi import DyrelStats
    nx, ny, nz = (s - 2 for s in X.shape)
    st = DyrelStats()
    fn = load().orc_dyrel_solve_dimless
    fn.restype = ctypes.c_int
    s = fn(_p(X), _p(R), _p(kx), _p(ky), _p(kz), ctypes.c_double(cX), ctypes.c_double(dx), ctypes.c_double(dy),
           ctypes.c_double(dz), int6(*bc_type6), dbl6(*bc_val6), ctypes.byref(params), ctypes.c_int(n_iter_fixed),
           _p(F), _p(F0), ctypes.byref(st), ctypes.c_longlong(nx), ctypes.c_longlong(ny), ctypes.c_longlong(nz))
    return s, st


def step_hrl(T, P, ktv, kfv, Vx, Vy, Vz, params):
    """One dimensionless HRL time step. Returns (status, stats_thermal, stats_darcy)."""
    from hydrothermal3d_gb300.abi import DyrelStats
    nx, ny, nz = (s - 2 for s in T.shape)
    st_t, st_d = DyrelStats(), DyrelStats()
    fn = load().orc_step_hrl
    fn.restype = ctypes.c_int
    s = fn(_p(T), _p(P), _p(ktv), _p(kfv), _p(Vx), _p(Vy), _p(Vz), ctypes.byref(params), ctypes.byref(st_t),
           ctypes.byref(st_d), ctypes.c_longlong(nx), ctypes.c_longlong(ny), ctypes.c_longlong(nz))
    return s, st_t, st_d


def step_v18(T, P, phc, phv, wN, kmul, Vx, Vy, Vz, params):
    """One dimensional (v18) time step. Returns (status, stats_thermal, stats_darcy)."""
    from hydrothermal3d_gb300.abi import DyrelStats
    nx, ny, nz = (s - 2 for s in T.shape)
    st_t, st_d = DyrelStats(), DyrelStats()
    fn = load().orc_step_v18
    fn.restype = ctypes.c_int
    s = fn(_p(T), _p(P), _p(phc), _p(phv), _p(wN), _p(kmul) if kmul is not None else None, _p(Vx), _p(Vy), _p(Vz),
           ctypes.byref(params), ctypes.byref(st_t), ctypes.byref(st_d), ctypes.c_longlong(nx), ctypes.c_longlong(ny),
           ctypes.c_longlong(nz))
    return s, st_t, st_d
