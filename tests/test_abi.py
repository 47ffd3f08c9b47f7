"""CPU checks of the C ABI: the library loads and exports every symbol the
header declares, and the ctypes structs match the C structs.  No kernel is
launched (there may be no GPU here)."""
import ctypes
import os

import pytest

from hydrothermal3d_gb300 import _lib, abi


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIBPATH):
        from hydrothermal3d_gb300 import build
        build.build()
    return _lib.load()


def test_header_parses_and_lists_entry_points():
    protos = _lib.parse_header()
    assert len(protos) >= 40
    for name in ("ht3d_ctx_create", "ht3d_ComputeFlux", "ht3d_dyrel_solve_dimless", "ht3d_step_hrl",
                 "ht3d_weno5_advect", "ht3d_reduce"):
        assert name in protos


def test_every_declared_symbol_is_exported(lib):
    handle = ctypes.CDLL(_lib.LIBPATH)
    missing = [n for n in _lib.parse_header() if not hasattr(handle, n)]
    assert not missing, missing


def test_struct_layouts_match(lib):
    assert lib.ht3d_abi_version() == 1
    assert lib.ht3d_sizeof_dyrel_params() == ctypes.sizeof(abi.DyrelParams)
    assert lib.ht3d_sizeof_dyrel_stats() == ctypes.sizeof(abi.DyrelStats)
    assert lib.ht3d_sizeof_hrl_params() == ctypes.sizeof(abi.HrlParams)
    assert lib.ht3d_sizeof_instance() == ctypes.sizeof(abi.Instance)
    assert lib.ht3d_sizeof_v18_params() == ctypes.sizeof(abi.V18Params)
    assert lib.ht3d_sizeof_post_params() == ctypes.sizeof(abi.PostParams)
    assert lib.ht3d_sizeof_post_fields() == ctypes.sizeof(abi.PostFields)


def test_status_strings(lib):
    assert lib.ht3d_status_string(0) == b"ok"
    assert b"NaN" in lib.ht3d_status_string(abi.ERR_NAN)
    assert b"diverged" in lib.ht3d_status_string(abi.ERR_DIVERGED)
    assert lib.ht3d_status_string(999) == b"unknown status"


def test_null_ctx_is_rejected_without_gpu(lib):
    assert lib.ht3d_ctx_destroy(None) == abi.ERR_ARG
    assert lib.ht3d_ctx_launch_count(None) == 0
    assert lib.ht3d_ComputeFlux(None, *([None] * 7), 1.0, 1.0, 1.0, 4, 4, 4) == abi.ERR_ARG


def _noalloc_args(ptr, bc_type, n_iter=3, n=(4, 4, 4)):
    """Arguments of ht3d_dyrel_iterate_noalloc with every array at `ptr` (never
    dereferenced: each case is refused, or does nothing, before a launch)."""
    return (ptr,) * 7 + (1.0, 0.25, 0.25, 0.25, abi.int6(*bc_type), abi.dbl6(0, 0, 1, 0, 0, 0), 0.9, 0.1, 0.01,
                         n_iter, *n, None)


def test_noalloc_rejects_bad_arguments_without_launching(lib):
    """Refusals of the allocation-free iteration happen on the host, before
    any CUDA call: null arrays, a BC type other than Neumann (0) or Dirichlet
    (1), a negative iteration count, empty grids, grids beyond the static
    scratch.  n_iter == 0 checks its arguments and touches nothing."""
    fake = ctypes.c_void_p(0x1000)  # stands in for a device array
    good = (0, 0, 1, 1, 0, 0)
    fn = lib.ht3d_dyrel_iterate_noalloc
    args = list(_noalloc_args(fake, good))
    for i in range(7):
        bad = list(args)
        bad[i] = None
        assert fn(*bad) == abi.ERR_ARG, i
    assert fn(*_noalloc_args(fake, (0, 0, 2, 1, 0, 0))) == abi.ERR_ARG
    assert fn(*_noalloc_args(fake, (0, 0, 1, 1, 0, -1))) == abi.ERR_ARG
    assert fn(*_noalloc_args(fake, good, n_iter=-1)) == abi.ERR_ARG
    assert fn(*_noalloc_args(fake, good, n=(0, 4, 4))) == abi.ERR_ARG
    assert fn(*_noalloc_args(fake, good, n=(100, 100, 100))) == abi.ERR_SCRATCH
    assert fn(*_noalloc_args(fake, good, n_iter=0)) == abi.OK
