"""CPU tests of the Breakpoint%05d.h5 restart files (ht3d_breakpoint_write_h5 /
_read_h5, Dimensional/HydroThermal3D_v18.jl:579-588 and :384-395) through the
library's host-only image writer and parser: a committed known-byte fixture,
the file structure checked field by field against an independent reading of
the HDF5 specification (tests/h5_spec.py), the Julia array order of the
datasets, the reader on files laid out differently (no root scratch-pad,
compact storage, continuation blocks, dataspace version 2, skipped messages),
and the refusals."""
import ctypes
import os

import numpy as np
import pytest

import h5_spec
from hydrothermal3d_gb300 import _lib, abi

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIBPATH):
        from hydrothermal3d_gb300 import build
        build.build()
    return _lib.load()


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _fixture_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_h5_fixture", os.path.join(GOLDEN, "make_h5_fixture.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def _parse(lib, path, n):
    nx, ny, nz = n
    T = np.zeros((nx + 2, ny + 2, nz + 2), order="F")
    P = np.zeros_like(T, order="F")
    t, dt = ctypes.c_double(), ctypes.c_double()
    st = lib.ht3d_h5_breakpoint_parse(path.encode(), _p(T), _p(P), ctypes.byref(t), ctypes.byref(dt), nx, ny, nz)
    return st, T, P, t.value, dt.value


def test_known_bytes(lib, tmp_path):
    m = _fixture_module()
    out = str(tmp_path / "b.h5")
    assert m.write(out) == abi.OK
    assert open(out, "rb").read() == open(m.PATH, "rb").read()


def test_structure_follows_the_specification(lib):
    m = _fixture_module()
    T, P, t, dt = m.state()
    d = h5_spec.parse(m.PATH)
    assert set(d) == {"Tc_ex", "Pc_ex", "time", "dt"}
    # HDF5.jl's order: dataspace (nz+2, ny+2, nx+2), the Julia (column-major) bytes unchanged
    for name, a in (("Tc_ex", T), ("Pc_ex", P)):
        dims, v = d[name]
        assert dims == (m.NZ + 2, m.NY + 2, m.NX + 2)
        np.testing.assert_array_equal(v.reshape(dims), np.ascontiguousarray(a.transpose(2, 1, 0)))
        np.testing.assert_array_equal(v, a.ravel(order="F"))
    assert d["time"][0] == () and d["time"][1][0] == t
    assert d["dt"][0] == () and d["dt"][1][0] == dt


def test_round_trip(lib, tmp_path):
    m = _fixture_module()
    T, P, t, dt = m.state()
    st, T2, P2, t2, dt2 = _parse(lib, m.PATH, (m.NX, m.NY, m.NZ))
    assert st == abi.OK
    np.testing.assert_array_equal(T2, T)
    np.testing.assert_array_equal(P2, P)
    assert (t2, dt2) == (t, dt)


@pytest.mark.parametrize("variant", [dict(), dict(cache_root=True), dict(compact_scalars=False, continuation=False),
                                     dict(dataspace_v2=False, extra_messages=False)])
def test_reader_accepts_other_layouts(lib, tmp_path, variant):
    n = (5, 3, 4)
    rng = np.random.default_rng(3)
    T = np.asfortranarray(rng.normal(size=(n[0] + 2, n[1] + 2, n[2] + 2)))
    P = np.asfortranarray(rng.normal(size=T.shape))
    path = str(tmp_path / "other.h5")
    h5_spec.build(path, {"Tc_ex": np.ascontiguousarray(T.transpose(2, 1, 0)),
                         "Pc_ex": np.ascontiguousarray(P.transpose(2, 1, 0)), "time": 7.5, "dt": 0.25,
                         "extra": np.arange(3.0)}, **variant)
    st, T2, P2, t, dt = _parse(lib, path, n)
    assert st == abi.OK
    np.testing.assert_array_equal(T2, T)
    np.testing.assert_array_equal(P2, P)
    assert (t, dt) == (7.5, 0.25)


def test_refusals(lib, tmp_path):
    m = _fixture_module()
    n = (m.NX, m.NY, m.NZ)
    assert _parse(lib, m.PATH, (m.NX + 1, m.NY, m.NZ))[0] == abi.ERR_ARG  # another grid
    data = open(m.PATH, "rb").read()
    bad = tmp_path / "trunc.h5"
    bad.write_bytes(data[:len(data) - 100])
    assert _parse(lib, str(bad), n)[0] == abi.ERR_IO  # truncated data
    bad.write_bytes(b"HT3DBRK1" + data[8:])
    assert _parse(lib, str(bad), n)[0] == abi.ERR_IO  # not HDF5
    assert _parse(lib, str(tmp_path / "missing.h5"), n)[0] == abi.ERR_IO
    path = str(tmp_path / "nodt.h5")
    T, P, t, dt = m.state()
    h5_spec.build(path, {"Tc_ex": np.ascontiguousarray(T.transpose(2, 1, 0)),
                         "Pc_ex": np.ascontiguousarray(P.transpose(2, 1, 0)), "time": t})
    assert _parse(lib, path, n)[0] == abi.ERR_IO  # no dt dataset
