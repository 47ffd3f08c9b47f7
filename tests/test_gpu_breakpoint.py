"""Restart files (Dimensional/HydroThermal3D_v18.jl:384-395 read, :579-588
write): Tc_ex, Pc_ex, time and dt round-trip bit for bit, a run restarted
from a breakpoint continues exactly like the uninterrupted run, and foreign,
truncated or mismatched files are rejected with a status."""
import numpy as np
import pytest

import hydrothermal3d_gb300 as ht
from hydrothermal3d_gb300 import api, abi, v18

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fmt", ["bin", "h5"])
def test_round_trip(ctx, tmp_path, fmt):
    rng = np.random.default_rng(0)
    n = (9, 7, 5)
    ex = tuple(s + 2 for s in n)
    T, P = (ht.from_numpy(rng.uniform(size=ex)) for _ in range(2))
    api.breakpoint_write(ctx, tmp_path / f"Breakpoint00003.{fmt}", T, P, 1.25e12, 3.5e10)
    T2, P2 = ht.zeros(*ex), ht.zeros(*ex)
    t, dt = api.breakpoint_read(ctx, tmp_path / f"Breakpoint00003.{fmt}", T2, P2)
    assert (t, dt) == (1.25e12, 3.5e10)
    assert np.array_equal(ht.to_numpy(T2), ht.to_numpy(T)) and np.array_equal(ht.to_numpy(P2), ht.to_numpy(P))


def test_rejections(ctx, tmp_path):
    ex = (6, 5, 4)
    T, P = ht.zeros(*ex), ht.zeros(*ex)
    api.breakpoint_write(ctx, tmp_path / "a.bin", T, P, 0.0, 1.0)
    with pytest.raises(api.Ht3dError) as e:  # another grid
        api.breakpoint_read(ctx, tmp_path / "a.bin", ht.zeros(7, 5, 4), ht.zeros(7, 5, 4))
    assert e.value.status == abi.ERR_ARG
    with pytest.raises(api.Ht3dError) as e:
        api.breakpoint_read(ctx, tmp_path / "missing.bin", T, P)
    assert e.value.status == abi.ERR_IO
    (tmp_path / "foreign.bin").write_bytes(b"\x89HDF\r\n\x1a\n" + bytes(100))
    with pytest.raises(api.Ht3dError) as e:
        api.breakpoint_read(ctx, tmp_path / "foreign.bin", T, P)
    assert e.value.status == abi.ERR_IO
    raw = (tmp_path / "a.bin").read_bytes()
    (tmp_path / "short.bin").write_bytes(raw[:-8])
    with pytest.raises(api.Ht3dError) as e:
        api.breakpoint_read(ctx, tmp_path / "short.bin", T, P)
    assert e.value.status == abi.ERR_IO


def test_h5_file_is_the_reference_layout(ctx, tmp_path):
    """The device write gives the file the independent reading of the HDF5
    specification expects: datasets Tc_ex, Pc_ex with dataspace (nz+2, ny+2,
    nx+2) holding the column-major bytes, scalars time and dt."""
    import h5_spec
    rng = np.random.default_rng(4)
    ex = (8, 6, 5)
    Th, Ph = rng.uniform(size=ex), rng.uniform(size=ex)
    api.breakpoint_write(ctx, tmp_path / "Breakpoint00010.h5", ht.from_numpy(Th), ht.from_numpy(Ph), 2.5, 0.5)
    d = h5_spec.parse(str(tmp_path / "Breakpoint00010.h5"))
    for name, a in (("Tc_ex", Th), ("Pc_ex", Ph)):
        assert d[name][0] == ex[::-1]
        np.testing.assert_array_equal(d[name][1], np.asfortranarray(a).ravel(order="F"))
    assert d["time"][1][0] == 2.5 and d["dt"][1][0] == 0.5


def test_h5_rejections(ctx, tmp_path):
    ex = (6, 5, 4)
    T, P = ht.zeros(*ex), ht.zeros(*ex)
    api.breakpoint_write(ctx, tmp_path / "a.h5", T, P, 0.0, 1.0)
    with pytest.raises(api.Ht3dError) as e:  # another grid
        api.breakpoint_read(ctx, tmp_path / "a.h5", ht.zeros(7, 5, 4), ht.zeros(7, 5, 4))
    assert e.value.status == abi.ERR_ARG
    api.breakpoint_write(ctx, tmp_path / "a.bin", T, P, 0.0, 1.0)
    (tmp_path / "raw.h5").write_bytes((tmp_path / "a.bin").read_bytes())
    with pytest.raises(api.Ht3dError) as e:  # not an HDF5 file
        api.breakpoint_read(ctx, tmp_path / "raw.h5", T, P)
    assert e.value.status == abi.ERR_IO
    raw = (tmp_path / "a.h5").read_bytes()
    (tmp_path / "short.h5").write_bytes(raw[:-16])
    with pytest.raises(api.Ht3dError) as e:
        api.breakpoint_read(ctx, tmp_path / "short.h5", T, P)
    assert e.value.status == abi.ERR_IO


@pytest.mark.parametrize("fmt", ["bin", "h5"])
def test_restart_continues_the_run(ctx, tmp_path, fmt):
    """Steps 0-1, breakpoint, step 2 -- against a fresh run that reads the
    breakpoint and takes step 2: identical T, P, time and dt (the velocities
    are recomputed inside each step, so the reference's four items suffice)."""
    n = (10, 9, 6)
    nx, ny, nz = n
    b = v18.box(*n, seed=7, nitout=50, tol=1e-9)
    static = [ht.from_numpy(b[k]) for k in ("phc", "phv", "wN", "kmul")]
    shapes = ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1))
    T, P = ht.from_numpy(b["T"]), ht.from_numpy(b["P"])
    V = [ht.zeros(*s) for s in shapes]
    p = b["params"]
    for it in range(2):
        p.it = it
        api.step_v18(ctx, T, P, *static, *V, p)
    api.breakpoint_write(ctx, tmp_path / f"Breakpoint00001.{fmt}", T, P, p.time, p.dt)
    p.it = 2
    api.step_v18(ctx, T, P, *static, *V, p)

    q = v18.box(*n, seed=7, nitout=50, tol=1e-9)["params"]
    T2, P2 = ht.zeros(*T.shape), ht.zeros(*P.shape)
    V2 = [ht.zeros(*s) for s in shapes]
    q.time, q.dt = api.breakpoint_read(ctx, tmp_path / f"Breakpoint00001.{fmt}", T2, P2)
    q.it = 2
    api.step_v18(ctx, T2, P2, *static, *V2, q)
    assert np.array_equal(ht.to_numpy(T2), ht.to_numpy(T))
    assert np.array_equal(ht.to_numpy(P2), ht.to_numpy(P))
    assert (q.time, q.dt) == (p.time, p.dt)
    for a, c in zip(V2, V):
        assert np.array_equal(ht.to_numpy(a), ht.to_numpy(c))
