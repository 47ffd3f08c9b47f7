"""ht3d_write_vtr (host code, no GPU): the VTK rectilinear-grid file of the
v18 driver's output step (Dimensional/HydroThermal3D_v18.jl:664-686), parsed
back with a small reader of the VTK XML appended-raw format."""
import re
import xml.etree.ElementTree as ET

import numpy as np
import pytest

from hydrothermal3d_gb300 import api, abi


def read_vtr(path):
    raw = open(path, "rb").read()
    head, _, rest = raw.partition(b"<AppendedData encoding=\"raw\">\n_")
    root = ET.fromstring(head + b"<AppendedData encoding=\"raw\"/></VTKFile>")
    assert root.get("type") == "RectilinearGrid" and root.get("header_type") == "UInt64"
    assert root.get("byte_order") == "LittleEndian"
    ext = [int(v) for v in root.find("RectilinearGrid").get("WholeExtent").split()]
    n = (ext[1] + 1, ext[3] + 1, ext[5] + 1)

    def block(el):
        off = int(el.get("offset"))
        size = int(np.frombuffer(rest[off:off + 8], dtype="<u8")[0])
        return np.frombuffer(rest[off + 8:off + 8 + size], dtype="<f8")

    fields = {}
    for el in root.iter("DataArray"):
        v = block(el)
        nc = int(el.get("NumberOfComponents", "1"))
        if el.get("Name") in ("x", "y", "z") and el in list(root.find(".//Coordinates")):
            fields["coord_" + el.get("Name")] = v
        elif nc == 1:
            fields[el.get("Name")] = v.reshape(n, order="F")
        else:
            fields[el.get("Name")] = tuple(v[c::3].reshape(n, order="F") for c in range(3))
    assert rest.rstrip().endswith(b"</AppendedData>\n</VTKFile>")
    return n, fields


def test_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    nx, ny, nz = 5, 4, 3
    xc, yc, zc = np.linspace(0, 1, nx), np.linspace(-2, 0, ny), np.linspace(3, 4, nz)
    T = np.asfortranarray(rng.uniform(size=(nx, ny, nz)))
    T[1, 2, 0] = np.nan  # air cells are NaN in the diagnostics
    V = tuple(np.asfortranarray(rng.uniform(size=(nx, ny, nz))) for _ in range(3))
    out = api.write_vtr(tmp_path / "HT3DOutput00010", xc, yc, zc, {"Temperature": T, "Velocity": V})
    assert out.endswith("HT3DOutput00010.vtr")
    n, f = read_vtr(out)
    assert n == (nx, ny, nz)
    assert np.array_equal(f["Temperature"], T, equal_nan=True)
    for a, b in zip(f["Velocity"], V):
        assert np.array_equal(a, b)
    assert np.array_equal(f["coord_x"], xc) and np.array_equal(f["coord_y"], yc) and np.array_equal(f["coord_z"], zc)


def test_rejects_bad_arguments(tmp_path):
    x = np.zeros(2)
    with pytest.raises(ValueError):
        api.write_vtr(tmp_path / "a", x, x, x, {"T": np.zeros((2, 2, 3))})
    with pytest.raises(api.Ht3dError) as e:  # quote in a name would break the XML
        api.write_vtr(tmp_path / "a", x, x, x, {'T"x': np.zeros((2, 2, 2))})
    assert e.value.status == abi.ERR_ARG
    with pytest.raises(api.Ht3dError) as e:  # longer than an XML attribute the writer accepts
        api.write_vtr(tmp_path / "a", x, x, x, {"T" * 201: np.zeros((2, 2, 2))})
    assert e.value.status == abi.ERR_ARG
    with pytest.raises(api.Ht3dError) as e:
        api.write_vtr(tmp_path / "no_such_dir" / "a", x, x, x, {"T": np.zeros((2, 2, 2))})
    assert e.value.status == abi.ERR_IO


def test_vector_field_across_interleave_chunks(tmp_path):
    """More points than one interleave chunk (65536): components stay aligned."""
    nx, ny, nz = 50, 41, 37  # 75850 points
    rng = np.random.default_rng(3)
    V = tuple(np.asfortranarray(rng.standard_normal((nx, ny, nz))) for _ in range(3))
    out = api.write_vtr(tmp_path / "big.vtr", np.arange(nx, dtype=float), np.arange(ny, dtype=float),
                        np.arange(nz, dtype=float), {"Velocity": V, "Peclet": V[0] * 2})
    assert out.endswith("big.vtr") and not out.endswith(".vtr.vtr")
    n, f = read_vtr(out)
    assert n == (nx, ny, nz)
    for a, b in zip(f["Velocity"], V):
        assert np.array_equal(a, b)
    assert np.array_equal(f["Peclet"], V[0] * 2)
