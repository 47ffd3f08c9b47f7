"""GPU parity of the output diagnostics (Dimensional/kernels_HT3D_postprocessing.jl)
and the Nusselt number (Dimensionless/HydroThermal3D_Alban_v6.jl:345-348)
against the oracle.

Every field is bit-identical, permeability and viscosity included: their
exponentials are the library's own (expo.h), compiled into the device code
and the oracle alike.  Air cells must hold NaN, or keep their previous value
where the reference leaves them untouched."""
import numpy as np
import pytest

import hydrothermal3d_gb300 as ht
from hydrothermal3d_gb300 import api, abi
from post_case import PARAMS, SENTINEL, case, oracle_fields

pytestmark = pytest.mark.gpu


def _same(name, got, ref):
    assert np.array_equal(got, ref, equal_nan=True), name


def _dev(c):
    return {k: ht.from_numpy(c[k]) for k in ("phc", "T", "P", "Vx", "Vy", "Vz")}


def _dout(n):
    return ht.from_numpy(np.full(n, SENTINEL, order="F"))


def _single(ctx, d, n):
    p = PARAMS
    r = {k: _dout(n) for k in abi.POST_FIELDS}
    api.Phase(ctx, r["phase"], d["phc"])
    api.Pressure(ctx, r["pressure"], d["P"], d["phc"], p["scale_sigma"])
    api.Temperature(ctx, r["temperature"], d["T"], d["phc"], p["scale_T"])
    api.Velocity(ctx, r["vx"], r["vy"], r["vz"], d["Vx"], d["Vy"], d["Vz"], d["phc"], p["scale_V"])
    api.EffectiveThermalConductivity(ctx, r["k_thermal"], d["T"], p["phi0"], d["phc"], p["scale_T"])
    api.EffectiveHeatCapacity(ctx, r["heat_capacity"], d["T"], d["P"], d["phc"], p["phi0"], p["scale_T"],
                              p["scale_sigma"], 1.0, 1.0)
    api.Permeability(ctx, r["permeability"], p["k_fact"], p["ymin"], p["dy"], d["phc"], p["delta"], p["scale_L"])
    api.FluidDensity(ctx, r["density"], d["T"], d["P"], d["phc"], p["scale_T"], p["scale_sigma"])
    api.Viscosity(ctx, r["viscosity"], d["T"], d["phc"], p["scale_T"])
    api.Peclet(ctx, r["peclet"], d["T"], d["P"], d["Vx"], d["Vy"], d["Vz"], d["phc"], p["phi0"], p["scale_T"],
               p["scale_sigma"], p["scale_V"], p["scale_L"])
    return {k: ht.to_numpy(v) for k, v in r.items()}


@pytest.mark.parametrize("n", [(13, 11, 6), (1, 1, 1), (33, 9, 17)])
def test_single_field_kernels(ctx, orc, n):
    c = case(*n, seed=sum(n))
    ref = oracle_fields(orc, c)
    got = _single(ctx, _dev(c), c["n"])
    for name in abi.POST_FIELDS:
        _same(name, got[name], ref[name])


def test_fused_pass_equals_single_kernels(ctx, orc):
    c = case(40, 21, 9, seed=11)
    d = _dev(c)
    single = _single(ctx, d, c["n"])
    fused = {k: _dout(c["n"]) for k in abi.POST_FIELDS}
    api.postprocess_fields(ctx, fused, d["T"], d["P"], d["Vx"], d["Vy"], d["Vz"], d["phc"], **PARAMS)
    for name in abi.POST_FIELDS:
        assert np.array_equal(ht.to_numpy(fused[name]), single[name], equal_nan=True), name


def test_fused_subset_needs_only_its_inputs(ctx, orc):
    """A subset that reads neither P nor V accepts NULL for them."""
    c = case(9, 7, 5, seed=4)
    d = _dev(c)
    ref = oracle_fields(orc, c)
    out = {"temperature": _dout(c["n"]), "k_thermal": _dout(c["n"]), "phase": _dout(c["n"])}
    api.postprocess_fields(ctx, out, d["T"], None, None, None, None, d["phc"], **PARAMS)
    for name, t in out.items():
        _same(name, ht.to_numpy(t), ref[name])
    with pytest.raises(api.Ht3dError):  # density needs P
        api.postprocess_fields(ctx, {"density": _dout(c["n"])}, d["T"], None, None, None, None, d["phc"], **PARAMS)
    with pytest.raises(api.Ht3dError):  # velocity needs all three outputs
        api.postprocess_fields(ctx, {"vx": _dout(c["n"])}, None, None, d["Vx"], d["Vy"], d["Vz"], d["phc"], **PARAMS)


@pytest.mark.parametrize("n", [(7, 9, 5), (1, 3, 1), (300, 4, 211)])
def test_nusselt(ctx, orc, n):
    nx, ny, nz = n
    rng = np.random.default_rng(nx)
    qy = np.asfortranarray(rng.uniform(-1, 3, (nx, ny + 1, nz)))
    got = api.Nusselt(ctx, ht.from_numpy(qy), 1.25, 0.5)
    assert got == orc.nusselt(qy, 1.25, 0.5)  # same canonical tree order


def test_nusselt_of_conduction_through_the_library(ctx):
    """ComputeFlux of T = 1 - y in the unit box, then Nu = 1 (pure conduction)."""
    nx, ny, nz = 16, 12, 10
    dy = 1.0 / ny
    yce = np.linspace(-dy / 2, 1 + dy / 2, ny + 2)
    T = ht.from_numpy(np.broadcast_to((1.0 - yce)[None, :, None], (nx + 2, ny + 2, nz + 2)).copy())
    S = dict(fx=(nx + 1, ny, nz), fy=(nx, ny + 1, nz), fz=(nx, ny, nz + 1))
    kx, ky, kz = (ht.from_numpy(np.ones(S[f])) for f in ("fx", "fy", "fz"))
    qx, qy, qz = (ht.zeros(*S[f]) for f in ("fx", "fy", "fz"))
    api.SetFaceBCs(ctx, T, (0, 0, 1, 1, 0, 0), (0, 0, 1.0, 0.0, 0, 0))
    api.ComputeFlux(ctx, qx, qy, qz, kx, ky, kz, T, float(nx), float(ny), float(nz))
    assert abs(api.Nusselt(ctx, qy, 1.0, 1.0) - 1.0) <= 1e-12
