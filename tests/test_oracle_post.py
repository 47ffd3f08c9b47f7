"""The oracle's output diagnostics (Dimensional/kernels_HT3D_postprocessing.jl)
against an independent numpy restatement in the reference's array-slice form,
and the Nusselt number (Dimensionless/HydroThermal3D_Alban_v6.jl:345-348)
against its known value 1 for pure conduction."""
import numpy as np

from post_case import PARAMS, SENTINEL, case, oracle_fields


def _law(orc, which, a, b=0.0):
    b = np.broadcast_to(b, a.shape)
    return np.array([orc.law(which, x, y) for x, y in zip(a.ravel(order="F"), b.ravel(order="F"))]).reshape(
        a.shape, order="F")


def _numpy_fields(orc, c):
    p = PARAMS
    inn = (slice(1, -1),) * 3
    ph = c["phc"][inn]
    air = ph == 1.0
    T = c["T"][inn] * p["scale_T"]
    P = c["P"][inn] * p["scale_sigma"]
    x = 0.5 * (c["Vx"][:-1, :, :] + c["Vx"][1:, :, :]) * p["scale_V"]
    y = 0.5 * (c["Vy"][:, :-1, :] + c["Vy"][:, 1:, :]) * p["scale_V"]
    z = 0.5 * (c["Vz"][:, :, :-1] + c["Vz"][:, :, 1:]) * p["scale_V"]
    phi = _law(orc, 9, ph, p["phi0"])
    keff = (1.0 - phi) * _law(orc, 0, T) + phi * _law(orc, 1, T)
    rho = _law(orc, 5, T - 273.15, P)
    V = np.sqrt(x * x + y * y + z * z)
    Pe = p["scale_L"] * rho * _law(orc, 2, T) * V / keff
    nx, ny, nz = c["n"]
    yc = p["ymin"] + np.arange(ny, dtype=float) * p["dy"] + p["dy"] / 2
    perm = _law(orc, 8, np.broadcast_to((yc * p["scale_L"])[None, :, None], (nx, ny, nz)).copy(order="F"),
                p["delta"] * p["scale_L"])
    perm = np.where(ph == 2.0, perm * p["k_fact"], perm)
    nan = lambda a: np.where(air, np.nan, a)
    keep = lambda a: np.where(air, SENTINEL, a)
    return dict(phase=nan(ph), pressure=nan(P), temperature=nan(T), vx=nan(x), vy=keep(y), vz=keep(z),
                k_thermal=nan(keff), heat_capacity=keep(_law(orc, 3, T)), permeability=nan(perm),
                density=nan(rho), viscosity=nan(_law(orc, 7, T)), peclet=nan(Pe))


def test_post_fields_match_array_form(orc):
    c = case()
    got = oracle_fields(orc, c)
    ref = _numpy_fields(orc, c)
    for name, r in ref.items():
        assert np.array_equal(got[name], r, equal_nan=True), name
    # every phase code occurs, air cells included
    assert set(np.unique(c["phc"][1:-1, 1:-1, 1:-1])) == {-1.0, 0.0, 1.0, 2.0, 3.0}


def test_nusselt_of_pure_conduction_is_one(orc):
    """Linear T = 1 - y in the unit box (the HRL setup's conductive state):
    qy = 1 everywhere, so Nu = 1."""
    nx, ny, nz = 7, 9, 5
    dy = 1.0 / ny
    yce = np.linspace(-dy / 2, 1 + dy / 2, ny + 2)
    T = np.asfortranarray(np.broadcast_to((1.0 - yce)[None, :, None], (nx + 2, ny + 2, nz + 2)).copy())
    orc.call("SetFaceBCs", T, orc.int6(0, 0, 1, 1, 0, 0), orc.dbl6(0, 0, 1.0, 0.0, 0, 0), nx, ny, nz)
    kx, ky, kz = (np.ones(s, order="F") for s in ((nx + 1, ny, nz), (nx, ny + 1, nz), (nx, ny, nz + 1)))
    qx, qy, qz = orc.zeros(nx + 1, ny, nz), orc.zeros(nx, ny + 1, nz), orc.zeros(nx, ny, nz + 1)
    orc.call("ComputeFlux", qx, qy, qz, kx, ky, kz, T, float(nx), float(ny), float(nz), nx, ny, nz)
    assert abs(orc.nusselt(qy, 1.0, 1.0) - 1.0) <= 1e-12


def test_nusselt_matches_plain_sum(orc):
    rng = np.random.default_rng(2)
    nx, ny, nz = 37, 5, 29
    qy = np.asfortranarray(rng.uniform(-1, 3, (nx, ny + 1, nz)))
    ref = np.sum(qy[:, -1, :]) / (1.5 * 0.75) / (nx * nz)
    assert abs(orc.nusselt(qy, 1.5, 0.75) - ref) <= 1e-14 * abs(ref)
