"""The C++ oracle against the golden fixtures of the independent numpy
restatement (tests/golden/make_golden.py)."""
import ctypes

import numpy as np
import pytest

from conftest import rel_err


def f(a):
    return np.asfortranarray(np.array(a, dtype=np.float64))


@pytest.fixture(scope="module")
def g(golden):
    return golden


def dims(g):
    return [int(x) for x in g["dims"]]


def test_compute_flux(orc, g):
    nx, ny, nz = dims(g)
    qx, qy, qz = orc.zeros(nx + 1, ny, nz), orc.zeros(nx, ny + 1, nz), orc.zeros(nx, ny, nz + 1)
    orc.call("ComputeFlux", qx, qy, qz, f(g["kx"]), f(g["ky"]), f(g["kz"]), f(g["T"]), 1 / g["dx"], 1 / g["dy"],
             1 / g["dz"], nx, ny, nz)
    for a, b in ((qx, "qx"), (qy, "qy"), (qz, "qz")):
        assert rel_err(a, g[b]) <= 1e-15


def test_residuals(orc, g):
    nx, ny, nz = dims(g)
    F = orc.zeros(nx, ny, nz)
    orc.call("ResidualDiffusionTransient", F, f(g["T"]), f(g["R"]), f(g["qx"]), f(g["qy"]), f(g["qz"]),
             float(g["_dt"]), 1 / g["dx"], 1 / g["dy"], 1 / g["dz"], nx, ny, nz)
    assert rel_err(F, g["F_transient"]) <= 1e-15
    orc.call("ResidualDiffusion", F, f(g["R"]), f(g["qx"]), f(g["qy"]), f(g["qz"]), 1 / g["dx"], 1 / g["dy"],
             1 / g["dz"], nx, ny, nz)
    assert rel_err(F, g["F_diffusion"]) <= 1e-15


def test_init_kernels(orc, g):
    nx, ny, nz = dims(g)
    Ty, kx, ky, kz = orc.zeros(nx, ny + 1, nz), orc.zeros(nx + 1, ny, nz), orc.zeros(nx, ny + 1, nz), orc.zeros(nx, ny, nz + 1)
    orc.call("InitDarcy", Ty, kx, ky, kz, f(g["T"]), f(g["kv"]), 1.0, nx, ny, nz)
    assert rel_err(Ty, g["Ty"]) <= 1e-15
    assert rel_err(kx, g["kx_v"]) <= 1e-15 and rel_err(ky, g["ky_v"]) <= 1e-15 and rel_err(kz, g["kz_v"]) <= 1e-15
    Rp = orc.zeros(nx, ny, nz)
    orc.call("Compute_Rp", Rp, f(g["ky"]), f(g["Ty"]), float(g["Ra"]), 1 / g["dy"], nx, ny, nz)
    assert rel_err(Rp, g["Rp"]) <= 1e-14
    Vx, Vy, Vz = orc.zeros(nx + 1, ny, nz), orc.zeros(nx, ny + 1, nz), orc.zeros(nx, ny, nz + 1)
    orc.call("Init_vel", Vx, Vy, Vz, f(g["kx"]), f(g["ky"]), f(g["kz"]), f(g["P"]), f(g["Ty"]), float(g["Ra"]),
             1 / g["dx"], 1 / g["dy"], 1 / g["dz"], nx, ny, nz)
    for a, b in ((Vx, "Vx"), (Vy, "Vy"), (Vz, "Vz")):
        assert rel_err(a, g[b]) <= 1e-15
    ktc = orc.zeros(nx, ny, nz)
    orc.call("SmoothConductivityV2C", ktc, f(g["kv"]), nx, ny, nz)
    assert rel_err(ktc, g["ktc_v2c"]) <= 1e-15


def test_face_bcs(orc, g):
    nx, ny, nz = dims(g)
    T = f(g["T"]).copy(order="F")
    orc.call("SetFaceBCs", T, orc.int6(*[int(x) for x in g["bc_types"]]), orc.dbl6(*g["bc_vals"]), nx, ny, nz)
    np.testing.assert_array_equal(T, g["T_bc"])


def test_gershgorin(orc, g):
    nx, ny, nz = dims(g)
    G, D = orc.zeros(nx, ny, nz), orc.zeros(nx, ny, nz)
    orc.call("GershgorinPoisson", G, D, f(g["rhoC"]), f(g["kx"]), f(g["ky"]), f(g["kz"]), 1.0, 0.3,
             float(g["dx"]), float(g["dy"]), float(g["dz"]), nx, ny, nz)
    assert rel_err(G, g["G"]) <= 1e-15 and rel_err(D, g["D"]) <= 1e-15


@pytest.mark.parametrize("which,cX", [("T", "dt"), ("P", None)])
def test_dyrel_iterations(orc, g, which, cX):
    from hydrothermal3d_gb300.abi import DyrelParams
    nx, ny, nz = dims(g)
    X = f(g[which]).copy(order="F")
    Fc, F0 = orc.zeros(nx, ny, nz), orc.zeros(nx, ny, nz)
    prm = DyrelParams.reference(nitout=3)
    if which == "T":
        types, vals = [int(x) for x in g["bc_types"]], list(g["bc_vals"])
    else:
        types, vals = [0] * 6, [0.0] * 6
    c = float(g["_dt"]) if cX else 0.0
    s, st = orc.dyrel_solve_dimless(X, f(g["R"]), f(g["kx"]), f(g["ky"]), f(g["kz"]), c, float(g["dx"]), float(g["dy"]),
                                    float(g["dz"]), types, vals, prm, Fc, F0, n_iter_fixed=7)
    assert s == 0 and st.iters == 7
    inner = (slice(1, -1),) * 3
    assert rel_err(X[inner], g[f"dyrel_{which}_X"][inner]) <= 1e-13
    assert rel_err(Fc, g[f"dyrel_{which}_F"]) <= 1e-12
    assert rel_err(F0, g[f"dyrel_{which}_F0"]) <= 1e-12
    lmin, h1, h2, lmax, dtau = g[f"dyrel_{which}_sc"]
    assert abs(st.lambda_max - lmax) <= 1e-14 * lmax and abs(st.dtau - dtau) <= 1e-14 * dtau
    assert abs(st.lambda_min - lmin) <= 1e-10 * lmin and abs(st.h1 - h1) <= 1e-12 and abs(st.h2 - h2) <= 1e-12 * abs(h2)


@pytest.mark.parametrize("variant,key", [(0, "weno_v1"), (1, "weno_v2")])
def test_weno(orc, g, variant, key):
    nx, ny, nz = dims(g)
    T = f(g["T"]).copy(order="F")
    wt = orc.int6(*[int(x) for x in g["weno_types"]])
    wv = orc.dbl6(*g["weno_vals"])
    h = (1 / g["dx"], 1 / g["dy"], 1 / g["dz"])
    if variant == 0:
        orc.call("AdvectWithWeno5_v1", T, f(g["wVx"]), f(g["wVy"]), f(g["wVz"]), float(g["weno_dt"]), *h, wt, wv, nx, ny, nz)
    else:
        orc.call("AdvectWithWeno5_v2", T, f(g["wVx"]), f(g["wVy"]), f(g["wVz"]), float(g["weno_dt"]), *h, wt, wv,
                 ctypes.c_int(1), nx, ny, nz)
    inner = (slice(1, -1),) * 3
    assert rel_err(T[inner], g[key][inner]) <= 1e-14


def test_laws(orc, g):
    Tg, pg = g["law_T"], g["law_p"]
    for idx in np.ndindex(Tg.shape):
        r = orc.law(5, Tg[idx], pg[idx])
        d = orc.law(6, Tg[idx], pg[idx])
        assert abs(r - g["rhof"][idx]) <= 1e-13 * abs(g["rhof"][idx])
        assert abs(d - g["drhodp"][idx]) <= 1e-13 * abs(g["drhodp"][idx])
